"""MC sweeps of boxes too large for shared memory (the box layout in global
memory): 5000 LJ spheres against the oracle's chain, and the 4096-water Ewald
box (12,288 atoms, 13,190 k-vectors) keeping its running energy equal to a
recomputation."""
import numpy as np
import pytest

import cassandra_gb300 as cg
from cassandra_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_large_lj_box_fp64_matches_oracle():
    n = 5000
    s = workloads.lj_nvt_system(nboxes=1, n=n, length=35.0 * (n / 500) ** (1 / 3), rcut=10.0, seed=8)
    out = []
    for open_ctx in (oracle.open_system, lambda x: cg.open_system(x, precision=abi.PREC_FP64)):
        with open_ctx(s) as c:
            c.system_total_energy(1)
            r, md, _ = c.mc_sweeps([1], 1, [[0.8]], [[0.0]], seed=12)
            out.append((r[0], md))
    (ro, mo), (rg, mg) = out
    assert ro["n_translate_accepted"] == rg["n_translate_accepted"] and ro["n_translate"] == n
    assert abs(ro["energy"]["total"] - rg["energy"]["total"]) <= 1e-9 * abs(ro["energy"]["inter_vdw"])
    assert np.allclose(mo, mg, rtol=1e-12)


def test_large_water_box_mixed_bookkeeping():
    s = workloads.water_gradient_system()
    with cg.open_system(s, precision=abi.PREC_MIXED) as g:
        g.system_total_energy(1)
        r, _, _ = g.mc_sweeps([1], 1, [[0.4]], [[0.3]], seed=3, prob_translate=0.5)
        assert r[0]["n_translate"] + r[0]["n_rotate"] == 4096
        assert r[0]["n_translate_accepted"] > 0 and r[0]["n_rotate_accepted"] > 0
        e, _ = g.system_total_energy(1)
        scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"])
        assert abs(r[0]["energy"]["total"] - e["total"]) <= 1e-6 * scale
