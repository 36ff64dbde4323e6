"""Volume moves on the GPU (cass_volume_scale / cass_volume_restore) and NPT
chains through the harness, against the oracle."""
import numpy as np
import pytest

import cassandra_gb300 as cg
from cassandra_gb300 import abi, npt, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def _coords(ctx, s):
    return np.concatenate([ctx.get_molecule(im, is_).ravel() for im, is_ in zip(s.molecules.im, s.molecules.is_)])


@pytest.mark.parametrize("factor", [1.03, 0.998])
def test_volume_scale_matches_oracle_and_restores(factor):
    s = workloads.water_nvt_system(nboxes=1)
    L = s.boxes[0].length[0]
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        eo0, _ = o.system_total_energy(1)
        eg0, _ = g.system_total_energy(1)
        x0 = _coords(g, s)
        eo, ovo = o.volume_scale(1, L * factor)
        eg, ovg = g.volume_scale(1, L * factor)
        assert ovo == ovg
        for k in ("total", "inter_vdw", "inter_q", "reciprocal", "lrc", "self"):
            assert abs(eg[k] - eo[k]) <= 1e-10 * (abs(eo[k]) + 1.0), k
        assert np.allclose(_coords(g, s), _coords(o, s), rtol=0, atol=1e-12)
        g.volume_restore(1)
        o.volume_restore(1)
        assert np.array_equal(_coords(g, s), x0)
        e2, _ = g.system_total_energy(1)
        assert abs(e2["total"] - eg0["total"]) <= 1e-10 * abs(eg0["total"])
        # sweeps continue from the restored state on both
        ro, _, _ = o.mc_sweeps([1], 1, [[0.5]], [[0.3]], seed=3, prob_translate=0.5)
        rg, _, _ = g.mc_sweeps([1], 1, [[0.5]], [[0.3]], seed=3, prob_translate=0.5)
        assert ro[0]["n_translate_accepted"] == rg[0]["n_translate_accepted"]
        assert abs(ro[0]["energy"]["total"] - rg[0]["energy"]["total"]) <= 1e-9 * abs(eo0["total"])


def test_npt_chain_fp64_matches_oracle():
    s = workloads.lj_nvt_system(nboxes=2, n=100, length=35.0 * (100 / 500) ** (1 / 3), rcut=10.0, seed=3)
    out = []
    for open_ctx in (oracle.open_system, lambda x: cg.open_system(x, precision=abi.PREC_FP64)):
        with open_ctx(s) as c:
            ch = npt.NPTChains(c, [1, 2], [100, 100], 150.0, 50.0, 300.0, [[0.8], [0.8]], [[0.0], [0.0]], seed=5)
            ch.start([b.length[0] for b in s.boxes])
            for _ in range(8):
                ch.sweeps(1)
                ch.volume_moves()
            out.append((list(ch.length), list(ch.energy), ch.n_vol_acc.copy()))
    (lo, eo, ao), (lg, eg, ag) = out
    assert np.array_equal(ao, ag) and ao.sum() > 0
    assert np.allclose(lg, lo, rtol=1e-12)
    assert np.allclose(eg, eo, rtol=1e-9)


def test_npt_chain_mixed_bookkeeping():
    s = workloads.water_nvt_system(nboxes=2, seed=5, rcut=8.0)
    with cg.open_system(s, precision=abi.PREC_MIXED) as g:
        ch = npt.NPTChains(g, [1, 2], [256, 256], 298.0, 1.0, 60.0, [[0.5], [0.5]], [[0.3], [0.3]], seed=9)
        ch.start([b.length[0] for b in s.boxes])
        for _ in range(6):
            ch.sweeps(1, prob_translate=0.5)
            ch.volume_moves()
        assert ch.n_vol_acc.sum() > 0
        for k, b in enumerate([1, 2]):
            e, _ = g.system_total_energy(b)
            scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"])
            assert abs(e["total"] - ch.energy[k]) <= 1e-6 * scale
