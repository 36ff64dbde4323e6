"""Device grand-canonical chains (cass_gcmc) against the CPU oracle's chains.

The FP64 kernel draws the same lfsr258 numbers in the same order as the
oracle, so over short runs both make the same decisions and agree in counts,
molecule numbers and energies.  The mixed kernel (FP32 pair energies against
the box) follows its own chain; its running energy must match a recomputation
of its final state."""
import numpy as np
import pytest

import cassandra_gb300 as cg
from cassandra_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

KEYS = ("n_translate", "n_translate_accepted", "n_rotate", "n_rotate_accepted", "n_insert", "n_insert_accepted",
        "n_delete", "n_delete_accepted", "n_regrow", "n_regrow_accepted", "n_molecules")


def _run(open_ctx, s, nsteps, seed, mu=(-22.0, -26.0)):
    with open_ctx(s) as g:
        for b in (1, 2):
            g.system_total_energy(b)
        r = g.gcmc([1, 2], nsteps, 1, list(mu), [[1.0], [1.0]], [[0.5], [0.5]], seed=seed)
        again = [g.system_total_energy(b)[0] for b in (1, 2)]
        where = g.molecule_boxes(1)
        for b, x in zip((1, 2), r):
            assert int((where == b).sum()) == x["n_molecules"]
        live = np.flatnonzero(where)
        xyz = np.stack([g.get_molecule(int(k) + 1, 1) for k in live]) if live.size else np.zeros((0, 4, 3))
    return r, again, (where, xyz)


STYLES = {"cut_tail": abi.VDW_SUM_CUT_TAIL, "cut": abi.VDW_SUM_CUT, "cut_shift": abi.VDW_SUM_CUT_SHIFT,
          "cut_switch": abi.VDW_SUM_CUT_SWITCH, "cut_shift_force": abi.VDW_SUM_CUT_SHIFT_FORCE,
          "minimum": abi.VDW_SUM_MINIMUM,
          # no atom cutoff: molecule pairs selected by Check_MoleculePair_Cutoff
          # (energy_routines.f90:3027-3088) in every energy of every move
          "charmm": abi.VDW_SUM_CHARMM}


@pytest.mark.parametrize("style", list(STYLES))
def test_fp64_gcmc_matches_oracle(style):
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300, rcut=12.0)
    for bx in s.boxes:
        bx.vdw_sum_style = STYLES[style]
        if style == "cut_switch":
            bx.ron_switch, bx.roff_switch = 10.0, 12.0
    ro, eo, so = _run(oracle.open_system, s, 600, seed=4)
    rg, eg, sg = _run(lambda x: cg.open_system(x, precision=abi.PREC_FP64), s, 600, seed=4)
    assert np.array_equal(so[0], sg[0])  # the same molecule slots live in the same boxes
    assert np.allclose(so[1], sg[1], rtol=0, atol=1e-9)
    for a, b in zip(ro, rg):
        for k in KEYS:
            assert a[k] == b[k], (k, a[k], b[k])
        assert abs(a["sum_n_molecules"] - b["sum_n_molecules"]) < 1e-9
        scale = abs(a["energy"]["inter_vdw"]) + abs(a["energy"]["dihedral"]) + 1.0
        for k, v in a["energy"].items():
            assert abs(b["energy"][k] - v) <= 1e-9 * scale, (k, v, b["energy"][k])
    for x, e in zip(rg, eg):  # the device's running energy against a recomputation of its final state
        assert abs(x["energy"]["total"] - e["total"]) <= 1e-9 * (abs(e["inter_vdw"]) + 1.0)


def test_mixed_gcmc_bookkeeping():
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300)
    r, again, _ = _run(lambda x: cg.open_system(x, precision=abi.PREC_MIXED), s, 3000, seed=8)
    for x, e in zip(r, again):
        assert x["n_insert_accepted"] > 0 and x["n_regrow_accepted"] > 0
        scale = abs(e["inter_vdw"]) + abs(e["angle"]) + abs(e["dihedral"])
        assert abs(x["energy"]["total"] - e["total"]) <= 1e-6 * scale, (x["energy"]["total"], e["total"])


def test_gcmc_errors():
    s = workloads.gcmc_system(nboxes=1, length=25.0, max_per_box=5)
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        with pytest.raises(abi.CassError) as e:
            g.gcmc([1], 10, 1, [-20.0], [[1.0]], [[0.5]], seed=1)
        assert e.value.code == abi.CASS_ESTATE
        g.system_total_energy(1)
        with pytest.raises(abi.CassError) as e:  # five free slots run out at a high chemical potential
            g.gcmc([1], 5000, 1, [-10.0], [[1.0]], [[0.5]], seed=1, cuts=(0.0, 0.0, 1.0, 1.0, 1.0))
        assert e.value.code == abi.CASS_ECAPACITY
