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


def _run(open_ctx, s, nsteps, seed, mu=(-22.0, -26.0), fill=0):
    with open_ctx(s) as g:
        for b in (1, 2):
            g.system_total_energy(b)
        if fill:  # insertions only first: a lone charged molecule's translation changes the
            # energy by rounding only (its reciprocal sum is translation invariant), and the
            # sign of such a change decides whether the acceptance test draws a number
            g.gcmc([1, 2], fill, 1, list(mu), [[1.0], [1.0]], [[0.5], [0.5]], seed=seed + 100,
                   cuts=(0.0, 0.0, 1.0, 1.0, 1.0))
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


# ---------------------------------------------------------------------------
# Charged species in Ewald boxes (move_insert.f90:274-291, move_delete.f90:
# 261-277, move_regrow.f90:338-354): real-space Coulomb in every pair sum,
# reciprocal energy from the box's running structure factors, self energy.

WATER_CUTS = (0.2, 0.4, 0.7, 1.0, 1.0)


def _water_run(open_ctx, s, nsteps, seed, then_mc=0):
    with open_ctx(s) as g:
        for b in (1, 2):
            g.system_total_energy(b)
        r = g.gcmc([1, 2], nsteps, 1, [-30.0, -34.0], [[0.5], [0.5]], [[0.4], [0.4]], seed=seed, kappa_ins=8,
                   kappa_dih=0, cuts=WATER_CUTS)
        mc = None
        if then_mc:  # NVT sweeps on the structure factors the chain left behind
            mc, _, _ = g.mc_sweeps([1, 2], then_mc, [[0.3], [0.3]], [[0.3], [0.3]], seed=seed + 1, prob_translate=0.5)
        again = [g.system_total_energy(b)[0] for b in (1, 2)]
        where = g.molecule_boxes(1)
        live = np.flatnonzero(where)
        xyz = np.stack([g.get_molecule(int(k) + 1, 1) for k in live]) if live.size else np.zeros((0, 3, 3))
    return r, mc, again, (where, xyz)


def _same_chain(ro, rg, comps=("total", "inter_vdw", "inter_q", "intra_q", "reciprocal", "self", "lrc")):
    for a, b in zip(ro, rg):
        for k in KEYS:
            assert a[k] == b[k], (k, a[k], b[k])
        scale = abs(a["energy"]["inter_vdw"]) + abs(a["energy"]["inter_q"]) + abs(a["energy"]["self"]) + 1.0
        for k in comps:
            assert abs(b["energy"][k] - a["energy"][k]) <= 1e-9 * scale, (k, a["energy"][k], b["energy"][k])


def test_fp64_gcmc_water_ewald_matches_oracle():
    s = workloads.water_gcmc_system(nboxes=2)
    ro, _, eo, so = _water_run(oracle.open_system, s, 1500, seed=7)
    rg, _, eg, sg = _water_run(lambda x: cg.open_system(x, precision=abi.PREC_FP64), s, 1500, seed=7)
    for x in rg:
        assert x["n_insert_accepted"] > 0 and x["n_delete_accepted"] > 0, x
    assert np.array_equal(so[0], sg[0])
    assert np.allclose(so[1], sg[1], rtol=0, atol=1e-9)
    _same_chain(ro, rg)
    for x, e in zip(rg, eg):  # running energy against a recomputation of the final state
        scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"]) + abs(e["self"])
        for comp in ("total", "inter_vdw", "inter_q", "intra_q", "reciprocal", "self"):
            assert abs(x["energy"][comp] - e[comp]) <= 1e-9 * scale, (comp, x["energy"][comp], e[comp])


def test_gcmc_water_leaves_structure_factors_for_mc():
    """The structure factors a chain commits (box sums, per-molecule rows of
    inserted molecules) carry NVT sweeps that follow without a recomputation;
    a mixed context runs charged boxes on the FP64 kernel (from its own
    mixed-precision starting energies, so its chain is its own)."""
    s = workloads.water_gcmc_system(nboxes=2)
    r64, mc, again, _ = _water_run(lambda x: cg.open_system(x, precision=abi.PREC_FP64), s, 600, seed=3, then_mc=2)
    rmx, _, again_mx, _ = _water_run(lambda x: cg.open_system(x, precision=abi.PREC_MIXED), s, 600, seed=3)
    for x, e in zip(rmx, again_mx):
        assert x["n_insert_accepted"] > 0
        scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"])
        assert abs(x["energy"]["total"] - e["total"]) <= 1e-6 * scale, (x["energy"]["total"], e["total"])
    for x, e in zip(mc, again):
        scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"])
        assert abs(x["energy"]["reciprocal"] - e["reciprocal"]) <= 1e-9 * scale, (x["energy"]["reciprocal"], e["reciprocal"])
        assert abs(x["energy"]["total"] - e["total"]) <= 1e-9 * scale, (x["energy"]["total"], e["total"])


def _charged_butane(l_coul_cbmc):
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300, rcut=12.0)
    sp = s.species[0]
    for a, q in zip(sp.atoms, (0.25, -0.25, -0.25, 0.25)):
        a.charge = q
    sp.l_coul_cbmc = l_coul_cbmc
    for bx in s.boxes:
        bx.charge_style, bx.charge_sum_style, bx.ewald_tol, bx.rcut_coul = abi.CHARGE_COUL, abi.QQ_EWALD, 1e-5, 12.0
    return s


@pytest.mark.parametrize("l_coul_cbmc", [False, True])
def test_fp64_gcmc_charged_butane_matches_oracle(l_coul_cbmc):
    """Partially charged butane: CBMC growth with (L_Coul_CBMC) or without
    intermolecular charges in the trial energies, and regrowth (Cut_N_Grow)
    moving the molecule's structure factors."""
    s = _charged_butane(l_coul_cbmc)
    ro, eo, so = _run(oracle.open_system, s, 600, seed=5, fill=40)
    rg, eg, sg = _run(lambda x: cg.open_system(x, precision=abi.PREC_FP64), s, 600, seed=5, fill=40)
    assert sum(x["n_regrow_accepted"] for x in rg) > 0 and sum(x["n_insert_accepted"] for x in rg) > 0
    assert np.array_equal(so[0], sg[0])
    assert np.allclose(so[1], sg[1], rtol=0, atol=1e-9)
    _same_chain(ro, rg, comps=("total", "inter_vdw", "inter_q", "intra_q", "reciprocal", "self", "dihedral"))
    for x, e in zip(rg, eg):
        scale = abs(e["inter_vdw"]) + abs(e["inter_q"]) + abs(e["reciprocal"]) + abs(e["self"]) + abs(e["dihedral"])
        assert abs(x["energy"]["total"] - e["total"]) <= 1e-9 * scale, (x["energy"]["total"], e["total"])


def test_gcmc_refuses_charges_without_ewald():
    s = workloads.water_gcmc_system(nboxes=1)
    s.boxes[0].charge_sum_style = abi.QQ_DSF
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        g.system_total_energy(1)
        with pytest.raises(abi.CassError) as e:
            g.gcmc([1], 10, 1, [-30.0], [[0.5]], [[0.4]], seed=1, kappa_ins=8, kappa_dih=0, cuts=WATER_CUTS)
        assert e.value.code == abi.CASS_EUNSUPPORTED
