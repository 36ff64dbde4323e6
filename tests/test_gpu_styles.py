"""Every vdW and charge style of Compute_AtomPair_Energy (energy_routines.f90:
1831-2082) and Check_AtomPair_Cutoff (:3092-3195) through the FP64 GPU path
against the oracle: LJ with cut, cut_tail, cut_shift, cut_switch, CHARMM,
minimum image and cut_shift_force; Mie with cut, cut_shift and cut_tail; charges
with the plain cut, minimum image, damped shifted force and Ewald.  Per style:
the system energy (every component), molecule energies with and without the
CBMC cutoffs, and Widom insertions record by record.  Where a style has no atom
cutoff (LJ CHARMM, minimum-image charges) and the vdW sum is not minimum image,
Check_MoleculePair_Cutoff (:3027-3088) selects the interacting molecules by their
COM distance; the system and molecule energies, the MC sweeps, the CBMC trial
energies, the Widom insertions and the grand-canonical moves apply it (the
allocation-free call refuses such boxes)."""
import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
from cassandra_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cassandra_gb300 import build
    build.build()
    oracle.build()


def _close(a, b, rel=TOL, abs_=1e-7):
    return abs(a - b) <= rel * max(abs(a), abs(b)) + abs_


def _lj_fluid(vdw_sum, vdw=("LJ", 120.0, 3.4), style=abi.VDW_LJ):
    return helpers.lj_fluid_system(vdw_sum, vdw, style)


def _water(charge_sum, rcut=9.0):
    s = helpers.pregen_system("water_spce", 4)
    s.species[0].libraries = [workloads.water_species().libraries[0] * 1.0]
    bx = s.boxes[0]
    bx.charge_style, bx.charge_sum_style = abi.CHARGE_COUL, charge_sum
    bx.rcut_coul = rcut
    bx.rcut_vdw = rcut
    return s


CASES = [("lj_" + n, lambda v=v: _lj_fluid(v)) for n, v in (
    ("cut", abi.VDW_SUM_CUT), ("cut_tail", abi.VDW_SUM_CUT_TAIL), ("cut_shift", abi.VDW_SUM_CUT_SHIFT),
    ("cut_switch", abi.VDW_SUM_CUT_SWITCH), ("charmm", abi.VDW_SUM_CHARMM), ("minimum", abi.VDW_SUM_MINIMUM),
    ("cut_shift_force", abi.VDW_SUM_CUT_SHIFT_FORCE))]
CASES += [("mie_" + n, lambda v=v: _lj_fluid(v, vdw=("Mie", 120.0, 3.4, 14.0, 6.0), style=abi.VDW_MIE)) for n, v in (
    ("cut", abi.VDW_SUM_CUT), ("cut_shift", abi.VDW_SUM_CUT_SHIFT), ("cut_tail", abi.VDW_SUM_CUT_TAIL))]
CASES += [("water_" + n, lambda v=v: _water(v)) for n, v in (
    ("qq_cut", abi.QQ_CUT), ("qq_minimum", abi.QQ_MINIMUM), ("qq_dsf", abi.QQ_DSF), ("qq_ewald", abi.QQ_EWALD))]


# styles without an atom cutoff whose vdW sum is not minimum image: the molecule
# pairs are selected by their COM distance (energy_routines.f90:3027-3088)
COMCUT = {"lj_charmm", "water_qq_minimum"}


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_style_matches_oracle(name, make):
    s = make()
    water = name.startswith("water")
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        eo, ovo = o.system_total_energy(1)
        eg, ovg = g.system_total_energy(1)
        assert ovo == ovg == False
        for k in eo:
            assert _close(eg[k], eo[k]), (name, k, eg[k], eo[k])
        for im in (1, 17, 60):
            for cbmc in (False, True):
                a = o.mol_inter_energy(im, 1, cbmc)
                b = g.mol_inter_energy(im, 1, cbmc)
                assert a[2] == b[2]
                assert _close(b[0], a[0]) and _close(b[1], a[1]), (name, im, cbmc, a, b)
        n = 64
        ro, to = o.widom_insert(1, [1], n, 8, 0, seed=3, trace=True)
        rg, tg = g.widom_insert(1, [1], n, 8, 0, seed=3, trace=True)
    assert np.array_equal(to["overlap"], tg["overlap"])
    assert np.array_equal(to["selected_trial"], tg["selected_trial"])
    ok = to["overlap"] == 0
    assert ok.sum() > 0
    assert np.allclose(tg["e_inter"][ok], to["e_inter"][ok], rtol=1e-9, atol=1e-6)
    assert np.allclose(tg["widom_var"][ok], to["widom_var"][ok], rtol=1e-8, atol=0)
    if not water:
        assert ro[0]["n_insertions"] == rg[0]["n_insertions"] == n


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_widom_butane_molecule_pair_cutoff(prec):
    """Butane Widom insertions into an LJ CHARMM box (no atom cutoff: every energy
    call of the growth selects molecule pairs by Check_MoleculePair_Cutoff,
    energy_routines.f90:3027-3088): the first fragment at its trial centre, the new
    atoms of each dihedral trial, then the whole folded molecule, each with the COM
    and max_dcom of its atoms -- against the oracle insertion by insertion.  A
    mixed context runs the FP64 kernel for this style."""
    s = workloads.widom_batch_system(nboxes=1, sizes=[300], seed=5, nconfig=200)
    s.boxes[0].vdw_sum_style = abi.VDW_SUM_CHARMM
    n = 256
    with oracle.open_system(s) as o, cg.open_system(s, precision=prec) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        ro, to = o.widom_insert(2, [1], n, 12, 12, seed=5, trace=True)
        rg, tg = g.widom_insert(2, [1], n, 12, 12, seed=5, trace=True)
    assert np.array_equal(to["overlap"], tg["overlap"])
    assert np.array_equal(to["selected_trial"], tg["selected_trial"])
    assert np.allclose(tg["ln_pbias"], to["ln_pbias"], rtol=1e-10, atol=1e-10)
    ok = to["overlap"] == 0
    assert ok.sum() > 0.3 * n
    assert np.allclose(tg["e_inter"][ok], to["e_inter"][ok], rtol=1e-9, atol=1e-6)
    assert np.allclose(tg["widom_var"][ok], to["widom_var"][ok], rtol=1e-8, atol=0)
    assert ro[0]["n_overlaps"] == rg[0]["n_overlaps"]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_style_mc_sweeps_match_oracle(name, make):
    """NVT sweeps (translation, and rotation for water) in every style: the FP64 chain
    equals the oracle's move by move (acceptances, adapted steps, energies).  In the
    styles without an atom cutoff (LJ CHARMM, minimum-image charges) the molecule
    pairs of both energies of a move are selected by Check_MoleculePair_Cutoff
    (energy_routines.f90:3027-3088) from the old and the trial COM."""
    s = make()
    water = name.startswith("water")
    pt = 0.5 if water else 1.0
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        ro, mdo, mro = o.mc_sweeps([1], 2, [[0.5]], [[0.3]], seed=9, prob_translate=pt, nupdate=50)
        rg, mdg, mrg = g.mc_sweeps([1], 2, [[0.5]], [[0.3]], seed=9, prob_translate=pt, nupdate=50)
        for k in ("n_translate", "n_translate_accepted", "n_rotate", "n_rotate_accepted"):
            assert ro[0][k] == rg[0][k], (name, k)
        assert np.allclose(mdg, mdo, rtol=1e-12) and np.allclose(mrg, mro, rtol=1e-12)
        for k in ro[0]["energy"]:
            assert _close(rg[0]["energy"][k], ro[0]["energy"][k], 1e-9, 1e-6), (name, k)


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_style_mixed_system_energy(name, make):
    """The mixed context's system energy in every style: FP32 pair terms where the
    style has an FP32 kernel (LJ cut / cut_tail, Ewald), FP64 elsewhere; within 1e-5
    of the sum of the magnitudes of the components."""
    s = make()
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as g:
        eo, _ = o.system_total_energy(1)
        eg, _ = g.system_total_energy(1)
    scale = abs(eo["inter_vdw"]) + abs(eo["inter_q"]) + abs(eo["intra"]) + abs(eo["reciprocal"])
    for k in ("total", "inter_vdw", "inter_q", "reciprocal", "lrc", "self"):
        assert abs(eg[k] - eo[k]) <= 1e-5 * scale, (name, k, eg[k], eo[k])


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_style_mixed_molecule_and_trial_energies(name, make):
    """The mixed context's molecule energies (cbmc_flag off and on) and CBMC trial
    energies against the oracle in every style.  Compute_AtomPair_Energy applies the
    shift, switch, shifted-force and CHARMM forms whatever the CBMC flag is
    (energy_routines.f90:1927-1970), so the mixed kernels must too: the FP32 pair form
    serves LJ cut, cut_tail and minimum image only.  Bound: 1e-5 of the summed pair
    magnitudes (a missing shift term is several per cent of it)."""
    s = make()
    bx = s.boxes[0]
    water = name.startswith("water")
    sp = s.species[0]
    types = list(sp.type_index)
    charges = [a.charge for a in sp.atoms]
    rmax = max(bx.rcut_vdw, bx.rcut_coul if bx.charge_style == abi.CHARGE_COUL else 0.0)
    all_pairs = name in ("lj_minimum", "lj_charmm", "water_qq_minimum")
    m = s.molecules
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        for im in (1, 17, 60):
            k = m.im.index(im)
            for cbmc in (False, True):
                a = o.mol_inter_energy(im, 1, cbmc)
                b = g.mol_inter_energy(im, 1, cbmc)
                assert a[2] == b[2]
                rc = bx.rcut_cbmc if cbmc else (None if all_pairs else rmax)
                scale = helpers.pair_magnitude_scale(s, m.xyz[k], types, charges, im, rc)
                err = abs(b[0] + b[1] - a[0] - a[1])
                assert err <= 1e-5 * scale, (name, im, cbmc, a, b, err / scale)
        rng = np.random.default_rng(11)
        L = bx.length[0]
        shape = np.asarray(m.xyz[0]) - np.asarray(m.xyz[0]).mean(axis=0)
        xyz = np.array([shape + (rng.random(3) - 0.5) * L for _ in range(24)])
        atoms = list(range(1, sp.natoms + 1))
        for cbmc in (True, False):
            eo, oo = o.cbmc_trial_energies(1, 1, atoms, xyz, cbmc=cbmc)
            eg, og = g.cbmc_trial_energies(1, 1, atoms, xyz, cbmc=cbmc)
            assert np.array_equal(oo, og)
            assert (~oo).sum() > 10
            rc = bx.rcut_cbmc if cbmc else (None if all_pairs else rmax)
            for t in np.nonzero(~oo)[0]:
                scale = helpers.pair_magnitude_scale(s, xyz[t], types, charges, 0, rc)
                assert abs(eg[t] - eo[t]) <= 1e-5 * scale, (name, cbmc, t, eg[t], eo[t])
