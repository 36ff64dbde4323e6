"""GPU parity: libcassgpu.so through its C-ABI against the FP64 oracle and the
reference's golden values.

FP64 path : same arithmetic as the reference; energies agree with the oracle to
            1e-10 relative (summation order is the only difference) and
            per-insertion Widom records (status, selected trial, ln_pbias,
            widom_var) agree insertion by insertion.
mixed path: FP32 pair math with FP64 accumulation; trial and total energies
            within 1e-5 of the FP64 oracle relative to the sum of |pair
            terms| (MIXED_TOL below), Widom statistics within their error.
"""
import math

import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
from cassandra_gb300 import abi, workloads
from cassandra_gb300.system import MoleculeSet
from oracle import oracle

pytestmark = pytest.mark.gpu

KJ = 0.01
FP64_TOL = 1e-10
MIXED_TOL = 1e-5
# Widom full-cutoff energies of grown molecules against the oracle: every cutoff
# and overlap decision is the FP64 one (pairs within FP32 rounding of a cutoff
# are decided again in FP64), and FP32 storage of absolute coordinates
# (|x| <= 35 A) bounds each displacement to a few 1e-6 A; the stated bound is
# 2e-5 of the sum of |pair energies| for every insertion (measured on 16,000
# benchmark insertions: max 1.4e-5, mean 1.5e-6).
MIXED_WIDOM_TOL = 2e-5


def close(a, b, rel, scale=1.0):
    return abs(a - b) <= rel * max(abs(b), scale)


def abs_pair_sum(system, im, cbmc):
    """Sum of |pair energies| of molecule im against its box (LJ + real-space
    Ewald), the conditioning scale of a mixed-precision energy."""
    bx = system.boxes[0]
    L = np.asarray(bx.length)
    xyz = system.molecules.xyz
    sp = system.species[0]
    q = np.array([a.charge for a in sp.atoms])
    eps_k = np.array([a.vdw[1] * 0.8314472 for a in sp.atoms])
    sig = np.array([a.vdw[2] for a in sp.atoms])
    alpha = math.sqrt(-math.log(bx.ewald_tol)) / bx.rcut_coul
    rc = bx.rcut_cbmc if cbmc else bx.rcut_vdw
    tot = 0.0
    for ia, a in enumerate(xyz[im - 1]):
        for jm, other in enumerate(xyz):
            if jm == im - 1:
                continue
            d = other - a
            d -= L * np.round(d / L)
            r = np.sqrt((d * d).sum(1))
            m = r <= rc
            e = np.sqrt(eps_k[ia] * eps_k)
            s = 0.5 * (sig[ia] + sig)
            with np.errstate(divide="ignore", invalid="ignore"):
                lj = np.where(e > 0, 4 * e * ((s / r) ** 12 - (s / r) ** 6), 0.0)
                qq = 138935.4558 * q[ia] * q / r * np.array([math.erfc(alpha * x) for x in r])
            tot += np.abs(lj[m]).sum() + (0.0 if cbmc else np.abs(qq[m]).sum())
    return tot


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cassandra_gb300 import build
    build.build()
    oracle.build()


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", ["water_spce", "pentane"])
def test_pregen_frame_totals(name, prec):
    d = helpers.golden(f"pregen_{name}.npz")
    for f, want in enumerate(d["energy_total_kjmol"]):
        s = helpers.pregen_system(name, f)
        with oracle.open_system(s) as o, cg.open_system(s, precision=prec) as g:
            eo, ovo = o.system_total_energy(1)
            eg, ovg = g.system_total_energy(1)
        assert ovo == ovg == False
        if prec == abi.PREC_FP64:
            for k in eo:
                assert close(eg[k], eo[k], FP64_TOL, 1e-6), (f, k, eg[k], eo[k])
            assert abs(eg["total"] * KJ - want) <= 5e-8 * abs(want) + 1e-4
        else:
            scale = abs(eo["inter_vdw"]) + abs(eo["inter_q"]) + abs(eo["intra"])
            assert abs(eg["total"] - eo["total"]) <= MIXED_TOL * scale, (f, eg["total"], eo["total"])


@pytest.mark.parametrize("k", range(4))
def test_nist_spce_fp64(k):
    s = helpers.nist_spce_system(k)
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        eo, _ = o.system_total_energy(1)
        eg, _ = g.system_total_energy(1)
    for key in eo:
        assert close(eg[key], eo[key], FP64_TOL, 1e-6), (key, eg[key], eo[key])


@pytest.mark.parametrize("k", range(8))
def test_nist_lj_fp64(k):
    d = helpers.golden("nist_lj.npz")
    f, L, rc, tot, vdw, lrc = d["checks"][k]
    s = helpers.single_atom_system(d[f"xyz{int(f)}"], L, rcut=rc)
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        eg, ov = g.system_total_energy(1)
    assert not ov
    for got, want in ((eg["total"], tot), (eg["inter_vdw"], vdw), (eg["lrc"], lrc)):
        assert abs(got * KJ - want) <= 1e-2 * abs(want)


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_molecule_energies(prec):
    s = helpers.pregen_system("water_spce", 3)
    rng = np.random.default_rng(3)
    with oracle.open_system(s) as o, cg.open_system(s, precision=prec) as g:
        for im in rng.choice(90, 12, replace=False) + 1:
            for cbmc in (False, True):
                a = o.mol_inter_energy(int(im), 1, cbmc)
                b = g.mol_inter_energy(int(im), 1, cbmc)
                assert a[2] == b[2]
                tol = FP64_TOL if prec == abi.PREC_FP64 else MIXED_TOL
                scale = abs(a[0]) + abs(a[1]) + 1.0
                if prec == abi.PREC_MIXED:
                    scale = max(scale, abs_pair_sum(s, int(im), cbmc))
                assert abs(a[0] - b[0]) <= tol * scale and abs(a[1] - b[1]) <= tol * scale, (im, cbmc, a, b)
            for cbmc in (False, True):
                ia = o.mol_intra_energy(int(im), 1, cbmc)
                ib = g.mol_intra_energy(int(im), 1, cbmc)
                assert ia[3] == ib[3]
                for x, y in zip(ia[:3], ib[:3]):
                    assert close(y, x, FP64_TOL, 1e-6)


def test_molecule_overlap_flag():
    s = helpers.pregen_system("water_spce", 0)
    xyz = s.molecules.xyz[1].copy()
    xyz += s.molecules.xyz[0][0] - xyz[0] + np.array([0.3, 0.0, 0.0])  # O atoms 0.3 A apart
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        for c in (o, g):
            c.set_molecules([2], [1], [1], xyz)
        assert o.mol_inter_energy(2, 1)[2] is True
        assert g.mol_inter_energy(2, 1)[2] is True
        assert g.system_total_energy(1)[1] is True


@pytest.mark.parametrize("move", [abi.MOVE_TRANSLATION, abi.MOVE_ROTATION, abi.MOVE_DELETION])
def test_ewald_update_and_restore(move):
    s = helpers.pregen_system("water_spce", 2)
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        e0o = o.system_total_energy(1)[0]["reciprocal"]
        e0g = g.system_total_energy(1)[0]["reciprocal"]
        assert close(e0g, e0o, FP64_TOL)
        xyz = s.molecules.xyz[6] + np.array([0.41, -0.27, 0.13])
        if move != abi.MOVE_DELETION:
            for c in (o, g):
                c.set_molecules([7], [1], [1], xyz)
        eo = o.ewald_update(7, 1, 1, move)
        eg = g.ewald_update(7, 1, 1, move)
        assert close(eg, eo, FP64_TOL), (eg, eo)
        g.ewald_restore(7, 1, 1)
        o.ewald_restore(7, 1, 1)
        # after a restore the next update from the restored state matches again
        eo2 = o.ewald_update(7, 1, 1, abi.MOVE_INTRA)
        eg2 = g.ewald_update(7, 1, 1, abi.MOVE_INTRA)
        assert close(eg2, eo2, FP64_TOL)


def test_ewald_widom_batch():
    s = helpers.pregen_system("water_spce", 5)
    rng = np.random.default_rng(5)
    base = s.molecules.xyz[0]
    L = s.boxes[0].length[0]
    xyz = np.concatenate([(base - base.mean(0)) @ workloads.random_rotation(rng).T + (rng.random(3) - 0.5) * L
                          for _ in range(24)])
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        a = o.ewald_widom(1, 1, xyz)
        b = g.ewald_widom(1, 1, xyz)
    assert np.allclose(b, a, rtol=FP64_TOL, atol=0)


def _butane_batch(sizes, seed=9):
    return workloads.widom_batch_system(nboxes=len(sizes), sizes=sizes, seed=seed, nconfig=200)


def _totals(ctx, nb):
    for b in range(1, nb + 1):
        ctx.system_total_energy(b)


def test_widom_fp64_matches_oracle_per_insertion():
    sizes = [200, 450, 900]
    s = _butane_batch(sizes)
    n = 384
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        _totals(o, 3)
        _totals(g, 3)
        ro, to = o.widom_insert(2, [1, 2, 3], n, 12, 12, seed=77, trace=True)
        rg, tg = g.widom_insert(2, [1, 2, 3], n, 12, 12, seed=77, trace=True)
    assert np.array_equal(to["overlap"], tg["overlap"])
    assert np.array_equal(to["selected_trial"], tg["selected_trial"])
    assert np.allclose(tg["ln_pbias"], to["ln_pbias"], rtol=1e-10, atol=1e-10)
    ok = to["overlap"] == 0
    assert ok.sum() > 0.5 * ok.size
    assert np.allclose(tg["widom_var"][ok], to["widom_var"][ok], rtol=1e-8, atol=0)
    assert np.allclose(tg["e_inter"][ok], to["e_inter"][ok], rtol=1e-9, atol=1e-8)
    assert np.allclose(tg["e_inter_abs"][ok], to["e_inter_abs"][ok], rtol=1e-9, atol=1e-8)
    for a, b in zip(ro, rg):
        assert a["n_overlaps"] == b["n_overlaps"] and a["n_trials"] == b["n_trials"]
        assert close(b["widom_sum"], a["widom_sum"], 1e-8)


def _mixed_vs_oracle(s, boxes, n, kappa_dih, seed, band=None):
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as m:
        _totals(o, len(boxes))
        _totals(m, len(boxes))
        if band is not None:
            m.set_widom_band(band)
        ro, to = o.widom_insert(2, boxes, n, 12, kappa_dih, seed=seed, trace=True)
        rm, tm = m.widom_insert(2, boxes, n, 12, kappa_dih, seed=seed, trace=True)
        fixups = m.stats()["widom_fixups"]
    return ro, to, rm, tm, fixups


def _check_mixed_records(ro, to, rm, tm):
    assert np.array_equal(to["overlap"], tm["overlap"])
    same = to["selected_trial"] == tm["selected_trial"]
    # a Boltzmann choice within FP32 rounding of a cumulative-weight boundary may
    # pick the neighbouring trial (about 1e-5 of insertions)
    assert same.mean() >= 0.999
    ok = same & (to["overlap"] == 0)
    assert ok.sum() > 0.7 * ok.size
    err = np.abs(tm["e_inter"][ok] - to["e_inter"][ok])
    scale = np.maximum(to["e_inter_abs"][ok], 1.0)
    rel = err / scale
    assert rel.max() <= MIXED_WIDOM_TOL, rel.max()
    assert rel.mean() <= 5e-6, rel.mean()
    for a, b in zip(ro, rm):
        assert a["n_overlaps"] == b["n_overlaps"]
        assert abs(b["widom_sum"] - a["widom_sum"]) <= 1e-4 * abs(a["widom_sum"])


def test_widom_mixed_matches_oracle_per_insertion():
    """The mixed Widom kernel against the FP64 oracle insertion by insertion, on
    four boxes of the benchmark batch (butane, kappa_ins = kappa_dih = 12): the
    same status and selected trial for every insertion (the draws are decided on
    their top 32 bits, library indices in exact integer arithmetic), and the
    full-cutoff inter energy of every insertion within MIXED_WIDOM_TOL of the sum
    of its |pair energies| -- no outlier allowance.  Pairs within FP32 rounding
    of the 14 A cutoff or of rcut_low are decided again in FP64 by k_widom_fix
    (about 1.4 % of the insertions have one), so every cutoff decision is the
    FP64 one; what remains is the FP32 rounding of the coordinates (a few 1e-6
    A), largest on steep repulsive pairs."""
    s = workloads.widom_batch_system(nboxes=4, seed=2024, nconfig=1000)
    ro, to, rm, tm, fixups = _mixed_vs_oracle(s, [1, 2, 3, 4], 2000, 12, 4242)
    assert fixups > 0  # the FP64 fix-up ran
    _check_mixed_records(ro, to, rm, tm)


@pytest.mark.parametrize("band", [30.0, 3000.0])
def test_widom_mixed_wide_bands_match_oracle(band):
    """Widened FP32 bands send many more pairs through the FP64 decisions of
    k_widom_fix -- at 30x about one in five insertions has a band pair, at
    3000x most have more than four and their full-cutoff pass is redone from
    the FP64 coordinates -- and the records still match the oracle to the
    same bound: the fix-up only ever replaces an FP32 decision by the FP64
    one."""
    s = workloads.widom_batch_system(nboxes=2, seed=2024, nconfig=1000)
    ro, to, rm, tm, fixups = _mixed_vs_oracle(s, [1, 2], 1500, 12, 99, band=band)
    assert fixups > (200 if band < 100 else 1000), fixups
    _check_mixed_records(ro, to, rm, tm)


def test_widom_mixed_charged_spce_matches_oracle():
    """Charged SPC/E water with Ewald in mixed precision against the oracle:
    real-space Ewald and LJ pairs in FP32, cutoff decisions as in FP64."""
    s = helpers.pregen_system("water_spce", 0)
    s.species[0].libraries = [workloads.water_species().libraries[0] * 1.0]
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as m:
        o.system_total_energy(1)
        m.system_total_energy(1)
        ro, to = o.widom_insert(1, [1], 1000, 12, 0, seed=11, trace=True)
        rm, tm = m.widom_insert(1, [1], 1000, 12, 0, seed=11, trace=True)
    _check_mixed_records(ro, to, rm, tm)


def _water_sticking_out(nmol=600, length=26.2, shift=1.3):
    """Waters shifted by `shift` A and folded back by their COM, so that some
    hydrogens lie outside the box; 26.2 A gives four cells of rcut_cbmc per
    side, so the CBMC queries reach periodic images through per-row shifts."""
    s = workloads.water_box(nmol, length)
    masses = np.array([15.999, 1.008, 1.008])
    ms = MoleculeSet()
    for im, is_, ib, x in zip(s.molecules.im, s.molecules.is_, s.molecules.ibox, s.molecules.xyz):
        x = np.asarray(x, dtype=np.float64).reshape(-1, 3) + shift
        com = (x * masses[:, None]).sum(0) / masses.sum()
        ms.add(im, is_, ib, x - length * np.floor((com + length / 2) / length))
    s.molecules = ms
    xyz = np.concatenate([np.asarray(v).reshape(-1, 3) for v in ms.xyz])
    assert (np.abs(xyz) > length / 2).sum() > 10
    return s


def test_widom_mixed_water_atoms_outside_box():
    """Atoms outside the box (a molecule is folded by its COM) in a box of four
    cells per side: the cell-sorted copies are wrapped, so the FP32 queries,
    which shift whole rows by a box length instead of folding each pair, see
    every neighbour at its minimum image."""
    s = _water_sticking_out()
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_MIXED) as m:
        o.system_total_energy(1)
        m.system_total_energy(1)
        ro, to = o.widom_insert(1, [1], 1000, 12, 0, seed=11, trace=True)
        rm, tm = m.widom_insert(1, [1], 1000, 12, 0, seed=11, trace=True)
    _check_mixed_records(ro, to, rm, tm)


def test_widom_deterministic():
    s = _butane_batch([400])
    with cg.open_system(s, precision=abi.PREC_MIXED) as g:
        g.system_total_energy(1)
        a = g.widom_insert(2, [1], 1000, 12, 12, seed=3)
        b = g.widom_insert(2, [1], 1000, 12, 12, seed=3)
    assert a == b


def test_widom_charged_spce_fp64():
    s = helpers.pregen_system("water_spce", 0)
    sp = s.species[0]
    sp.libraries = [workloads.water_species().libraries[0] * 1.0]
    n = 96
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        ro, to = o.widom_insert(1, [1], n, 12, 0, seed=11, trace=True)
        rg, tg = g.widom_insert(1, [1], n, 12, 0, seed=11, trace=True)
    assert np.array_equal(to["overlap"], tg["overlap"])
    assert np.array_equal(to["selected_trial"], tg["selected_trial"])
    ok = to["overlap"] == 0
    assert np.allclose(tg["e_inter"][ok], to["e_inter"][ok], rtol=1e-9, atol=1e-7)
    assert np.allclose(tg["widom_var"][ok], to["widom_var"][ok], rtol=1e-8, atol=0)


def test_widom_edge_cases():
    s = _butane_batch([200, 250])
    with cg.open_system(s, precision=abi.PREC_MIXED) as g:
        with pytest.raises(abi.CassError) as e:
            g.widom_insert(2, [1], 10, 12, 12, seed=1)
        assert e.value.code == abi.CASS_ESTATE
        g.system_total_energy(1)
        g.system_total_energy(2)
        with pytest.raises(abi.CassError):
            g.widom_insert(2, [1], 10, 33, 12, seed=1)
        with pytest.raises(abi.CassError):
            g.widom_insert(2, [3], 10, 12, 12, seed=1)
        r = g.widom_insert(2, [1, 2], 0, 12, 12, seed=1)
        assert r[0]["widom_sum"] == 0.0 and r[0]["n_insertions"] == 0
    # an empty box: every insertion is an ideal-gas insertion (no neighbours)
    s2 = _butane_batch([200])
    s2.molecules = type(s2.molecules)()
    with oracle.open_system(s2) as o, cg.open_system(s2, precision=abi.PREC_FP64) as g:
        o.system_total_energy(1)
        g.system_total_energy(1)
        ro, to = o.widom_insert(2, [1], 64, 12, 12, seed=4, trace=True)
        rg, tg = g.widom_insert(2, [1], 64, 12, 12, seed=4, trace=True)
    assert np.allclose(tg["widom_var"], to["widom_var"], rtol=1e-9)


def test_cbmc_trial_energies_match_oracle():
    s = _butane_batch([300, 500], seed=8)
    rng = np.random.default_rng(4)
    L = s.boxes[1].length[0]
    # 40 random positions of butane's first fragment (atoms 2, 1, 3) in box 2, and
    # single LJ spheres including one placed on molecule 7 of the box
    frag = np.array([[0.0, 0.0, 0.0], [1.54, 0.0, 0.0], [-0.63, 1.40, 0.0]])
    xyz = np.array([frag + (rng.random(3) - 0.5) * L for _ in range(40)])
    m = s.molecules
    k7 = [k for k in range(len(m.im)) if m.ibox[k] == 2][6]
    sph = np.concatenate([(rng.random((15, 1, 3)) - 0.5) * L, m.xyz[k7][None, :, :]])
    with oracle.open_system(s) as o:
        with cg.open_system(s, precision=abi.PREC_FP64) as g:
            for cbmc in (True, False):
                eo, oo = o.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=cbmc)
                eg, og = g.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=cbmc)
                assert np.array_equal(oo, og)
                assert np.allclose(eg, eo, rtol=FP64_TOL, atol=1e-9)
            eo, oo = o.cbmc_trial_energies(2, 1, [1], sph)
            eg, og = g.cbmc_trial_energies(2, 1, [1], sph)
            assert np.array_equal(oo, og) and og[-1]
            assert np.allclose(eg, eo, rtol=FP64_TOL, atol=1e-9)
            # the same position with the molecule itself excluded (deletion / regrowth)
            eo, oo = o.cbmc_trial_energies(2, 1, [1], sph[-1:], skip_im=m.im[k7])
            eg, og = g.cbmc_trial_energies(2, 1, [1], sph[-1:], skip_im=m.im[k7])
            assert not og[0] and oo[0] == og[0]
            assert abs(eg[0] - eo[0]) <= FP64_TOL * abs(eo[0])


@pytest.mark.parametrize("cbmc", [True, False])
def test_atom_intra_energies_match_oracle(cbmc):
    """Compute_Atom_Nonbond_Intra_Energy for batches of pentane conformations with
    partial growth (exist flags): united atoms whose only scaled pair is 1-5,
    and the same chain with charges in an Ewald box (the -erf part)."""
    import dataclasses
    rng = np.random.default_rng(17)
    for charged in (False, True):
        s = helpers.pregen_system("pentane", 1)
        if charged:
            sp = s.species[0]
            sp.atoms = [dataclasses.replace(a, charge=q) for a, q in zip(sp.atoms, (0.3, -0.2, 0.1, -0.4, 0.2))]
            bx = s.boxes[0]
            bx.charge_style, bx.charge_sum_style = abi.CHARGE_COUL, abi.QQ_EWALD
            bx.rcut_coul, bx.ewald_tol = 14.0, 1e-3
        na = s.species[0].natoms
        base = np.asarray(s.molecules.xyz[0])
        xyz = np.stack([base + rng.normal(scale=0.4, size=base.shape) for _ in range(40)])
        xyz[3, 0] = xyz[3, 4] + np.array([0.05, 0.0, 0.0])  # atoms 1 and 5 (the scaled 1-5 pair) overlap in trial 3
        xyz[5, 1] = xyz[5, 3] + np.array([0.05, 0.0, 0.0])  # atoms 2 and 4 (1-3, zero scales): skipped, no overlap
        with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
            for ia in (1, 2, 3, 5):
                for exist in (None, [1] * (na - 1) + [0], [1, 1, 1, 0, 0]):
                    eo, oo = o.atom_intra_energies(1, 1, ia, xyz, exist, cbmc)
                    eg, og = g.atom_intra_energies(1, 1, ia, xyz, exist, cbmc)
                    assert np.array_equal(oo, og)
                    assert np.allclose(eg, eo, rtol=1e-12, atol=1e-9), (charged, ia, exist)
                    if exist is None and ia in (1, 5):  # the 1-5 pair is the chain's only scaled pair
                        assert np.abs(eo).sum() > 0
                        if charged:
                            assert np.abs(eo[:, 2]).sum() > 0
            assert g.atom_intra_energies(1, 1, 1, xyz)[1][3] and not g.atom_intra_energies(1, 1, 2, xyz)[1][5]


def test_molecule_intra_cbmc_coulomb_rule():
    """Compute_Molecule_Nonbond_Intra_Energy with cbmc_flag drops the charge pairs of a
    species whose L_Coul_CBMC is set (energy_routines.f90:1062-1064)."""
    for lcc in (False, True):
        s = helpers.pregen_system("water_spce", 2)
        s.species[0].l_coul_cbmc = lcc
        with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
            for im in (1, 7, 40):
                for cbmc in (False, True):
                    a = o.mol_intra_energy(im, 1, cbmc)
                    b = g.mol_intra_energy(im, 1, cbmc)
                    assert a[3] == b[3]
                    for x, y in zip(a[:3], b[:3]):
                        assert close(y, x, FP64_TOL, 1e-9), (lcc, im, cbmc, a, b)
                    if cbmc and lcc:
                        assert a[1] == 0.0 and a[2] == 0.0
                    else:
                        assert a[2] != 0.0  # the -erf part of the intramolecular Ewald pairs
