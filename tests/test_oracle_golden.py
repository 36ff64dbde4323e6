"""Pin the CPU oracle to the reference's own golden values (no GPU needed).

Golden sources (Cassandra test suite, extracted by tests/golden/make_golden.py):
  Test1/Test2 analytic LJ / Mie pair energies (Test1_LJ_StartEnergy.py:145-147,
  Test2_Mie_StartEnergy.py:155-158), tolerance 1e-5;
  Test6 NIST SRSW LJ totals (Test6_NIST_LennardJonesEnergy.py:151-158), 1e-2;
  Test7 NIST SPC/E Ewald components (Test7_Water.py:49-52, tolerances :87);
  Test8 analytic 2-charge Ewald (Test8_Coul_StartEnergy.py:154-188), 1e-5;
  pregen Widom fixtures: per-frame Energy_Total printed by the reference
  (exampleResults/Widom/{water_spce,pentane}/*.prp), 5e-4 in Test13 -- held
  here to 5e-8, the precision of the printed values.
"""
import math

import numpy as np
import pytest

import helpers
from cassandra_gb300 import abi
from oracle import oracle

KJ = 0.01  # atomic energy units -> kJ/mol


def total(system):
    with oracle.open_system(system) as ctx:
        e, ov = ctx.system_total_energy(1)
    assert not ov
    return e


def lj(r, eps, sig):
    return 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)


def mie(r, eps, sig, n, m):
    return (n / (n - m)) * (n / m) ** (m / (n - m)) * eps * ((sig / r) ** n - (sig / r) ** m)


@pytest.mark.parametrize("a,b", [((0, 0, 0), (1, 0, 0)), ((0, 0, 0), (2 ** (1 / 6), 0, 0))])
def test_lj_pair_analytic(a, b):
    eps_K = 120.272
    sysm = helpers.single_atom_system([a, b], 100.0, vdw=("LJ", eps_K, 1.0), vdw_sum=abi.VDW_SUM_MINIMUM,
                                      rcut=10.0, rcut_low=0.1)
    r = math.dist(a, b)
    want = lj(r, eps_K * 0.0083144598, 1.0)
    got = total(sysm)["total"] * KJ
    assert abs(got - want) <= 1e-5 * max(abs(want), 1e-3)


def test_lj_pair_periodic_image():
    eps_K = 120.272
    d = 2 ** (1 / 6)
    sysm = helpers.single_atom_system([(-50 + d / 2, 0, 0), (50 - d / 2, 0, 0)], 100.0,
                                      vdw=("LJ", eps_K, 1.0), vdw_sum=abi.VDW_SUM_MINIMUM, rcut=10, rcut_low=0.1)
    want = lj(d, eps_K * 0.0083144598, 1.0)
    got = total(sysm)["total"] * KJ
    assert abs(got - want) <= 1e-5 * abs(want)


@pytest.mark.parametrize("a,b", [((0, 0, 0), (1, 0, 0)), ((-49.5, 0, 0), (49.5, 0, 0)),
                                 ((0, 0, 0), (1.12246205, 0, 0)), ((0, 0, 0), (5.0, 0, 0))])
def test_mie_pair_analytic(a, b):
    eps_K = 120.272
    sysm = helpers.single_atom_system([a, b], 100.0, vdw=("Mie", eps_K, 1.0, 14.0, 6.0), vdw_style=abi.VDW_MIE,
                                      vdw_sum=abi.VDW_SUM_CUT_TAIL, rcut=7.0, rcut_low=0.5)
    rvec = np.subtract(b, a).astype(float)
    rvec -= 100.0 * np.round(rvec / 100.0)
    r = float(np.linalg.norm(rvec))
    want = mie(r, eps_K * 0.0083144598, 1.0, 14.0, 6.0) if r <= 7.0 else 0.0
    got = total(sysm)["inter_vdw"] * KJ
    assert abs(got - want) <= 1e-5 * max(abs(want), 1e-3)


@pytest.mark.parametrize("k", range(8))
def test_nist_lj(k):
    d = helpers.golden("nist_lj.npz")
    f, L, rc, tot, vdw, lrc = d["checks"][k]
    e = total(helpers.single_atom_system(d[f"xyz{int(f)}"], L, rcut=rc))
    for got, want in ((e["total"], tot), (e["inter_vdw"], vdw), (e["lrc"], lrc)):
        assert abs(got * KJ - want) <= 1e-2 * abs(want)


@pytest.mark.parametrize("k", range(4))
def test_nist_spce(k):
    d = helpers.golden("nist_spce.npz")
    e = total(helpers.nist_spce_system(k))
    got = [e["inter_vdw"], e["lrc"], e["inter_q"], e["reciprocal"], e["self"], e["total"]]
    for g, want, tol in zip(got, d["checks"][k][4:], d["tolerances"]):
        assert abs(g * KJ - want) <= tol * abs(want)


def _ewald_two_charges(dist, box, rcut, tol):
    """Analytic 2-charge Ewald sum with the A&S erf, as Test8_Coul_StartEnergy.py:154-188 states it."""
    cf = 1.602176565 ** 2 * 6.02214129 / (4 * np.pi * 8.854187817) * 10000
    alpha = math.sqrt(-math.log(tol)) / rcut
    k2_cut = (math.log(tol) / rcut / math.pi) ** 2
    nmax = int(-2.0 * math.log(tol) / rcut * box / (2 * math.pi)) + 1

    def erf_as(x):
        t = 1.0 / (1.0 + 0.3275911 * x)
        return 1.0 - (((((1.061405429 * t - 1.453152027) * t) + 1.421413741) * t - 0.284496736) * t
                      + 0.254829592) * t * math.exp(-x * x)

    real = -cf * (1 - erf_as(alpha * dist)) / dist if dist < rcut else 0.0
    n = np.arange(-nmax, nmax)
    kx, ky, kz = np.meshgrid(n / box, n / box, n / box, indexing="ij")
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    mask = (k2 != 0) & (k2 <= k2_cut)
    s2 = (1.0 - np.cos(2 * np.pi * kx * dist)) ** 2 + np.sin(2 * np.pi * kx * dist) ** 2
    recip = np.sum(np.where(mask, np.exp(-(np.pi / alpha) ** 2 * k2) / np.where(mask, k2, 1) * s2, 0.0))
    recip = recip * cf / (2 * np.pi * box ** 3)
    self_e = -alpha / math.sqrt(math.pi) * 2 * cf
    return real, recip, self_e


@pytest.mark.parametrize("dist", [1.0, 11.0])
def test_coulomb_ewald_two_charges(dist):
    from cassandra_gb300.system import Atom, BoxSpec, ForceField, MoleculeSet, Species, System
    sps = [Species(atoms=[Atom("C", 1.0, 1.0, ())], scale_vdw=(0, 0, 0, 0), scale_qq=(0, 0, 0, 0)),
           Species(atoms=[Atom("A", 1.0, -1.0, ())], scale_vdw=(0, 0, 0, 0), scale_qq=(0, 0, 0, 0))]
    for s in sps:
        s.atoms[0].vdw = ("LJ", 0.0, 0.0)
    ff = ForceField(sps)
    ms = MoleculeSet()
    ms.add(1, 1, 1, [(0.0, 0.0, 0.0)])
    ms.add(1, 2, 1, [(dist, 0.0, 0.0)])
    bx = BoxSpec(length=(39.0,) * 3, vdw_style=abi.VDW_NONE, rcut_vdw=10.0, rcut_coul=10.0, rcut_low=0.1,
                 charge_style=abi.CHARGE_COUL, charge_sum_style=abi.QQ_EWALD, ewald_tol=1e-5)
    e = total(System(sps, [bx], ms, ff, [1, 1]))
    real, recip, self_e = _ewald_two_charges(dist, 39.0, 10.0, 1e-5)
    assert abs(e["self"] * KJ - self_e) <= 1e-5 * abs(self_e)
    assert abs(e["reciprocal"] * KJ - recip) <= 1e-5 * abs(recip)
    if dist < 10:
        assert abs(e["inter_q"] * KJ - real) <= 1e-5 * abs(real)
    else:
        assert e["inter_q"] == 0.0


@pytest.mark.parametrize("name", ["water_spce", "pentane"])
def test_pregen_frame_energies(name):
    d = helpers.golden(f"pregen_{name}.npz")
    for f, want in enumerate(d["energy_total_kjmol"]):
        got = total(helpers.pregen_system(name, f))["total"] * KJ
        assert abs(got - want) <= 5e-8 * abs(want) + 1e-4, (f, got, want)


def test_rng_reference_stream():
    """lfsr258 of random_generators.f90: values in (0,1), deterministic, seeds as init_seeds."""
    a = oracle.rng_reference(1, 2, 1000)
    b = oracle.rng_reference(1, 2, 1000)
    assert np.array_equal(a, b)
    assert a.min() > 0.0 and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.05


def test_rng_streams_independent():
    s = [oracle.rng_stream(7, 1, k, 200) for k in range(4)]
    for i in range(4):
        for j in range(i + 1, 4):
            assert abs(np.corrcoef(s[i], s[j])[0, 1]) < 0.3
    assert np.array_equal(oracle.rng_stream(7, 2, 5, 10), oracle.rng_stream(7, 2, 5, 10))
