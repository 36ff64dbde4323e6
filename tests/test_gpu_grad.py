"""The adjoint (cass_system_gradient) and its torch.autograd.Function against
central finite differences of the CPU oracle's FP64 energy and, for LJ, an
analytic NumPy gradient."""
import copy

import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
import mc_helpers
from cassandra_gb300 import abi
from oracle import oracle

pytestmark = pytest.mark.gpu

H_REL = 1e-6   # finite-difference step, relative to the perturbed value (1e-6 A for coordinates below 1 A)
FD_TOL = 1e-6  # relative to the largest gradient component


def _box_order(system, ibox=1):
    m = system.molecules
    sel = [k for k, b in enumerate(m.ibox) if b == ibox]
    return sorted(sel, key=lambda k: (m.is_[k], m.im[k]))


def _oracle_energy(system, xyz_by_mol, eps=None, sig=None, species=None):
    s = copy.copy(system)
    if species is not None:
        s.species = species
    with s.open(oracle.fns()) as o:
        if eps is not None:
            o.set_nonbond_table(eps, sig, system.ff.mie_n, system.ff.mie_m)
        m = s.molecules
        o.set_molecules(m.im, m.is_, m.ibox, np.concatenate([x.ravel() for x in xyz_by_mol]))
        return o.system_total_energy(1)[0]["total"]


def _gpu_gradient(system):
    with cg.open_system(system, precision=abi.PREC_FP64) as g:
        n = sum(system.species[system.molecules.is_[k] - 1].natoms for k in _box_order(system))
        return g.system_gradient(1, n)


def _lj_numpy_gradient(system):
    """Minimum-image LJ forces for a one-type, one-atom-per-molecule box."""
    m = system.molecules
    order = _box_order(system)
    x = np.array([m.xyz[k][0] for k in order])
    L = system.boxes[0].length[0]
    rc2 = system.boxes[0].rcut_vdw ** 2
    eps, sig2 = system.ff.eps[0, 0], system.ff.sig[0, 0] ** 2
    d = x[:, None, :] - x[None, :, :]
    d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
    r2 = (d ** 2).sum(-1)
    np.fill_diagonal(r2, np.inf)
    s6 = (sig2 / r2) ** 3
    dEdr2 = np.where(r2 <= rc2, 4 * eps * (-6 * s6 * s6 + 3 * s6) / r2, 0.0)
    return (2 * dEdr2[:, :, None] * d).sum(1)


def test_lj_gradient_matches_numpy_and_fd():
    s = mc_helpers.lj_small(nboxes=1)
    e, g, de, ds, dq = _gpu_gradient(s)
    ref = _lj_numpy_gradient(s)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(g - ref)) <= 1e-10 * scale
    # central differences of the oracle energy for a few coordinates and both LJ parameters
    m = s.molecules
    order = _box_order(s)
    rng = np.random.default_rng(1)
    for k in rng.choice(len(order), 4, replace=False):
        for d in range(3):
            xyz = [x.copy() for x in m.xyz]
            h = H_REL * max(1.0, abs(xyz[order[k]][0, d]))
            xyz[order[k]][0, d] += h
            ep = _oracle_energy(s, xyz)
            xyz[order[k]][0, d] -= 2 * h
            em = _oracle_energy(s, xyz)
            assert abs((ep - em) / (2 * h) - g[k, d]) <= FD_TOL * scale
    for tab, dref in (("eps", de[0, 0]), ("sig", ds[0, 0])):
        eps, sig = s.ff.eps.copy(), s.ff.sig.copy()
        t = eps if tab == "eps" else sig
        h = H_REL * t[0, 0]
        t[0, 0] += h
        ep = _oracle_energy(s, m.xyz, eps, sig)
        t[0, 0] -= 2 * h
        em = _oracle_energy(s, m.xyz, eps, sig)
        fd = (ep - em) / (2 * h)
        assert abs(fd - dref) <= 1e-6 * abs(fd), (tab, fd, dref)


STYLES = {"lj_cut_shift": (abi.VDW_LJ, abi.VDW_SUM_CUT_SHIFT), "lj_cut_switch": (abi.VDW_LJ, abi.VDW_SUM_CUT_SWITCH),
          "lj_cut_shift_force": (abi.VDW_LJ, abi.VDW_SUM_CUT_SHIFT_FORCE),
          "lj_minimum": (abi.VDW_LJ, abi.VDW_SUM_MINIMUM),
          "mie_cut": (abi.VDW_MIE, abi.VDW_SUM_CUT), "mie_cut_shift": (abi.VDW_MIE, abi.VDW_SUM_CUT_SHIFT)}


@pytest.mark.parametrize("name", list(STYLES))
def test_vdw_style_gradients_match_fd(name):
    """dU/dr, dU/d(eps) and dU/d(sigma) in the shifted, switched, shifted-force and
    minimum-image LJ sums and the Mie cut and cut_shift forms, against central
    differences of the oracle's energy (300 atoms, 10 A cutoff, switch 8-10 A)."""
    style, vsum = STYLES[name]
    vdw = ("Mie", 120.0, 3.4, 14.0, 6.0) if style == abi.VDW_MIE else ("LJ", 120.0, 3.4)
    s = helpers.lj_fluid_system(vsum, vdw, style)
    e, g, de, ds, dq = _gpu_gradient(s)
    m = s.molecules
    order = _box_order(s)
    scale = np.max(np.abs(g))
    rng = np.random.default_rng(7)
    for k in rng.choice(len(order), 4, replace=False):
        for d in range(3):
            xyz = [x.copy() for x in m.xyz]
            h = H_REL * max(1.0, abs(xyz[order[k]][0, d]))
            xyz[order[k]][0, d] += h
            ep = _oracle_energy(s, xyz)
            xyz[order[k]][0, d] -= 2 * h
            em = _oracle_energy(s, xyz)
            assert abs((ep - em) / (2 * h) - g[k, d]) <= FD_TOL * scale, (name, k, d)
    for tab, dref in (("eps", de[0, 0]), ("sig", ds[0, 0])):
        eps, sig = s.ff.eps.copy(), s.ff.sig.copy()
        t = eps if tab == "eps" else sig
        h = H_REL * t[0, 0]
        t[0, 0] += h
        ep = _oracle_energy(s, m.xyz, eps, sig)
        t[0, 0] -= 2 * h
        em = _oracle_energy(s, m.xyz, eps, sig)
        fd = (ep - em) / (2 * h)
        assert abs(fd - dref) <= 1e-6 * abs(fd), (name, tab, fd, dref)


def test_water_ewald_gradient_matches_fd():
    s = mc_helpers.water_small()
    e, g, de, ds, dq = _gpu_gradient(s)
    m = s.molecules
    order = _box_order(s)
    scale = np.max(np.abs(g))
    rng = np.random.default_rng(2)
    for atom in rng.choice(len(order) * 3, 5, replace=False):
        k, a = divmod(int(atom), 3)
        for d in range(3):
            xyz = [x.copy() for x in m.xyz]
            h = H_REL * max(1.0, abs(xyz[order[k]][a, d]))
            xyz[order[k]][a, d] += h
            ep = _oracle_energy(s, xyz)
            xyz[order[k]][a, d] -= 2 * h
            em = _oracle_energy(s, xyz)
            assert abs((ep - em) / (2 * h) - g[3 * k + a, d]) <= FD_TOL * scale, (k, a, d)
    # charge of the oxygen (all molecules) and the O-O LJ parameters
    for ia in (0, 1):
        sp = copy.deepcopy(s.species)
        q0 = sp[0].atoms[ia].charge
        h = H_REL * abs(q0)
        sp[0].atoms[ia].charge = q0 + h
        ep = _oracle_energy(s, m.xyz, species=sp)
        sp[0].atoms[ia].charge = q0 - h
        em = _oracle_energy(s, m.xyz, species=sp)
        fd = (ep - em) / (2 * h)
        assert abs(fd - dq[ia]) <= 1e-6 * abs(fd), (ia, fd, dq[ia])
    for tab, dref in (("eps", de[0, 0]), ("sig", ds[0, 0])):
        eps, sig = s.ff.eps.copy(), s.ff.sig.copy()
        t = eps if tab == "eps" else sig
        h = H_REL * t[0, 0]
        t[0, 0] += h
        ep = _oracle_energy(s, m.xyz, eps, sig)
        t[0, 0] -= 2 * h
        em = _oracle_energy(s, m.xyz, eps, sig)
        fd = (ep - em) / (2 * h)
        assert abs(fd - dref) <= 1e-6 * abs(fd), (tab, fd, dref)


def test_autograd_function_chain_rule():
    torch = pytest.importorskip("torch")
    from cassandra_gb300.autograd import BoxEnergy, BoxModel, lorentz_berthelot

    s = mc_helpers.lj_small(nboxes=1)
    model = BoxModel(s)
    try:
        xyz = torch.tensor(model.initial_xyz(), dtype=torch.float64, requires_grad=True)
        eps_t = torch.tensor([s.ff.eps[0, 0]], dtype=torch.float64, requires_grad=True)
        sig_t = torch.tensor([s.ff.sig[0, 0]], dtype=torch.float64, requires_grad=True)
        q = torch.tensor(model.charges(), dtype=torch.float64, requires_grad=True)
        et, st = lorentz_berthelot(eps_t, sig_t)
        E = BoxEnergy.apply(xyz, et, st, q, model)
        E.backward()
        e_ref, g, de, ds, _ = model.ctx.system_gradient(1, model.n_atoms)
        assert abs(E.item() - e_ref["total"]) <= 1e-12 * abs(e_ref["total"])
        assert np.allclose(xyz.grad.numpy(), g, rtol=0, atol=1e-12 * np.max(np.abs(g)))
        # per-type epsilon through the mixing rule: finite differences of the Function itself
        h = H_REL * eps_t.item()
        with torch.no_grad():
            ep = BoxEnergy.apply(xyz, *lorentz_berthelot(eps_t + h, sig_t), q, model).item()
            em = BoxEnergy.apply(xyz, *lorentz_berthelot(eps_t - h, sig_t), q, model).item()
        fd = (ep - em) / (2 * h)
        assert abs(eps_t.grad.item() - fd) <= 1e-6 * abs(fd)
    finally:
        model.close()


def test_flexible_pentane_gradient_matches_fd():
    """Pentane (60 molecules from the reference's pregen example) with its
    harmonic angles and Ryckaert-Bellemans dihedrals, plus harmonic bonds (k 450
    K/A^2) and a harmonic improper per molecule added for the test: dU/dr against
    central differences of the oracle's energy, every atom of three molecules."""
    s = helpers.pregen_system("pentane", 0)
    sp = copy.deepcopy(s.species[0])
    sp.bonds = [(a, b, "harmonic", 450.0, 0.97 * l0) for (a, b, _, l0, _t) in sp.bonds]  # strained
    sp.impropers = [(1, 2, 3, 4, "harmonic", 25.0, 170.0)]
    s.species = [sp]
    e, g, de, ds, dq = _gpu_gradient(s)
    m = s.molecules
    order = _box_order(s)
    scale = np.max(np.abs(g))
    rng = np.random.default_rng(4)
    for k in rng.choice(len(order), 3, replace=False):
        for a in range(sp.natoms):
            for d in range(3):
                xyz = [x.copy() for x in m.xyz]
                h = H_REL * max(1.0, abs(xyz[order[k]][a, d]))
                xyz[order[k]][a, d] += h
                ep = _oracle_energy(s, xyz)
                xyz[order[k]][a, d] -= 2 * h
                em = _oracle_energy(s, xyz)
                assert abs((ep - em) / (2 * h) - g[sp.natoms * k + a, d]) <= FD_TOL * scale, (k, a, d)


def test_gradient_rejects_charmm():
    s = helpers.lj_fluid_system(abi.VDW_SUM_CHARMM)
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        with pytest.raises(abi.CassError) as e:
            g.system_gradient(1, 300)
        assert e.value.code == abi.CASS_EUNSUPPORTED
