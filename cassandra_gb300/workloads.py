"""Seeded synthetic systems with the shapes of the benchmark configurations.

* lj_fluid_box        -- single-site LJ spheres placed uniformly at random with
                         overlaps below a minimum distance rejected (the
                         500-sphere NVT case and the frozen Widom boxes);
* butane_species      -- 4-site united-atom n-butane (TraPPE-like parameters of
                         the pentane fixture) with CBMC fragments and fragment
                         libraries sampled from the Boltzmann distribution of the
                         harmonic bend (p(theta) ~ sin(theta) exp(-beta k (theta-theta0)^2));
* widom_batch_system  -- nboxes frozen LJ boxes of uneven size (N uniform in
                         [nmin, nmax], reduced density rho* = 0.6) plus the
                         butane solute species, for batched CBMC Widom insertion;
* water_box           -- rigid 3-site SPC/E-like water on a lattice with
                         random orientations.
Nothing here is on the timed path.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .system import Atom, BoxSpec, ForceField, MoleculeSet, Species, System, KBOLTZ


def lj_fluid_box(n: int, length: float, min_dist: float, rng: np.random.Generator) -> np.ndarray:
    """Random sequential addition in [-L/2, L/2)^3 with a cell grid for the overlap test."""
    nc = max(1, int(length // min_dist))
    cell = length / nc
    grid: dict = {}
    pos = np.zeros((n, 3))
    md2 = min_dist * min_dist
    k = 0
    tries = 0
    while k < n:
        tries += 1
        if tries > 200 * n + 10000:
            raise RuntimeError("could not place all spheres")
        p = (rng.random(3) - 0.5) * length
        c = tuple(int((p[d] + 0.5 * length) // cell) % nc for d in range(3))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get(((c[0] + dx) % nc, (c[1] + dy) % nc, (c[2] + dz) % nc), ()):
                        d = pos[j] - p
                        d -= length * np.round(d / length)
                        if d @ d < md2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pos[k] = p
            grid.setdefault(c, []).append(k)
            k += 1
    return pos


def lj_sphere_species(eps_K: float = 148.0, sigma: float = 3.73, name: str = "LJ") -> Species:
    return Species(atoms=[Atom(name, 16.04, 0.0, ("LJ", eps_K, sigma))], scale_vdw=(0, 0, 0, 0),
                   scale_qq=(0, 0, 0, 0), fragments=[[1]], libraries=[np.zeros((1, 1, 3))])


def _bend_library(nconfig: int, bond: float, theta0_deg: float, k_K: float, temperature: float,
                  rng: np.random.Generator) -> np.ndarray:
    """[nconfig, 3, 3]: anchor at the origin, atom 2 on +x, atom 3 in the xy plane at the sampled angle."""
    beta_k = k_K / temperature  # k in K/rad^2, E/kT = beta k (theta - theta0)^2
    t0 = math.radians(theta0_deg)
    out = np.zeros((nconfig, 3, 3))
    width = 6.0 / math.sqrt(2.0 * beta_k)
    lo, hi = max(1e-3, t0 - width), min(math.pi - 1e-3, t0 + width)
    fmax = 1.0
    k = 0
    while k < nconfig:
        th = lo + (hi - lo) * rng.random()
        f = math.sin(th) * math.exp(-beta_k * (th - t0) ** 2)
        if rng.random() * fmax < f:
            out[k, 1] = (bond, 0.0, 0.0)
            out[k, 2] = (bond * math.cos(th), bond * math.sin(th), 0.0)
            k += 1
    return out


def butane_species(temperature: float = 150.0, nconfig: int = 1000, seed: int = 7, eps_scale: float = 1.0) -> Species:
    """n-butane, united atom: CH3-CH2-CH2-CH3, fixed 1.54 A bonds, harmonic 114 deg bend
    (k = 31250 K/rad^2 in the E = k (theta-theta0)^2 form), OPLS dihedral of the pentane fixture.
    eps_scale = 0 gives the ideal (non-interacting) chain."""
    rng = np.random.default_rng(seed)
    atoms = [Atom("CH3", 15.034, 0.0, ("LJ", 98.0 * eps_scale, 3.75)),
             Atom("CH2", 14.027, 0.0, ("LJ", 46.0 * eps_scale, 3.95)),
             Atom("CH2", 14.027, 0.0, ("LJ", 46.0 * eps_scale, 3.95)),
             Atom("CH3", 15.034, 0.0, ("LJ", 98.0 * eps_scale, 3.75))]
    sp = Species(atoms=atoms,
                 bonds=[(1, 2, "fixed", 1.54), (2, 3, "fixed", 1.54), (3, 4, "fixed", 1.54)],
                 angles=[(1, 2, 3, "harmonic", 31250.0, 114.0), (2, 3, 4, "harmonic", 31250.0, 114.0)],
                 dihedrals=[(1, 2, 3, 4, "OPLS", 0.0, 2.952, -0.567, 6.579)],
                 scale_vdw=(0.0, 0.0, 0.0, 1.0), scale_qq=(0.0, 0.0, 0.0, 1.0),
                 fragments=[[2, 1, 3], [3, 2, 4]], frag_connect=[(1, 2)])
    sp.libraries = [_bend_library(nconfig, 1.54, 114.0, 31250.0, temperature, rng) for _ in range(2)]
    return sp


def widom_batch_system(nboxes: int = 64, nmin: int = 200, nmax: int = 4000, rho_star: float = 0.6,
                       sigma: float = 3.73, eps_K: float = 148.0, temperature: float = 150.0,
                       rcut: float = 14.0, rcut_cbmc: float = 6.5, rcut_low: float = 2.0,
                       seed: int = 2024, nconfig: int = 1000, sizes=None) -> System:
    rng = np.random.default_rng(seed)
    if sizes is None:
        sizes = rng.integers(nmin, nmax + 1, size=nboxes)
    sizes = [int(s) for s in sizes]
    solvent = lj_sphere_species(eps_K, sigma)
    solute = butane_species(temperature, nconfig, seed + 1)
    ff = ForceField([solvent, solute])
    boxes, ms = [], MoleculeSet()
    loc = 1
    for b, n in enumerate(sizes):
        L = (n / rho_star) ** (1.0 / 3.0) * sigma
        pos = lj_fluid_box(n, L, 0.8 * sigma, rng)
        for p in pos:
            ms.add(loc, 1, b + 1, p[None, :])
            loc += 1
        boxes.append(BoxSpec(length=(L, L, L), rcut_vdw=min(rcut, 0.5 * L), rcut_cbmc=rcut_cbmc, rcut_low=rcut_low,
                             temperature=temperature))
    return System([solvent, solute], boxes, ms, ff, [loc - 1, 1])


def water_species(nconfig: int = 1) -> Species:
    """Rigid 3-site water of the benchmark: O-H 1.0 A, H-O-H 109.47 deg, SPC/E charges, O-only LJ."""
    t = math.radians(109.47)
    lib = np.array([[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [math.cos(t), math.sin(t), 0.0]]] * nconfig)
    return Species(atoms=[Atom("O", 15.999, -0.8476, ("LJ", 78.2, 3.166)), Atom("H", 1.008, 0.4238, ("LJ", 0.0, 0.0)),
                          Atom("H", 1.008, 0.4238, ("LJ", 0.0, 0.0))],
                   bonds=[(1, 2, "fixed", 1.0), (1, 3, "fixed", 1.0)], angles=[(2, 1, 3, "fixed", 109.47)],
                   scale_vdw=(0, 0, 0, 1.0), scale_qq=(0, 0, 0, 1.0), fragments=[[1, 2, 3]], libraries=[lib])


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_box(nmol: int, length: float, temperature: float = 298.0, rcut: float = 9.8, tol: float = 1e-5,
              seed: int = 11) -> System:
    rng = np.random.default_rng(seed)
    sp = water_species()
    ff = ForceField([sp])
    n_side = int(math.ceil(nmol ** (1.0 / 3.0)))
    a = length / n_side
    base = sp.libraries[0][0]
    com = (base * np.array([15.999, 1.008, 1.008])[:, None]).sum(0) / (15.999 + 2 * 1.008)
    ms = MoleculeSet()
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                if k >= nmol:
                    break
                c = (np.array([ix, iy, iz]) + 0.5) * a - 0.5 * length
                xyz = (base - com) @ random_rotation(rng).T + c
                ms.add(k + 1, 1, 1, xyz)
                k += 1
    bx = BoxSpec(length=(length,) * 3, rcut_vdw=rcut, rcut_coul=rcut, rcut_cbmc=min(6.5, rcut), rcut_low=0.85,
                 charge_style=abi.CHARGE_COUL, charge_sum_style=abi.QQ_EWALD, ewald_tol=tol, temperature=temperature)
    return System([sp], [bx], ms, ff, [nmol])


def lj_nvt_system(nboxes: int = 1, n: int = 500, length: float = 35.0, sigma: float = 3.73, eps_K: float = 148.0,
                  temperature: float = 150.0, rcut: float = 14.0, rcut_low: float = 1.0, seed: int = 2024) -> System:
    """Single-site LJ fluid for NVT translation MC: n spheres per cubic box, uniform random
    start with overlaps below 0.8 sigma rejected; boxes are independent replicas."""
    rng = np.random.default_rng(seed)
    sp = lj_sphere_species(eps_K, sigma)
    ff = ForceField([sp])
    boxes, ms = [], MoleculeSet()
    loc = 1
    for b in range(nboxes):
        for p in lj_fluid_box(n, length, 0.8 * sigma, rng):
            ms.add(loc, 1, b + 1, p[None, :])
            loc += 1
        boxes.append(BoxSpec(length=(length,) * 3, rcut_vdw=rcut, rcut_cbmc=min(6.5, rcut), rcut_low=rcut_low,
                             temperature=temperature))
    return System([sp], boxes, ms, ff, [loc - 1])


def water_nvt_system(nboxes: int = 1, nmol: int = 256, length: float = 19.7, temperature: float = 298.0,
                     rcut: float = 9.8, tol: float = 1e-5, seed: int = 11) -> System:
    """Rigid 3-site water on a lattice with random orientations, LJ + Ewald; boxes are
    independent replicas (each its own orientations)."""
    rng = np.random.default_rng(seed)
    sp = water_species()
    ff = ForceField([sp])
    n_side = int(math.ceil(nmol ** (1.0 / 3.0)))
    a = length / n_side
    base = sp.libraries[0][0]
    com = (base * np.array([15.999, 1.008, 1.008])[:, None]).sum(0) / (15.999 + 2 * 1.008)
    ms, boxes = MoleculeSet(), []
    loc = 1
    for b in range(nboxes):
        k = 0
        for ix in range(n_side):
            for iy in range(n_side):
                for iz in range(n_side):
                    if k >= nmol:
                        break
                    c = (np.array([ix, iy, iz]) + 0.5) * a - 0.5 * length
                    ms.add(loc, 1, b + 1, (base - com) @ random_rotation(rng).T + c)
                    loc += 1
                    k += 1
        boxes.append(BoxSpec(length=(length,) * 3, rcut_vdw=rcut, rcut_coul=rcut, rcut_cbmc=min(6.5, rcut),
                             rcut_low=0.85, charge_style=abi.CHARGE_COUL, charge_sum_style=abi.QQ_EWALD,
                             ewald_tol=tol, temperature=temperature))
    return System([sp], boxes, ms, ff, [loc - 1])


def water_gradient_system(nmol: int = 4096, length: float = 49.7, temperature: float = 298.0, rcut: float = 12.0,
                          tol: float = 1e-6, min_inter: float = 1.5, seed: int = 13, nboxes: int = 1) -> System:
    """Rigid 3-site waters on a cubic lattice with random orientations, each
    orientation redrawn until its atoms are at least min_inter from every atom
    of the molecules already placed; one Ewald box (the gradient workload).
    With nboxes > 1 the further boxes are copies of the first shifted by a
    random periodic translation (replicas for independent chains)."""
    rng = np.random.default_rng(seed)
    sp = water_species()
    ff = ForceField([sp])
    n_side = int(math.ceil(nmol ** (1.0 / 3.0)))
    a = length / n_side
    base = sp.libraries[0][0]
    com = (base * np.array([15.999, 1.008, 1.008])[:, None]).sum(0) / (15.999 + 2 * 1.008)
    ms = MoleculeSet()
    placed = {}  # lattice site -> atoms
    md2 = min_inter * min_inter
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                if k >= nmol:
                    break
                c = (np.array([ix, iy, iz]) + 0.5) * a - 0.5 * length
                near = [placed[(ix + dx) % n_side, (iy + dy) % n_side, (iz + dz) % n_side]
                        for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)
                        if ((ix + dx) % n_side, (iy + dy) % n_side, (iz + dz) % n_side) in placed]
                others = np.concatenate(near) if near else np.zeros((0, 3))
                for _ in range(1000):
                    xyz = (base - com) @ random_rotation(rng).T + c
                    d = xyz[:, None, :] - others[None, :, :]
                    d -= length * np.round(d / length)
                    if not others.size or (d ** 2).sum(-1).min() >= md2:
                        break
                placed[(ix, iy, iz)] = xyz
                ms.add(k + 1, 1, 1, xyz)
                k += 1
    boxes = [BoxSpec(length=(length,) * 3, rcut_vdw=rcut, rcut_coul=rcut, rcut_cbmc=min(6.5, rcut), rcut_low=0.85,
                     charge_style=abi.CHARGE_COUL, charge_sum_style=abi.QQ_EWALD, ewald_tol=tol,
                     temperature=temperature) for _ in range(nboxes)]
    first = list(ms.xyz)
    for b in range(2, nboxes + 1):
        shift = rng.uniform(-0.5 * length, 0.5 * length, 3)
        for m, xyz in enumerate(first):
            x = xyz + shift
            c = x.mean(0)
            x = x - length * np.round(c / length)  # fold by the molecule's centre
            ms.add(m + 1 + (b - 1) * nmol, 1, b, x)
    return System([sp], boxes, ms, ff, [nmol * nboxes])


def gcmc_system(nboxes: int = 16, length: float = 40.0, temperature: float = 300.0, rcut: float = 14.0,
                rcut_cbmc: float = 6.5, rcut_low: float = 1.0, max_per_box: int = 800, seed: int = 2025,
                nconfig: int = 1000, eps_scale: float = 1.0) -> System:
    """Empty cubic boxes for grand-canonical runs of the n-butane chain (one species)."""
    sp = butane_species(temperature, nconfig, seed, eps_scale)
    ff = ForceField([sp])
    boxes = [BoxSpec(length=(length,) * 3, rcut_vdw=rcut, rcut_cbmc=rcut_cbmc, rcut_low=rcut_low,
                     temperature=temperature) for _ in range(nboxes)]
    return System([sp], boxes, MoleculeSet(), ff, [max_per_box * nboxes])


def water_gcmc_system(nboxes: int = 2, nmol: int = 27, length: float = 16.0, temperature: float = 298.0,
                      rcut: float = 7.0, tol: float = 1e-5, max_per_box: int = 120, seed: int = 11) -> System:
    """Rigid 3-site waters (LJ + Ewald) on a lattice with random orientations in
    boxes with free slots, for grand-canonical runs of a charged species."""
    s = water_nvt_system(nboxes=nboxes, nmol=nmol, length=length, temperature=temperature, rcut=rcut, tol=tol,
                         seed=seed)
    s.max_molecules = [max_per_box * nboxes]
    return s


def ideal_gas_system(nboxes: int = 2, length: float = 30.0, temperature: float = 300.0,
                     max_per_box: int = 400) -> System:
    """Non-interacting spheres (epsilon 0) for checks of the grand-canonical acceptance rules."""
    sp = lj_sphere_species(0.0, 3.0, name="IG")
    ff = ForceField([sp])
    boxes = [BoxSpec(length=(length,) * 3, rcut_vdw=10.0, rcut_cbmc=6.5, rcut_low=1e-3,
                     temperature=temperature) for _ in range(nboxes)]
    return System([sp], boxes, MoleculeSet(), ff, [max_per_box * nboxes])
