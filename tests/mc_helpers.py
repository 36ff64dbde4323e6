"""Small NVT Monte Carlo systems shared by the CPU and GPU sweep tests."""
from __future__ import annotations

import numpy as np

from cassandra_gb300 import workloads


def lj_small(nboxes: int = 2, seed: int = 5):
    # 200 spheres at the density of the 500-sphere, 35 A benchmark box
    L = 35.0 * (200 / 500) ** (1.0 / 3.0)
    return workloads.lj_nvt_system(nboxes=nboxes, n=200, length=L, rcut=12.0, seed=seed)


def water_small(nboxes: int = 1, seed: int = 3):
    # 64 waters at the density of the 256-water, 19.7 A benchmark box; 6 A cutoffs
    L = 19.7 * (64 / 256) ** (1.0 / 3.0)
    return workloads.water_nvt_system(nboxes=nboxes, nmol=64, length=L, rcut=6.0, seed=seed)


def positions(ctx, system) -> np.ndarray:
    m = system.molecules
    return np.concatenate([ctx.get_molecule(im, is_).ravel() for im, is_ in zip(m.im, m.is_)])


def recomputed_totals(fns, system, xyz, boxes):
    """FP64 energies of the configuration xyz, from a fresh context on `fns`."""
    m = system.molecules
    ctx = system.open(fns)
    with ctx:
        ctx.set_molecules(m.im, m.is_, m.ibox, xyz)
        return [ctx.system_total_energy(b)[0] for b in boxes]
