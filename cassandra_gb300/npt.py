"""NPT Monte Carlo over the C-ABI, with the loop shape of nptmc_driver.f90:
blocks of translate / rotate sweeps on the device (cass_mc_sweeps, one chain
per box) alternating with one volume move per box (Volume_Change,
move_volume.f90:24-679) whose random draw, acceptance rule and counters are
here on the host and whose rebuild runs on the device
(cass_volume_scale / cass_volume_restore).

Units are Cassandra's: energies in amu A^2/ps^2, pressure given in bar and
divided by atomic_to_bar (global_variables.f90:201, input_routines.f90:
4179-4183)."""
from __future__ import annotations

import math

import numpy as np

KBOLTZ = 0.8314472
ATOMIC_TO_BAR = 166.054
MAX_KBT = 708.0


def accept(ln_pacc: float, u: float) -> bool:
    """accept_or_reject (accept_or_reject.f90:22-65)."""
    if ln_pacc <= 0.0:
        return True
    if ln_pacc < MAX_KBT:
        return u <= math.exp(-ln_pacc)
    return False


class NPTChains:
    """NPT chains of the listed cubic boxes of an open context (GPU or oracle)."""

    def __init__(self, ctx, boxes, n_molecules, temperature: float, pressure_bar: float, dv_max, max_disp,
                 max_rot, seed: int):
        self.ctx = ctx
        self.boxes = list(boxes)
        self.n = list(n_molecules)
        self.beta = 1.0 / (KBOLTZ * temperature)
        self.p = pressure_bar / ATOMIC_TO_BAR
        self.dv_max = np.broadcast_to(np.asarray(dv_max, dtype=np.float64), (len(self.boxes),)).copy()
        self.max_disp = np.array(max_disp, dtype=np.float64)
        self.max_rot = np.array(max_rot, dtype=np.float64)
        self.rng = np.random.default_rng(seed)
        self.seed = seed
        self.block = 0
        self.length = [None] * len(self.boxes)
        self.energy = [None] * len(self.boxes)   # running total energy of each box
        self.components = [None] * len(self.boxes)  # its components (CassEnergy as a dict)
        self.n_vol = np.zeros(len(self.boxes), dtype=np.int64)
        self.n_vol_acc = np.zeros(len(self.boxes), dtype=np.int64)

    def start(self, lengths) -> None:
        for k, b in enumerate(self.boxes):
            e, ov = self.ctx.system_total_energy(b)
            if ov:
                raise RuntimeError(f"box {b} starts with an overlap")
            self.energy[k] = e["total"]
            self.components[k] = e
            self.length[k] = float(lengths[k])

    def sweeps(self, nsweeps: int, prob_translate: float = 1.0) -> None:
        res, self.max_disp, self.max_rot = self.ctx.mc_sweeps(
            self.boxes, nsweeps, self.max_disp, self.max_rot, seed=self.seed * 7919 + self.block,
            prob_translate=prob_translate)
        self.block += 1
        for k, r in enumerate(res):
            self.energy[k] = r["energy"]["total"]
            self.components[k] = r["energy"]

    def volume_moves(self) -> None:
        for k, b in enumerate(self.boxes):
            self.n_vol[k] += 1
            L = self.length[k]
            v_old = L ** 3
            dv = (1.0 - 2.0 * self.rng.random()) * self.dv_max[k]  # move_volume.f90:147-148
            v_new = v_old + dv
            u = self.rng.random()
            if v_new <= 0.0:
                continue
            L_new = v_new ** (1.0 / 3.0)
            e_new, ov = self.ctx.volume_scale(b, L_new)
            if ov:
                self.ctx.volume_restore(b)
                continue
            ln_pacc = (self.beta * (e_new["total"] - self.energy[k]) + self.beta * self.p * dv -
                       self.n[k] * math.log(v_new / v_old))  # move_volume.f90:443-446
            if accept(ln_pacc, u):
                self.n_vol_acc[k] += 1
                self.length[k] = L_new
                self.energy[k] = e_new["total"]
                self.components[k] = e_new
            else:
                self.ctx.volume_restore(b)

    def densities(self, mass_per_molecule_amu: float) -> np.ndarray:
        """Mass densities in g/cm^3."""
        v = np.array(self.length) ** 3 * 1e-24
        return np.array(self.n) * mass_per_molecule_amu / 6.02214076e23 / v
