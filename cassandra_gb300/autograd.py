"""torch.autograd.Function over the C-ABI: a box's total energy and its adjoint.

`BoxEnergy.apply(xyz, eps_table, sig_table, charges, model)` returns the total
energy of one box (Cassandra's internal units, amu A^2/ps^2) as computed by
`cass_system_total_energy`, and back-propagates the derivatives that
`cass_system_gradient` returns:

* xyz       [n_atoms, 3]  coordinates of the box's live molecules, species-major
                          and in locate order (``BoxModel.order``);
* eps_table [nt, nt]      mixed LJ epsilon table (symmetric);
* sig_table [nt, nt]      mixed LJ sigma table (symmetric);
* charges   [sum natoms]  charge of each species atom (shared by its molecules).

The tables enter the energy only through their symmetric pairs, so the
derivative of a symmetric pair parameter is split evenly between the two table
entries; building both entries from the same per-type parameters (for example
with `lorentz_berthelot`) then recovers the full derivative through autograd.
The forward pass runs on the GPU through the CUDA library; the backward pass
uses the adjoint computed in the same call.  Double precision throughout.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from . import abi


def lorentz_berthelot(eps: torch.Tensor, sig: torch.Tensor):
    """Mixed tables eps_tu = sqrt(eps_t eps_u), sigma_tu = (sigma_t + sigma_u)/2
    (create_nonbond_table.f90), differentiable in torch."""
    e = torch.sqrt(eps[:, None] * eps[None, :])
    s = 0.5 * (sig[:, None] + sig[None, :])
    return e, s


class BoxModel:
    """One box of a System on a GPU context, with the molecule order of the C-ABI."""

    def __init__(self, system, ibox: int = 1, device: int = 0):
        import cassandra_gb300 as cg
        self.system = system
        self.ibox = ibox
        self.species = [copy.deepcopy(sp) for sp in system.species]
        self.ctx = cg.open_system(system, precision=abi.PREC_FP64, device=device)
        m = system.molecules
        sel = [k for k, b in enumerate(m.ibox) if b == ibox]
        self.order = sorted(sel, key=lambda k: (m.is_[k], m.im[k]))  # species-major, locate order
        self.n_atoms = sum(self.species[m.is_[k] - 1].natoms for k in self.order)
        self._charges = np.concatenate([[a.charge for a in sp.atoms] for sp in self.species])

    def close(self) -> None:
        self.ctx.close()

    def initial_xyz(self) -> np.ndarray:
        m = self.system.molecules
        return np.concatenate([m.xyz[k] for k in self.order])

    def charges(self) -> np.ndarray:
        return self._charges.copy()

    def evaluate(self, xyz: np.ndarray, eps: np.ndarray, sig: np.ndarray, q: np.ndarray):
        """Energy and adjoint at (xyz, tables, charges); returns (E, dU/dxyz, dU/deps, dU/dsig, dU/dq)."""
        m = self.system.molecules
        if not np.array_equal(q, self._charges):
            off = 0
            for k, sp in enumerate(self.species):
                for a, at in enumerate(sp.atoms):
                    at.charge = float(q[off + a])
                off += sp.natoms
                self.ctx.set_species(k + 1, sp)
            self._charges = np.array(q, dtype=np.float64)
        nt = eps.shape[0]
        self.ctx.set_nonbond_table(np.asarray(eps, dtype=np.float64), np.asarray(sig, dtype=np.float64),
                                   np.zeros((nt, nt)), np.zeros((nt, nt)))
        self.ctx.set_molecules([m.im[k] for k in self.order], [m.is_[k] for k in self.order],
                               [m.ibox[k] for k in self.order], np.asarray(xyz, dtype=np.float64).ravel())
        e, g, de, ds, dq = self.ctx.system_gradient(self.ibox, self.n_atoms)
        return e["total"], g, de, ds, dq


def _split_symmetric(d: np.ndarray) -> np.ndarray:
    """Derivative per table entry from the derivative per symmetric pair."""
    out = 0.5 * d
    np.fill_diagonal(out, np.diag(d))
    return out


class BoxEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, eps_table, sig_table, charges, model: BoxModel):
        E, g, de, ds, dq = model.evaluate(xyz.detach().cpu().numpy(), eps_table.detach().cpu().numpy(),
                                          sig_table.detach().cpu().numpy(), charges.detach().cpu().numpy())
        dev = xyz.device
        ctx.save_for_backward(torch.from_numpy(g).to(dev), torch.from_numpy(_split_symmetric(de)).to(dev),
                              torch.from_numpy(_split_symmetric(ds)).to(dev), torch.from_numpy(dq).to(dev))
        return torch.tensor(E, dtype=torch.float64, device=dev)

    @staticmethod
    def backward(ctx, grad_e):
        g, de, ds, dq = ctx.saved_tensors
        return grad_e * g, grad_e * de, grad_e * ds, grad_e * dq, None


def fluctuation_sensitivity(a: np.ndarray, dudtheta: np.ndarray, beta: float) -> float:
    """d<A>/dtheta = -beta (<A dU/dtheta> - <A><dU/dtheta>) over canonical samples of A and
    dU/dtheta taken on the same configurations (A itself independent of theta)."""
    a = np.asarray(a, dtype=np.float64)
    d = np.asarray(dudtheta, dtype=np.float64)
    return float(-beta * (np.mean(a * d) - np.mean(a) * np.mean(d)))
