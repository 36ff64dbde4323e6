"""System builders shared by the tests (golden fixtures and small synthetic cases)."""
from __future__ import annotations

import json
import os

import numpy as np

from cassandra_gb300 import abi
from cassandra_gb300.io import read_mcf
from cassandra_gb300.system import Atom, BoxSpec, ForceField, MoleculeSet, Species, System

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATOMIC_TO_KJMOL = 0.01


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def single_atom_system(coords, box_len, vdw=("LJ", 120.272, 3.54), vdw_style=abi.VDW_LJ,
                       vdw_sum=abi.VDW_SUM_CUT_TAIL, rcut=10.62, rcut_low=0.0, charge=0.0,
                       temperature=300.0, extra_slots=1):
    sp = Species(atoms=[Atom("LJ", 1.0, charge, vdw)], scale_vdw=(0, 0, 0, 0), scale_qq=(0, 0, 0, 0),
                 fragments=[[1]], libraries=[np.zeros((1, 1, 3))])
    ff = ForceField([sp], style=vdw_style)
    coords = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    ms = MoleculeSet()
    for k, x in enumerate(coords):
        ms.add(k + 1, 1, 1, x)
    bx = BoxSpec(length=(box_len,) * 3, vdw_style=vdw_style, vdw_sum_style=vdw_sum, rcut_vdw=rcut,
                 rcut_cbmc=min(6.5, rcut), rcut_low=rcut_low, temperature=temperature)
    return System([sp], [bx], ms, ff, [len(coords) + extra_slots])


def water_species(atoms_json=None, mcf_text=None):
    if mcf_text is not None:
        return read_mcf(mcf_text)
    atoms = json.loads(atoms_json)[0]
    at = [Atom(a[0], a[2], a[3], ("LJ", a[5], a[6])) for a in atoms]
    return Species(atoms=at, bonds=[(1, 2, "fixed", 1.0), (1, 3, "fixed", 1.0)],
                   angles=[(2, 1, 3, "fixed", 109.47)], scale_vdw=(0, 0, 0, 1.0), scale_qq=(0, 0, 0, 1.0),
                   fragments=[[1, 2, 3]])


def nist_spce_system(k: int) -> System:
    d = golden("nist_spce.npz")
    nmol, L, rc, tol = d["checks"][k][:4]
    sp = water_species(str(d["atoms"]))
    ff = ForceField([sp])
    xyz = d[f"xyz{k}"]
    ms = MoleculeSet()
    for m in range(int(nmol)):
        ms.add(m + 1, 1, 1, xyz[3 * m:3 * m + 3])
    bx = BoxSpec(length=(L,) * 3, rcut_vdw=10.0, rcut_coul=rc, rcut_low=0.85, charge_style=abi.CHARGE_COUL,
                 charge_sum_style=abi.QQ_EWALD, ewald_tol=tol, temperature=300.0)
    return System([sp], [bx], ms, ff, [int(nmol) + 1])


def _inp_sections(text):
    out, cur = {}, None
    for raw in text.splitlines():
        line = raw.split("!")[0].strip()
        if not line:
            continue
        if line.startswith("#"):
            cur = line[1:].strip().split()[0]
            out[cur] = []
        elif cur:
            out[cur].append(line.split())
    return out


def pregen_system(name: str, frame: int) -> System:
    d = golden(f"pregen_{name}.npz")
    inp = _inp_sections(str(d["inp"]))
    sp = read_mcf(str(d["mcf"]))
    nmol = int(inp["Molecule_Files"][0][1])
    mixing = inp.get("Mixing_Rule", [["LB"]])[0][0]
    ff = ForceField([sp], mixing=mixing)
    vdw = inp["VDW_Style"][0]
    sums = {"cut_tail": abi.VDW_SUM_CUT_TAIL, "cut": abi.VDW_SUM_CUT, "cut_shift": abi.VDW_SUM_CUT_SHIFT}
    bx = BoxSpec(length=tuple(d["boxes"][frame]), vdw_style=abi.VDW_LJ, vdw_sum_style=sums[vdw[1].lower()],
                 rcut_vdw=float(vdw[2]), rcut_low=float(inp["Rcutoff_Low"][0][0]),
                 temperature=float(inp["Temperature_Info"][0][0]))
    if "Charge_Style" in inp and inp["Charge_Style"][0][0].lower() == "coul":
        cs = inp["Charge_Style"][0]
        bx.charge_style = abi.CHARGE_COUL
        bx.charge_sum_style = abi.QQ_EWALD
        bx.rcut_coul = float(cs[2])
        bx.ewald_tol = float(cs[3])
    cbmc = {r[0]: r[1] for r in inp.get("CBMC_Info", []) if len(r) > 1}
    if "rcut_cbmc" in cbmc:
        bx.rcut_cbmc = float(cbmc["rcut_cbmc"])
    xyz = d["frames"][frame]
    na = sp.natoms
    ms = MoleculeSet()
    for m in range(nmol):
        ms.add(m + 1, 1, 1, xyz[na * m:na * (m + 1)])
    return System([sp], [bx], ms, ff, [nmol + 1])


def pentane_widom_system(frame: int) -> System:
    """A frame of the reference's pentane Widom fixture with its fragment libraries
    (exampleResources/Widom/pentane: 60 united-atom pentanes in a 100 A box, 336 K,
    rcut_low 2 A, rcut_cbmc 6.5 A, 14 A cut_tail)."""
    s = pregen_system("pentane", frame)
    d = golden("widom_pentane.npz")
    s.species[0].libraries = [d["frag1"], d["frag2"], d["frag3"]]
    return s


def de_broglie(system: System, is_: int = 1, ibox: int = 1) -> float:
    """h / sqrt(2 pi m kT) in A with the reference's h_plank and kboltz (input_routines.f90:4265-4268)."""
    import math
    T = system.boxes[ibox - 1].temperature
    beta = 1.0 / (0.8314472 * T)
    mw = sum(a.mass for a in system.species[is_ - 1].atoms)
    return 39.9031268605 * math.sqrt(beta / (2.0 * math.pi * mw))


def pair_magnitude_scale(s, q_xyz, q_types, q_charges, skip_im, rc):
    """Sum of |plain LJ| + |bare Coulomb| over the box-1 pairs of the query atoms within rc
    (minimum image; rc None: every pair): the magnitude scale of a mixed-precision energy."""
    bx = s.boxes[0]
    L = np.asarray(bx.length, dtype=np.float64)
    m = s.molecules
    tot = 0.0
    for k in range(len(m.im)):
        if m.ibox[k] != 1 or (m.is_[k] == 1 and m.im[k] == skip_im):
            continue
        sp = s.species[m.is_[k] - 1]
        for ja, pj in enumerate(m.xyz[k]):
            tj = sp.type_index[ja]
            qj = sp.atoms[ja].charge
            for pa, ta, qa in zip(q_xyz, q_types, q_charges):
                d = pa - pj
                d -= L * np.round(d / L)
                r2 = float(d @ d)
                if rc is not None and r2 > rc * rc:
                    continue
                if ta > 0 and tj > 0:
                    eps, sig = s.ff.eps[ta - 1][tj - 1], s.ff.sig[ta - 1][tj - 1]
                    s6 = (sig * sig / r2) ** 3
                    tot += abs(4.0 * eps * (s6 * s6 - s6))
                tot += abs(138935.4558 * qa * qj / np.sqrt(r2))
    return tot


def lj_fluid_system(vdw_sum, vdw=("LJ", 120.0, 3.4), style=abi.VDW_LJ):
    """300 single-site LJ (or Mie) atoms in a 25 A box, cutoff 10 A (switch 8-10 A)."""
    from cassandra_gb300 import workloads
    rng = np.random.default_rng(5)
    xyz = workloads.lj_fluid_box(300, 25.0, 3.0, rng)
    s = single_atom_system(xyz, 25.0, vdw=vdw, vdw_style=style, vdw_sum=vdw_sum, rcut=10.0, rcut_low=1.0,
                           extra_slots=2)
    if vdw_sum == abi.VDW_SUM_CUT_SWITCH:
        s.boxes[0].ron_switch, s.boxes[0].roff_switch = 8.0, 10.0
    return s
