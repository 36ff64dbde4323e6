"""Host-side description of species, boxes and force-field tables.

Mirrors the parts of Cassandra's input processing that feed the energy hot
path: unit conversions of the .mcf parameters (input_routines.f90:1573,
1904-1905, 2083-2098), the OPLS -> Ryckaert-Bellemans conversion
(input_routines.f90:2100-2106), the intramolecular scaling table
(create_intra_exclusion_table.f90:22-184) and the LB / geometric mixing rules
(create_nonbond_table.f90:331-372).  Everything here is plain numpy and runs
once per set-up; the per-step work happens in the CUDA library.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

# global_variables.f90:182-210 (truncated pi kept on purpose: it enters k-vectors, Cn, LRC)
PI = 3.1415926536
TWOPI = 6.2831853072
KBOLTZ = 0.8314472
KJMOL_TO_ATOMIC = 100.0
ATOMIC_TO_KJMOL = 0.01
CHARGE_FACTOR = 138935.4558


@dataclass
class Atom:
    name: str          # nonbond type name (.mcf column 2)
    mass: float
    charge: float
    vdw: tuple = ()    # ("LJ", eps_K, sigma) or ("Mie", eps_K, sigma, n, m) or () for none


@dataclass
class Species:
    """One molecule type, in .mcf terms (1-based atom indices)."""
    atoms: list
    bonds: list = field(default_factory=list)       # (a1, a2, "fixed"|"harmonic", p1, p2)
    angles: list = field(default_factory=list)      # (a1, a2, a3, "fixed", theta0_deg) | (.., "harmonic", k_K, theta0_deg)
    dihedrals: list = field(default_factory=list)   # (a1..a4, "OPLS", a0..a3 kJ/mol)
    impropers: list = field(default_factory=list)   # (a1..a4, "harmonic", k_K, phi0_deg)
    scale_vdw: tuple = (0.0, 0.0, 0.5, 1.0)         # 1-2, 1-3, 1-4, 1-N
    scale_qq: tuple = (0.0, 0.0, 0.5, 1.0)
    fragments: list = field(default_factory=list)   # list of atom lists, anchor first
    frag_connect: list = field(default_factory=list)  # list of (f1, f2) 1-based
    libraries: list = field(default_factory=list)   # per fragment: array [nconfig, natoms_f, 3]
    l_coul_cbmc: bool = False
    type_index: list = field(default_factory=list)  # filled by ForceField.assign_types (1-based, 0 = none)

    @property
    def natoms(self) -> int:
        return len(self.atoms)

    def intra_scale_tables(self):
        """vdw/charge intra scale and l_bonded, create_intra_exclusion_table.f90:35-120."""
        n = self.natoms
        sv = np.full((n, n), self.scale_vdw[3])
        sq = np.full((n, n), self.scale_qq[3])
        np.fill_diagonal(sv, 0.0)
        np.fill_diagonal(sq, 0.0)
        for d in self.dihedrals:
            i, j = d[0] - 1, d[3] - 1
            sv[i, j] = sv[j, i] = self.scale_vdw[2]
            sq[i, j] = sq[j, i] = self.scale_qq[2]
        for a in self.angles:
            i, j = a[0] - 1, a[2] - 1
            sv[i, j] = sv[j, i] = self.scale_vdw[1]
            sq[i, j] = sq[j, i] = self.scale_qq[1]
        bonded = np.zeros((n, n), dtype=np.int32)
        for b in self.bonds:
            i, j = b[0] - 1, b[1] - 1
            sv[i, j] = sv[j, i] = self.scale_vdw[0]
            sq[i, j] = sq[j, i] = self.scale_qq[0]
            bonded[i, j] = bonded[j, i] = 1
        return sv, sq, bonded

    def desc_arrays(self) -> dict:
        """Arrays of a CassSpeciesDesc (kept alive by the caller while the call runs)."""
        n = self.natoms
        sv, sq, bonded = self.intra_scale_tables()
        d: dict = {"natoms": n}
        d["atom_type"] = np.asarray(self.type_index, dtype=np.int32)
        d["charge"] = np.asarray([a.charge for a in self.atoms], dtype=np.float64)
        d["mass"] = np.asarray([a.mass for a in self.atoms], dtype=np.float64)
        d["vdw_intra_scale"] = np.ascontiguousarray(sv, dtype=np.float64).ravel()
        d["charge_intra_scale"] = np.ascontiguousarray(sq, dtype=np.float64).ravel()
        d["bonded"] = np.ascontiguousarray(bonded).ravel()
        ba, bk, bp = [], [], []
        for b in self.bonds:
            ba += [b[0], b[1]]
            if b[2].lower() == "fixed":
                bk.append(abi.BONDED_FIXED)
                bp += [b[3], b[4] if len(b) > 4 else 0.1]
            else:  # harmonic: k in K/A^2 -> atomic, l0
                bk.append(abi.BONDED_HARMONIC)
                bp += [KBOLTZ * b[3], b[4]]
        d["nbonds"] = len(self.bonds)
        d["bond_atoms"] = np.asarray(ba, dtype=np.int32)
        d["bond_kind"] = np.asarray(bk, dtype=np.int32)
        d["bond_param"] = np.asarray(bp, dtype=np.float64)
        aa, ak, ap = [], [], []
        for a in self.angles:
            aa += [a[0], a[1], a[2]]
            if a[3].lower() == "fixed":
                ak.append(abi.BONDED_FIXED)
                ap += [a[4], a[5] if len(a) > 5 else 1.0]
            else:
                ak.append(abi.BONDED_HARMONIC)
                ap += [KBOLTZ * a[4], (PI / 180.0) * a[5]]
        d["nangles"] = len(self.angles)
        d["angle_atoms"] = np.asarray(aa, dtype=np.int32)
        d["angle_kind"] = np.asarray(ak, dtype=np.int32)
        d["angle_param"] = np.asarray(ap, dtype=np.float64)
        da, rb = [], []
        for dh in self.dihedrals:
            if dh[4].upper() != "OPLS":
                raise ValueError("only OPLS dihedrals are supported")
            p = [KJMOL_TO_ATOMIC * v for v in dh[5:9]]
            if all(abs(v) < 1e-7 for v in p):
                continue
            da += list(dh[0:4])
            # input_routines.f90:2100-2106
            rb += [p[2] + sum(p), p[1] - 3.0 * p[3], -2.0 * p[2], 4.0 * p[3], 0.0, 0.0]
        d["ndihedrals"] = len(da) // 4
        d["dihedral_atoms"] = np.asarray(da, dtype=np.int32)
        d["dihedral_rb"] = np.asarray(rb, dtype=np.float64)
        ia, ip = [], []
        for im in self.impropers:
            ia += list(im[0:4])
            ip += [KBOLTZ * im[5], (PI / 180.0) * im[6]]
        d["nimpropers"] = len(self.impropers)
        d["improper_atoms"] = np.asarray(ia, dtype=np.int32)
        d["improper_param"] = np.asarray(ip, dtype=np.float64)
        nf = len(self.fragments)
        d["nfragments"] = nf
        d["frag_natoms"] = np.asarray([len(f) for f in self.fragments], dtype=np.int32)
        d["frag_atoms"] = np.asarray([a for f in self.fragments for a in f], dtype=np.int32)
        conn = [[] for _ in range(nf)]
        for f1, f2 in self.frag_connect:
            conn[f1 - 1].append(f2)
            conn[f2 - 1].append(f1)
        d["frag_nconnect"] = np.asarray([len(c) for c in conn], dtype=np.int32)
        d["frag_connect"] = np.asarray([x for c in conn for x in c], dtype=np.int32)
        libs = list(self.libraries) + [np.zeros((0, len(f), 3)) for f in self.fragments[len(self.libraries):]]
        d["frag_nconfig"] = np.asarray([len(lib) for lib in libs], dtype=np.int32)
        d["frag_library"] = (np.concatenate([np.asarray(l, dtype=np.float64).ravel() for l in libs])
                             if libs else np.zeros(0))
        d["l_coul_cbmc"] = int(self.l_coul_cbmc)
        return d


@dataclass
class BoxSpec:
    length: tuple
    vdw_style: int = abi.VDW_LJ
    vdw_sum_style: int = abi.VDW_SUM_CUT_TAIL
    rcut_vdw: float = 14.0
    rcut_coul: float = 0.0
    rcut_cbmc: float = 6.5
    rcut_low: float = 1.0
    ron_switch: float = 0.0
    roff_switch: float = 0.0
    charge_style: int = abi.CHARGE_NONE
    charge_sum_style: int = abi.QQ_EWALD
    ewald_tol: float = 1e-5
    alpha_dsf: float = 0.0
    temperature: float = 300.0

    @property
    def volume(self) -> float:
        return float(np.prod(self.length))


class ForceField:
    """Atom types and mixed vdw tables (create_nonbond_table.f90)."""

    def __init__(self, species: list, mixing: str = "LB", style: int = abi.VDW_LJ):
        names: list = []
        params: dict = {}
        for sp in species:
            idx = []
            for a in sp.atoms:
                if not a.vdw or a.vdw[0].upper() == "NONE":
                    idx.append(0)  # vdw_type NONE has atom_type_number 0
                    continue
                key = a.name
                if key not in params:
                    names.append(key)
                    params[key] = a.vdw
                idx.append(names.index(key) + 1)
            sp.type_index = idx
        nt = len(names)
        eps = np.zeros((nt, nt))
        sig = np.zeros((nt, nt))
        mn = np.zeros((nt, nt))
        mm = np.zeros((nt, nt))
        tiny = 1e-7
        for i, k in enumerate(names):
            v = params[k]
            if v:
                e = KBOLTZ * v[1]
                eps[i, i] = 0.0 if v[1] <= tiny else e
                sig[i, i] = 0.0 if v[2] <= tiny else v[2]
                if v[0].upper() == "MIE":
                    mn[i, i], mm[i, i] = v[3], v[4]
        for i in range(nt):
            for j in range(i + 1, nt):
                ei, ej = eps[i, i], eps[j, j]
                eps[i, j] = 0.0 if (ei <= tiny or ej <= tiny) else math.sqrt(ei * ej)
                si, sj = sig[i, i], sig[j, j]
                if si <= tiny or sj <= tiny:
                    sig[i, j] = 0.0
                elif mixing == "LB":
                    sig[i, j] = (si + sj) * 0.5
                else:
                    sig[i, j] = math.sqrt(si * sj)
                if style == abi.VDW_MIE:
                    if mn[i, i] != mn[j, j] or mm[i, i] != mm[j, j]:
                        raise ValueError("Mie mixing needs equal exponents (create_nonbond_table.f90:430)")
                    mn[i, j], mm[i, j] = mn[i, i], mm[i, i]
                eps[j, i], sig[j, i], mn[j, i], mm[j, i] = eps[i, j], sig[i, j], mn[i, j], mm[i, j]
        self.names = names
        self.ntypes = nt
        self.eps, self.sig, self.mie_n, self.mie_m = eps, sig, mn, mm


@dataclass
class MoleculeSet:
    """Molecules placed in boxes: parallel lists of locate, species, box and coordinates."""
    im: list = field(default_factory=list)
    is_: list = field(default_factory=list)
    ibox: list = field(default_factory=list)
    xyz: list = field(default_factory=list)

    def add(self, im: int, is_: int, ibox: int, xyz) -> None:
        self.im.append(im)
        self.is_.append(is_)
        self.ibox.append(ibox)
        self.xyz.append(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))

    def flat_xyz(self) -> np.ndarray:
        return np.concatenate([x.ravel() for x in self.xyz]) if self.xyz else np.zeros(0)


@dataclass
class System:
    species: list
    boxes: list
    molecules: MoleculeSet
    ff: ForceField
    max_molecules: list

    def load(self, ctx: abi.Context) -> abi.Context:
        ctx.set_nonbond_table(self.ff.eps, self.ff.sig, self.ff.mie_n, self.ff.mie_m)
        for k, sp in enumerate(self.species):
            ctx.set_species(k + 1, sp)
        for k, bx in enumerate(self.boxes):
            ctx.set_box(k + 1, bx)
        m = self.molecules
        if m.im:
            ctx.set_molecules(m.im, m.is_, m.ibox, m.flat_xyz())
        return ctx

    def open(self, fns: dict, precision: int = abi.PREC_FP64, device: int = 0,
             max_kvectors: int = 100000) -> abi.Context:
        ctx = abi.Context(fns, len(self.species), self.ff.ntypes, len(self.boxes), self.max_molecules,
                          precision=precision, device=device, max_kvectors=max_kvectors)
        return self.load(ctx)
