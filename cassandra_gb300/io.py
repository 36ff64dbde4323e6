"""Readers for the subset of Cassandra input formats the hot path needs.

read_mcf follows the section layout parsed by input_routines.f90 (Atom_Info,
Bond_Info, Angle_Info, Dihedral_Info, Improper_Info, Intra_Scaling,
Fragment_Info, Fragment_Connectivity); units are converted later, in
cassandra_gb300.system.  read_frag_library reads a fragment library .dat as
written by Cassandra's fragment runs (coordinates per conformation).
write_xyz_frame / write_H_frame write the two files of a pregenerated
trajectory in the layout Load_Next_Frame reads (load_next_frame.f90:184-228,
307-328); the trajectory itself is read by the library (cass_traj_open).
"""
from __future__ import annotations

import numpy as np

from .system import Atom, Species


def _sections(text: str) -> dict:
    out: dict = {}
    cur = None
    for raw in text.splitlines():
        line = raw.split("!")[0].strip()
        if not line:
            continue
        if line.startswith("#"):
            cur = line[1:].strip().split()[0]
            out[cur] = []
        elif line.upper() == "END":
            cur = None
        elif cur is not None:
            out[cur].append(line.split())
    return out


def read_mcf(text: str) -> Species:
    sec = _sections(text)
    atoms = []
    for row in sec["Atom_Info"][1:1 + int(sec["Atom_Info"][0][0])]:
        name, mass, q, style = row[1], float(row[3]), float(row[4]), row[5].upper()
        if style == "LJ":
            vdw = ("LJ", float(row[6]), float(row[7]))
        elif style == "MIE":
            vdw = ("Mie", float(row[6]), float(row[7]), float(row[8]), float(row[9]))
        else:
            vdw = ()
        atoms.append(Atom(name=name, mass=mass, charge=q, vdw=vdw))
    bonds = []
    for row in sec.get("Bond_Info", [["0"]])[1:]:
        a1, a2, kind = int(row[1]), int(row[2]), row[3].lower()
        if kind == "fixed":
            bonds.append((a1, a2, "fixed", float(row[4]), float(row[5]) if len(row) > 5 else 0.1))
        else:
            bonds.append((a1, a2, "harmonic", float(row[4]), float(row[5])))
    angles = []
    for row in sec.get("Angle_Info", [["0"]])[1:]:
        a = (int(row[1]), int(row[2]), int(row[3]))
        if row[4].lower() == "fixed":
            angles.append(a + ("fixed", float(row[5]), float(row[6]) if len(row) > 6 else 1.0))
        else:
            angles.append(a + ("harmonic", float(row[5]), float(row[6])))
    dihedrals = []
    for row in sec.get("Dihedral_Info", [["0"]])[1:]:
        a = (int(row[1]), int(row[2]), int(row[3]), int(row[4]))
        if row[5].upper() == "OPLS":
            dihedrals.append(a + ("OPLS",) + tuple(float(v) for v in row[6:10]))
        elif row[5].upper() != "NONE":
            raise ValueError(f"dihedral style {row[5]} not supported")
    impropers = []
    for row in sec.get("Improper_Info", [["0"]])[1:]:
        if row[5].lower() == "harmonic":
            impropers.append((int(row[1]), int(row[2]), int(row[3]), int(row[4]), "harmonic",
                              float(row[6]), float(row[7])))
    scale = sec.get("Intra_Scaling", [])
    sv = tuple(float(v) for v in scale[0][:4]) if scale else (0.0, 0.0, 0.5, 1.0)
    sq = tuple(float(v) for v in scale[1][:4]) if len(scale) > 1 else sv
    frags = []
    for row in sec.get("Fragment_Info", [["0"]])[1:]:
        n = int(row[1])
        frags.append([int(v) for v in row[2:2 + n]])
    conn = [(int(r[1]), int(r[2])) for r in sec.get("Fragment_Connectivity", [["0"]])[1:]]
    return Species(atoms=atoms, bonds=bonds, angles=angles, dihedrals=dihedrals, impropers=impropers,
                   scale_vdw=sv, scale_qq=sq, fragments=frags, frag_connect=conn)


def read_frag_library(text: str, natoms: int) -> np.ndarray:
    """Fragment library: repeated blocks of `natoms` lines 'element x y z'
    (optionally preceded by an atom-count line and a comment line)."""
    rows = []
    for raw in text.splitlines():
        parts = raw.split()
        if len(parts) >= 4:
            try:
                rows.append([float(parts[1]), float(parts[2]), float(parts[3])])
            except ValueError:
                continue
    arr = np.asarray(rows, dtype=np.float64)
    return arr.reshape(-1, natoms, 3)


def write_xyz_frame(f, xyz, elements, step: int = 0) -> None:
    """One .xyz frame: the atom count, a comment record, 'element x y z' per atom
    (17 significant digits, so that a read gives back the same doubles)."""
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    f.write(f"{len(xyz):12d}\n MC_STEP: {step:12d}\n")
    for e, (x, y, z) in zip(elements, xyz):
        f.write(f"{e:<4s}{x:26.17e}{y:26.17e}{z:26.17e}\n")


def write_H_frame(f, box, nmols) -> None:
    """One .H frame: the volume, the three rows of the box matrix, a blank record,
    the number of species and one 'species nmols' record each."""
    b = np.asarray(box, dtype=np.float64)
    m = np.diag(b) if b.shape == (3,) else b.reshape(3, 3)
    f.write(f"{abs(np.linalg.det(m)):26.17e}\n")
    for r in m:
        f.write("".join(f"{v:26.17e}" for v in r) + "\n")
    f.write("\n")
    f.write(f"{len(nmols):12d}\n")
    for k, n in enumerate(nmols):
        f.write(f"{k + 1:12d}{int(n):12d}\n")
