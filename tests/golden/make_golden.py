"""Extract golden vectors from the reference's own test suite into small fixtures.

Usage: python tests/golden/make_golden.py <path of the Cassandra source tree>
(or set CASSANDRA_REFERENCE to that path).  The fixtures it writes travel with
the repository so that the tests can run where the reference is absent.  Everything is read as text or data: no
reference code is executed.

Sources (paths inside the Cassandra tree):
  Scripts/testSuite/Test6_NIST_LennardJonesEnergy.py + Resources/testConfigurations/nist{1..4}.xyz
  Scripts/testSuite/Test7_Water.py + Resources/inputFiles/test7.water{1..4}.xyz
  Scripts/testSuite/Resources/exampleResources/Widom/{pentane,water_spce}/  (trajectories, .mcf, .inp)
  Scripts/testSuite/Resources/exampleResults/Widom/{pentane,water_spce}/*.prp  (per-frame Energy_Total)
  Scripts/testSuite/Resources/exampleResults/Widom/pentane/*.wprp, *.wprp2, *.log  (Widom statistics)
  Scripts/testSuite/Resources/exampleResources/Widom/pentane/species1/frag*/frag*.dat  (fragment libraries)
  Scripts/testSuite/Resources/exampleResources/Widom/{water_spce,pentane}/*_traj.{xyz,H}  (raw text, reader pin)
"""
from __future__ import annotations

import ast
import json
import os
import re
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CASSANDRA_REFERENCE", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_golden.py <Cassandra source tree>  (or set CASSANDRA_REFERENCE)")
TS = os.path.join(REF, "Scripts", "testSuite")
OUT = os.path.dirname(os.path.abspath(__file__))


def read_xyz(path):
    with open(path) as f:
        lines = f.read().split("\n")
    n = int(lines[0].split()[0])
    xyz = np.array([[float(v) for v in ln.split()[1:4]] for ln in lines[2:2 + n]])
    return xyz


def _arith(node):
    """Evaluate a literal made of numbers, tuples and +/- only."""
    if isinstance(node, ast.Expression):
        return _arith(node.body)
    if isinstance(node, ast.Tuple):
        return tuple(_arith(e) for e in node.elts)
    if isinstance(node, ast.Constant):
        return node.value
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        return -_arith(node.operand)
    if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub)):
        a, b = _arith(node.left), _arith(node.right)
        return a + b if isinstance(node.op, ast.Add) else a - b
    raise ValueError("unsupported literal")


def literal(src, pattern):
    m = re.search(pattern, src, re.S)
    return _arith(ast.parse(m.group(1), mode="eval"))


def nist_lj():
    src = open(os.path.join(TS, "Test6_NIST_LennardJonesEnergy.py")).read()
    answers = [literal(src, r"analyticAnswer\[%d\] = (\(.*?\))" % i) for i in range(8)]
    box = literal(src, r"box = (\(.*?\))")
    vdw = literal(src, r"vdwStyle = (\(.*?\))")
    files = ["nist1.xyz", "nist3.xyz", "nist2.xyz", "nist4.xyz"] * 2
    vdw_atom = literal(src, r"atomParms\[s\]\[a\]\['vdw'\] = (\(.*?\))")
    data = {}
    for k in range(4):
        data[f"xyz{k}"] = read_xyz(os.path.join(TS, "Resources", "testConfigurations", files[k]))
    checks = np.array([[k % 4, box[k], float(vdw[k].split()[-1]), *answers[k]] for k in range(8)])
    data["checks"] = checks  # file index, box, rcut, total, inter vdw, lrc (kJ/mol)
    data["eps_K"] = float(vdw_atom[1])
    data["sigma"] = float(vdw_atom[2])
    np.savez_compressed(os.path.join(OUT, "nist_lj.npz"), **data)


def nist_spce():
    src = open(os.path.join(TS, "Test7_Water.py")).read()
    nist = literal(src, r"nistAnswer = (\(\(.*?\)\))\n")
    atom = literal(src, r"atomParms = (\(\(\(.*?\)\),\))")
    nmols = literal(src, r"nMols = (\(.*?\))")
    box = literal(src, r"box = (\(.*?\))")
    charge = literal(src, r"chargeStyle = (\(.*?\))")
    tol = literal(src, r"errorTol = (\(.*?\))")
    kb = 1.3806488 * 6.02214129 / 1000
    data = {}
    for k in range(4):
        data[f"xyz{k}"] = read_xyz(os.path.join(TS, "Resources", "inputFiles", f"test7.water{k + 1}.xyz"))
    rows = []
    for k in range(4):
        parts = charge[k].split()
        rows.append([nmols[k], box[k], float(parts[2]), float(parts[3]), *[v * kb for v in nist[k]]])
    data["checks"] = np.array(rows)  # nmol, box, rcut, tol, intervdw, lrc, interq, recip, self, total (kJ/mol)
    data["tolerances"] = np.array(tol)
    data["atoms"] = json.dumps(atom)
    np.savez_compressed(os.path.join(OUT, "nist_spce.npz"), **data)


def read_traj(xyz_path, h_path, nframes):
    with open(xyz_path) as f:
        lines = f.read().split("\n")
    frames, pos = [], 0
    for _ in range(nframes):
        n = int(lines[pos].split()[0])
        frames.append(np.array([[float(v) for v in ln.split()[1:4]] for ln in lines[pos + 2:pos + 2 + n]]))
        pos += 2 + n
    with open(h_path) as f:
        hl = [ln for ln in f.read().split("\n")]
    boxes, pos = [], 0
    for _ in range(nframes):
        while not hl[pos].strip():
            pos += 1
        pos += 1  # volume
        m = np.array([[float(v) for v in hl[pos + r].split()] for r in range(3)])
        boxes.append(np.diag(m).copy())
        pos += 3
        while not hl[pos].strip():
            pos += 1
        nsp = int(hl[pos].split()[0])
        pos += 1 + nsp
    return np.array(frames), np.array(boxes)


def read_prp(path):
    rows = []
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        rows.append([float(v) for v in ln.split()])
    return np.array(rows)


def pregen(name, traj, prp, mcf, inp):
    base = os.path.join(TS, "Resources", "exampleResources", "Widom", name)
    res = os.path.join(TS, "Resources", "exampleResults", "Widom", name)
    e = read_prp(os.path.join(res, prp))
    frames, boxes = read_traj(os.path.join(base, traj + ".xyz"), os.path.join(base, traj + ".H"), len(e))
    data = {"frames": frames, "boxes": boxes, "energy_total_kjmol": e[:, 1],
            "mcf": open(os.path.join(base, mcf)).read(), "inp": open(os.path.join(base, inp)).read()}
    np.savez_compressed(os.path.join(OUT, f"pregen_{name}.npz"), **data)


def widom_pentane():
    """The pentane Widom fixture's statistics: per-frame averages of widom_var
    (.spec1.wprp), the three sub-interval averages per frame (.spec1.wprp2),
    the shifted chemical potential of the log, and the fragment libraries the
    run used (species1/frag*/frag*.dat, as arrays)."""
    base = os.path.join(TS, "Resources", "exampleResources", "Widom", "pentane")
    res = os.path.join(TS, "Resources", "exampleResults", "Widom", "pentane")
    wprp = np.loadtxt(os.path.join(res, "pentane_widom.out.spec1.wprp"), skiprows=1)
    wprp2 = np.loadtxt(os.path.join(res, "pentane_widom.out.spec1.wprp2"))
    log = open(os.path.join(res, "pentane_widom.out.log")).read()
    mu = float(re.search(r"Shifted chemical potential for species 1 in box 1 is\s+([-0-9.Ee+]+)", log).group(1))
    data = {"widom_var_mean": wprp[:, 1], "widom_var_sub": wprp2, "n_overlaps": wprp[:, 3], "mu_prime_kjmol": mu}
    for f in (1, 2, 3):
        rows = []
        for ln in open(os.path.join(base, "species1", f"frag{f}", f"frag{f}.dat")):
            parts = ln.split()
            if len(parts) == 4:
                rows.append([float(v) for v in parts[1:]])
        data[f"frag{f}"] = np.array(rows).reshape(-1, 3, 3)
    np.savez_compressed(os.path.join(OUT, "widom_pentane.npz"), **data)


def traj_text():
    """Raw text of the reference's pregenerated trajectories, to pin the
    library's .xyz/.H reader: all .H records and the first .xyz frames of the
    water_spce and pentane Widom examples."""
    base = os.path.join(TS, "Resources", "exampleResources", "Widom")
    data = {}
    for name, traj, nfr in (("water_spce", "spce_traj", 3), ("pentane", "pentane_traj", 2)):
        lines = open(os.path.join(base, name, traj + ".xyz")).read().split("\n")
        pos = 0
        for _ in range(nfr):
            pos += 2 + int(lines[pos].split()[0])
        data[f"{name}_xyz"] = "\n".join(lines[:pos]) + "\n"
        data[f"{name}_H"] = open(os.path.join(base, name, traj + ".H")).read()
        data[f"{name}_nframes_xyz"] = nfr
    np.savez_compressed(os.path.join(OUT, "traj_text.npz"), **data)


if __name__ == "__main__":
    nist_lj()
    nist_spce()
    pregen("water_spce", "spce_traj", "spce_widom.out.prp", "spce.mcf", "spce_widom.inp")
    pregen("pentane", "pentane_traj", "pentane_widom.out.prp", "pentane.mcf", "pentane_widom.inp")
    widom_pentane()
    traj_text()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
