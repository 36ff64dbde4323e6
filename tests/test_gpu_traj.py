"""The trajectory feed on the GPU: cass_load_next_frame (Load_Next_Frame,
load_next_frame.f90:5-330) followed by cass_system_total_energy, frame after
frame, against the per-frame energies the reference printed for its pregen
Widom examples and against the FP64 oracle; COM folding (Apply_PBC_Anint),
molecules dropping out of a frame, box changes with their k-vectors, and the
pregen Widom loop against contexts built frame by frame."""
import math
import os

import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
from cassandra_gb300 import abi, io, pregen
from cassandra_gb300.system import Atom, BoxSpec, ForceField, MoleculeSet, Species, System
from oracle import oracle

pytestmark = pytest.mark.gpu

KJ = 0.01
ELEMENTS = {"water_spce": ["O", "H", "H"], "pentane": ["C"] * 5}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cassandra_gb300 import build
    build.build()
    oracle.build()


def _close(a, b, rel, abs_=1e-6):
    return abs(a - b) <= rel * max(abs(a), abs(b)) + abs_


def write_fixture_traj(tmp_path, name):
    d = helpers.golden(f"pregen_{name}.npz")
    na = len(ELEMENTS[name])
    xp, hp = os.path.join(tmp_path, f"{name}.xyz"), os.path.join(tmp_path, f"{name}.H")
    with open(xp, "w") as fx, open(hp, "w") as fh:
        for k, x in enumerate(d["frames"]):
            io.write_xyz_frame(fx, x, ELEMENTS[name] * (len(x) // na), k)
            io.write_H_frame(fh, d["boxes"][k], [len(x) // na])
    return xp, hp, d


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", ["water_spce", "pentane"])
def test_frames_match_reference_energies(tmp_path, name, prec):
    xp, hp, d = write_fixture_traj(tmp_path, name)
    nfr = len(d["frames"])
    with cg.open_system(helpers.pregen_system(name, 0), precision=prec) as g, \
            cg.open_trajectory(xp, hp, [len(ELEMENTS[name])]) as t:
        for f in range(nfr):
            assert not g.load_next_frame([t])
            eg, ov = g.system_total_energy(1)
            assert not ov
            with oracle.open_system(helpers.pregen_system(name, f)) as o:
                eo, _ = o.system_total_energy(1)
            if prec == abi.PREC_FP64:
                for k in eo:
                    assert _close(eg[k], eo[k], 1e-10), (f, k, eg[k], eo[k])
                want = d["energy_total_kjmol"][f]
                assert abs(eg["total"] * KJ - want) <= 5e-8 * abs(want) + 1e-4
            else:
                scale = abs(eo["inter_vdw"]) + abs(eo["inter_q"]) + abs(eo["intra"])
                assert abs(eg["total"] - eo["total"]) <= 1e-5 * scale
        assert g.load_next_frame([t])  # the end of the trajectory
        assert g.load_next_frame([t])


def _water():
    sp = Species(atoms=[Atom("O", 15.999, -0.8476, ("LJ", 78.2, 3.166)), Atom("H", 1.008, 0.4238, ()),
                        Atom("H", 1.008, 0.4238, ())],
                 bonds=[(1, 2, "fixed", 1.0), (1, 3, "fixed", 1.0)], angles=[(2, 1, 3, "fixed", 109.47)],
                 scale_vdw=(0, 0, 0, 1.0), scale_qq=(0, 0, 0, 1.0), fragments=[[1, 2, 3]])
    return sp


def _mol(c, rng):
    from cassandra_gb300.workloads import random_rotation
    b = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [math.cos(math.radians(109.47)), math.sin(math.radians(109.47)), 0.0]])
    m = np.array([15.999, 1.008, 1.008])
    b = b - (m[:, None] * b).sum(0) / m.sum()
    return b @ random_rotation(rng).T + c


def test_folding_membership_and_box_change(tmp_path):
    rng = np.random.default_rng(11)
    sp = _water()
    L0, L1 = 20.0, 21.5
    # frame 0: 6 waters, two with their COM outside the box; frame 1: 4 waters in a larger box
    c0 = [(0.0, 0.0, 0.0), (14.0, -3.0, 2.0), (-5.0, 26.5, -12.0), (4.0, 4.0, 4.0), (-7.0, 1.0, 8.0), (2.0, -8.0, -6.0)]
    c1 = [(1.0, 1.0, 1.0), (-9.0, 3.0, 0.0), (12.0, 12.0, -12.5), (-2.0, -6.0, 7.0)]
    fr = [np.concatenate([_mol(np.array(c), rng) for c in cs]) for cs in (c0, c1)]
    xp, hp = os.path.join(tmp_path, "w.xyz"), os.path.join(tmp_path, "w.H")
    with open(xp, "w") as fx, open(hp, "w") as fh:
        for k, (x, L) in enumerate(zip(fr, (L0, L1))):
            io.write_xyz_frame(fx, x, ["O", "H", "H"] * (len(x) // 3), k)
            io.write_H_frame(fh, [L] * 3, [len(x) // 3])

    def system(xyz, L):
        ms = MoleculeSet()
        for m in range(len(xyz) // 3):
            ms.add(m + 1, 1, 1, xyz[3 * m:3 * m + 3])
        bx = BoxSpec(length=(L,) * 3, rcut_vdw=9.0, rcut_coul=9.0, rcut_low=0.5, charge_style=abi.CHARGE_COUL,
                     charge_sum_style=abi.QQ_EWALD, ewald_tol=1e-5, temperature=298.0)
        return System([sp], [bx], ms, ForceField([sp]), [8])

    def folded(x, L):
        out = x.copy()
        m = np.array([15.999, 1.008, 1.008])
        for k in range(len(x) // 3):
            r = x[3 * k:3 * k + 3]
            com = (m[:, None] * r).sum(0) / m.sum()
            cn = com - L * np.round(com / L)  # ANINT: halves away from zero, as np.round is not; no halves here
            out[3 * k:3 * k + 3] = r + cn - com
        return out

    with cg.open_system(system(fr[0], L0), precision=abi.PREC_FP64) as g, \
            cg.open_trajectory(xp, hp, [3]) as t:
        for k, L in enumerate((L0, L1)):
            assert not g.load_next_frame([t])
            want = folded(fr[k], L)
            n = len(fr[k]) // 3
            for m in range(n):
                assert np.allclose(g.get_molecule(m + 1, 1), want[3 * m:3 * m + 3], rtol=0, atol=1e-12)
            boxes = g.molecule_boxes(1)
            assert list(boxes[:n]) == [1] * n and not boxes[n:].any()
            eg, _ = g.system_total_energy(1)
            with oracle.open_system(system(want, L)) as o:
                eo, _ = o.system_total_energy(1)
            for key in eo:
                assert _close(eg[key], eo[key], 1e-10), (k, key, eg[key], eo[key])
        # the folded COMs lie inside the box
        x = np.concatenate([g.get_molecule(m + 1, 1) for m in range(4)])
        assert np.all(np.abs(x.reshape(-1, 3, 3).mean(1)) < L1 / 2 + 1.0)


def test_capacity_and_species_checks(tmp_path):
    sp = _water()
    xyz = np.concatenate([_mol(np.array([3.0 * k, 0.0, 0.0]), np.random.default_rng(k)) for k in range(3)])
    xp, hp = os.path.join(tmp_path, "c.xyz"), os.path.join(tmp_path, "c.H")
    with open(xp, "w") as fx, open(hp, "w") as fh:
        io.write_xyz_frame(fx, xyz, ["O", "H", "H"] * 3, 0)
        io.write_H_frame(fh, [20.0] * 3, [3])
    ms = MoleculeSet()
    ms.add(1, 1, 1, xyz[:3])
    bx = BoxSpec(length=(20.0,) * 3, rcut_vdw=9.0, rcut_low=0.5, temperature=298.0)
    s = System([sp], [bx], ms, ForceField([sp]), [2])  # room for 2 molecules only
    with cg.open_system(s, precision=abi.PREC_FP64) as g, cg.open_trajectory(xp, hp, [3]) as t:
        with pytest.raises(abi.CassError, match="max_molecules"):
            g.load_next_frame([t])
    with cg.open_system(s, precision=abi.PREC_FP64) as g, cg.open_trajectory(xp, hp, [4]) as t:
        with pytest.raises(abi.CassError, match="atom count"):
            g.load_next_frame([t])


def test_pregen_widom_matches_frame_by_frame_contexts(tmp_path):
    xp, hp, d = write_fixture_traj(tmp_path, "pentane")
    nfr, nins = 3, 3000
    opts = {"energy_table_res": 1000, "sector_overlap": True, "rmin_u_max": 300.0}
    with cg.open_system(helpers.pentane_widom_system(0), precision=abi.PREC_FP64) as g, \
            cg.open_trajectory(xp, hp, [5]) as t:
        g.set_cbmc_options(**opts)
        recs = pregen.pregen_widom(g, [t], [1], nins, 4, 4, seed=77, max_frames=nfr, trace=True)
    assert [r["frame"] for r in recs] == list(range(nfr))
    for f, r in enumerate(recs):
        with cg.open_system(helpers.pentane_widom_system(f), precision=abi.PREC_FP64) as g:
            g.system_total_energy(1)
            g.set_cbmc_options(**opts)
            want, wtr = g.widom_insert(1, [1], nins, 4, 4, seed=77 + 1000 * f + 1, trace=True)
        got, gtr = r["widom"][1], r["trace"][1]
        assert got[0]["n_overlaps"] == want[0]["n_overlaps"]
        assert np.array_equal(gtr["selected_trial"], wtr["selected_trial"])
        assert np.allclose(gtr["widom_var"], wtr["widom_var"], rtol=1e-9, atol=0)
        assert _close(got[0]["widom_sum"], want[0]["widom_sum"], 1e-9, 0.0)
        assert _close(r["energy"][0]["total"] * KJ, d["energy_total_kjmol"][f], 5e-8, 1e-4)


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", ["water_spce", "pentane"])
def test_widom_after_frame_load_needs_no_total_energy(tmp_path, name, prec):
    """cass_load_next_frame sets up the long-range correction and the structure
    factors as Set_Frame_Coords does; Widom right after it equals Widom after a
    full cass_system_total_energy of the same frame."""
    from cassandra_gb300 import workloads
    xp, hp, d = write_fixture_traj(tmp_path, name)
    s = helpers.pregen_system(name, 0) if name == "water_spce" else helpers.pentane_widom_system(0)
    if name == "water_spce":
        s.species[0].libraries = [workloads.water_species().libraries[0] * 1.0]
    kd = 0 if name == "water_spce" else 4
    with cg.open_system(s, precision=prec) as g, cg.open_trajectory(xp, hp, [len(ELEMENTS[name])]) as t:
        for f in range(3):
            assert not g.load_next_frame([t])
            a, ta = g.widom_insert(1, [1], 400, 8, kd, seed=5 + f, trace=True)
            with pytest.raises(abi.CassError, match="system energy"):
                g.mc_sweeps([1], 1, [[0.1]], [[0.1]], seed=1)  # MC needs the full energy
            e, _ = g.system_total_energy(1)
            b, tb = g.widom_insert(1, [1], 400, 8, kd, seed=5 + f, trace=True)
            assert a[0]["n_overlaps"] == b[0]["n_overlaps"]
            assert np.array_equal(ta["selected_trial"], tb["selected_trial"])
            assert np.array_equal(ta["widom_var"], tb["widom_var"])
            assert a[0]["widom_sum"] == b[0]["widom_sum"]


def test_two_ewald_boxes_growing_kvectors(tmp_path):
    """Two Ewald boxes loaded together, the second growing by 30 % in its second
    frame (more k-vectors, so the molecule rows are resized): both boxes are ready
    for Widom after each load and match the oracle's energies."""
    import copy
    from cassandra_gb300 import workloads
    d = helpers.golden("pregen_water_spce.npz")
    base = helpers.pregen_system("water_spce", 0)
    base.species[0].libraries = [workloads.water_species().libraries[0] * 1.0]
    nmol = len(d["frames"][0]) // 3
    frames = {1: [d["frames"][0], d["frames"][1]], 2: [d["frames"][2], d["frames"][3] * 1.3]}
    boxes = {1: [d["boxes"][0], d["boxes"][1]], 2: [d["boxes"][2], d["boxes"][3] * 1.3]}
    trajs_paths = {}
    for b in (1, 2):
        xp, hp = os.path.join(tmp_path, f"b{b}.xyz"), os.path.join(tmp_path, f"b{b}.H")
        with open(xp, "w") as fx, open(hp, "w") as fh:
            for k in range(2):
                io.write_xyz_frame(fx, frames[b][k], ["O", "H", "H"] * nmol, k)
                io.write_H_frame(fh, boxes[b][k], [nmol])
        trajs_paths[b] = (xp, hp)
    s = copy.deepcopy(base)
    s.boxes = [copy.deepcopy(base.boxes[0]), copy.deepcopy(base.boxes[0])]
    s.max_molecules = [2 * nmol + 2]
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        t1 = cg.open_trajectory(*trajs_paths[1], [3])
        t2 = cg.open_trajectory(*trajs_paths[2], [3])
        for k in range(2):
            assert not g.load_next_frame([t1, t2])
            g.widom_insert(1, [1, 2], 50, 4, 0, seed=k)  # both boxes ready after the load
            for b in (1, 2):
                eg, _ = g.system_total_energy(b)
                one = helpers.pregen_system("water_spce", 0)
                one.boxes[0].length = tuple(boxes[b][k])
                one.molecules = type(one.molecules)()
                for m in range(nmol):
                    one.molecules.add(m + 1, 1, 1, frames[b][k][3 * m:3 * m + 3])
                with oracle.open_system(one) as o:
                    eo, _ = o.system_total_energy(1)
                for key in eo:
                    assert _close(eg[key], eo[key], 1e-10), (k, b, key, eg[key], eo[key])
        t1.close()
        t2.close()
