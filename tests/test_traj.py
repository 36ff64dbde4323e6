"""The library's pregenerated-trajectory reader (cass_traj_open / cass_traj_next,
the Read_H_frame and Read_xyz_frame steps of load_next_frame.f90:184-228,
307-328), on the host: the reference's own trajectory text (water_spce and
pentane Widom examples) must give the coordinates and boxes that the fixture
arrays hold, bit for bit; the package's writers must round-trip; malformed
records fail with their line number.  No GPU is needed: only files are read."""
import os

import numpy as np
import pytest

import cassandra_gb300 as cg
import helpers
from cassandra_gb300 import abi, build, io

NATOMS = {"water_spce": 3, "pentane": 5}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def _write(tmp_path, name, text):
    p = os.path.join(tmp_path, name)
    with open(p, "w") as f:
        f.write(text)
    return p


@pytest.mark.parametrize("name", ["water_spce", "pentane"])
def test_reader_matches_reference_text(tmp_path, name):
    raw = helpers.golden("traj_text.npz")
    ref = helpers.golden(f"pregen_{name}.npz")
    xp = _write(tmp_path, "t.xyz", str(raw[f"{name}_xyz"]))
    hp = _write(tmp_path, "t.H", str(raw[f"{name}_H"]))
    nfr = int(raw[f"{name}_nframes_xyz"])
    with cg.open_trajectory(xp, hp, [NATOMS[name]]) as t:
        for k in range(nfr):
            fr = t.next()
            assert fr is not None and fr["index"] == k
            assert np.array_equal(fr["xyz"], ref["frames"][k])
            assert np.array_equal(np.diag(fr["box"]), ref["boxes"][k])
            assert fr["box"][0, 1] == 0.0 and fr["box"][2, 0] == 0.0
            assert fr["nmols"][0] * NATOMS[name] == len(ref["frames"][k])
        # the .H file goes on, the .xyz file ends: the end of the run (load_next_frame.f90:311-315)
        assert t.next() is None
        assert t.next() is None
        assert t.stats()["frames"] == nfr




def test_writer_round_trip_and_prefetch_order(tmp_path):
    rng = np.random.default_rng(3)
    frames, boxes, nmols = [], [], []
    for k in range(25):  # more frames than buffers: the reader runs ahead and waits
        n1, n2 = int(rng.integers(0, 7)), int(rng.integers(0, 5))
        frames.append(rng.normal(scale=30.0, size=(3 * n1 + 2 * n2, 3)))
        boxes.append(rng.uniform(20.0, 40.0, size=3))
        nmols.append([n1, n2])
    xp, hp = os.path.join(tmp_path, "w.xyz"), os.path.join(tmp_path, "w.H")
    with open(xp, "w") as fx, open(hp, "w") as fh:
        for k in range(25):
            io.write_xyz_frame(fx, frames[k], ["X"] * len(frames[k]), k)
            io.write_H_frame(fh, boxes[k], nmols[k])
    with cg.open_trajectory(xp, hp, [3, 2]) as t:
        for k in range(25):
            fr = t.next()
            assert fr["index"] == k
            assert np.array_equal(fr["xyz"], frames[k])
            assert np.array_equal(np.diag(fr["box"]), boxes[k])
            assert list(fr["nmols"]) == nmols[k]
        assert t.next() is None


def test_H_lists_a_subset_of_species(tmp_path):
    xp = _write(tmp_path, "a.xyz", "2\ncomment\nC 1.0 2.0 3.0\nC 4.0 5.0 6.0D0\n")
    hp = _write(tmp_path, "a.H", " 1000.0\n 10.0 0.0 0.0\n 0.0 10.0 0.0\n 0.0 0.0 10.0\n\n 1\n 2 1\n")
    with cg.open_trajectory(xp, hp, [3, 2]) as t:
        fr = t.next()
        assert list(fr["nmols"]) == [0, 1]
        assert np.array_equal(fr["xyz"], [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])  # D exponent read as E


def test_fixed_counts_without_H(tmp_path):
    x = np.arange(18, dtype=np.float64).reshape(6, 3) * 0.5
    xp = os.path.join(tmp_path, "f.xyz")
    with open(xp, "w") as f:
        for k in range(3):
            io.write_xyz_frame(f, x + k, ["O", "H", "H"] * 2, k)
    with cg.open_trajectory(xp, None, [3], nmols=[2], box=[15.0, 16.0, 17.0]) as t:
        for k in range(3):
            fr = t.next()
            assert np.array_equal(fr["xyz"], x + k)
            assert np.array_equal(fr["box"], np.diag([15.0, 16.0, 17.0]))
        assert t.next() is None


def test_truncated_frame_fails_with_line(tmp_path):
    xp = _write(tmp_path, "b.xyz", "3\nc\nO 0 0 0\nH 1 0 0\n")
    with cg.open_trajectory(xp, None, [3], nmols=[1], box=[10.0, 10.0, 10.0]) as t:
        with pytest.raises(abi.CassError, match="frame ends early"):
            t.next()


def test_bad_records_fail(tmp_path):
    xp = _write(tmp_path, "c.xyz", "1\nc\nO 0 0 zero\n")
    with cg.open_trajectory(xp, None, [1], nmols=[1], box=[10.0, 10.0, 10.0]) as t:
        with pytest.raises(abi.CassError, match="bad coordinate at line 3"):
            t.next()
    hp = _write(tmp_path, "c.H", " 1.0\n 1 0 0\n 0 1 0\n 0 0 1\n\n 1\n 3 5\n")
    xp = _write(tmp_path, "d.xyz", "0\nc\n")
    with cg.open_trajectory(xp, hp, [1, 1]) as t:
        with pytest.raises(abi.CassError, match="species / molecule-count record at line 7"):
            t.next()
    with pytest.raises(abi.CassError, match="cannot open"):
        cg.open_trajectory(os.path.join(tmp_path, "missing.xyz"), None, [1], nmols=[1], box=[1.0, 1.0, 1.0])
