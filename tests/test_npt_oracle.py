"""Volume moves of the oracle (move_volume.f90) and the NPT harness on it:
the rebuilt energy of a scaled box against a fresh context loaded with the
scaled coordinates, restore to the exact previous state, and NPT chains that
keep their running energy equal to a recomputation."""
import numpy as np

from cassandra_gb300 import npt, workloads
from oracle import oracle


def test_volume_scale_and_restore():
    s = workloads.water_nvt_system(nboxes=1)
    L = s.boxes[0].length[0]
    with oracle.open_system(s) as o:
        e0, _ = o.system_total_energy(1)
        x0 = np.concatenate([o.get_molecule(im, is_).ravel() for im, is_ in zip(s.molecules.im, s.molecules.is_)])
        e1, ov = o.volume_scale(1, L * 1.02)
        assert not ov
        x1 = np.concatenate([o.get_molecule(im, is_).ravel() for im, is_ in zip(s.molecules.im, s.molecules.is_)])
        # rigid molecules: intramolecular distances kept, COMs scaled
        d0 = (x0.reshape(-1, 3, 3)[:, 1] - x0.reshape(-1, 3, 3)[:, 0])
        d1 = (x1.reshape(-1, 3, 3)[:, 1] - x1.reshape(-1, 3, 3)[:, 0])
        assert np.allclose(d0, d1, atol=1e-12)
        assert abs(e1["total"] - e0["total"]) > 1e-6 * abs(e0["total"])
        o.volume_restore(1)
        e2, _ = o.system_total_energy(1)
        x2 = np.concatenate([o.get_molecule(im, is_).ravel() for im, is_ in zip(s.molecules.im, s.molecules.is_)])
        assert np.array_equal(x0, x2)
        assert abs(e2["total"] - e0["total"]) <= 1e-10 * abs(e0["total"])
    # the scaled energy equals that of a fresh context built at the new edge
    s2 = workloads.water_nvt_system(nboxes=1)
    s2.boxes[0].length = (L * 1.02,) * 3
    with oracle.open_system(s2) as o2:
        o2.set_molecules(s.molecules.im, s.molecules.is_, s.molecules.ibox, x1)
        e3, _ = o2.system_total_energy(1)
    for k in ("total", "inter_vdw", "inter_q", "reciprocal", "lrc", "self"):
        assert abs(e3[k] - e1[k]) <= 1e-10 * (abs(e1[k]) + 1.0), k


def test_npt_chain_bookkeeping():
    s = workloads.lj_nvt_system(nboxes=1, n=100, length=35.0 * (100 / 500) ** (1 / 3), rcut=10.0, seed=3)
    with oracle.open_system(s) as o:
        ch = npt.NPTChains(o, [1], [100], 150.0, 50.0, 300.0, [[0.8]], [[0.0]], seed=5)
        ch.start([s.boxes[0].length[0]])
        for _ in range(6):
            ch.sweeps(1)
            ch.volume_moves()
        assert ch.n_vol_acc[0] > 0
        e, _ = o.system_total_energy(1)
        assert abs(e["total"] - ch.energy[0]) <= 1e-9 * abs(e["total"])
