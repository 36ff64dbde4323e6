"""The CBMC atom-pair energy table (energy_table N of CBMC_Info) in the oracle
against an independent NumPy restatement of Create_Atompair_Nrg_table and
Estimate_MoleculePair_Energy (atompair_nrg_table_routines.f90:149-261,
energy_routines.f90:1528-1587): bins in r^2 from rcut_low^2 to rcut_cbmc^2,
each bin the LJ energy at its midpoint; pairs at or beyond rcut_cbmc skipped,
a pair below rcut_low an overlap."""
import numpy as np

from cassandra_gb300 import workloads
from oracle import oracle


def table_energy(system, xyz_trial, atoms, res):
    b = system.boxes[0]
    ff = system.ff
    L = np.array(b.length)
    rlow2, rc2 = b.rcut_low ** 2, b.rcut_cbmc ** 2
    step = (rc2 - rlow2) / res
    shift = rlow2 - step
    sp = system.species
    m = system.molecules
    box_xyz = np.concatenate([m.xyz[k] for k in range(len(m.im)) if m.ibox[k] == 1])
    box_t = np.concatenate([np.array(sp[m.is_[k] - 1].type_index) for k in range(len(m.im)) if m.ibox[k] == 1])
    ta = np.array(sp[1].type_index)[np.asarray(atoms) - 1]
    out, ovs = [], []
    for x in xyz_trial:
        e, ov = 0.0, False
        for a, p in enumerate(x):
            d = box_xyz - p
            d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
            rs = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2] - shift
            sel = rs < rc2 - shift
            if np.any(rs[sel] < step):
                ov = True
                break
            bins = (rs[sel] / step).astype(int)
            mp = shift + step * bins + 0.5 * step
            tj = box_t[sel] - 1
            eps = ff.eps[ta[a] - 1, tj]
            s2 = ff.sig[ta[a] - 1, tj] ** 2 / mp
            s6 = s2 ** 3
            e += float(np.sum(4.0 * eps * (s6 * s6 - s6)))
        out.append(0.0 if ov else e)
        ovs.append(ov)
    return np.array(out), np.array(ovs)


def test_oracle_energy_table_matches_numpy():
    s = workloads.widom_batch_system(nboxes=1, sizes=[600], seed=3, nconfig=20)
    rng = np.random.default_rng(1)
    L = s.boxes[0].length[0]
    atoms = [1, 2, 3]
    base = np.array([[0.0, 0.0, 0.0], [1.54, 0.0, 0.0], [2.05, 1.45, 0.0]])
    xyz = np.stack([base + rng.uniform(-L / 2, L / 2, 3) for _ in range(200)])
    for res in (1000, 37):
        with oracle.open_system(s) as o:
            o.system_total_energy(1)
            o.set_cbmc_options(energy_table_res=res)
            e, ov = o.cbmc_trial_energies(1, 2, atoms, xyz, cbmc=True)
            o.set_cbmc_options()
            e_off, ov_off = o.cbmc_trial_energies(1, 2, atoms, xyz, cbmc=True)
        ref, rov = table_energy(s, xyz, atoms, res)
        assert np.array_equal(ov, rov)
        assert ov.sum() > 0 and (~ov).sum() > 40
        ok = ~ov
        assert np.allclose(e[ok], ref[ok], rtol=1e-10, atol=1e-8 * np.abs(ref).max())
        # the table differs from the exact pair energies by the bin width
        assert not np.allclose(e[ok], e_off[ok], rtol=1e-12, atol=0)
        assert np.median(np.abs(e[ok] - e_off[ok]) / (np.abs(e_off[ok]) + 1.0)) < (0.02 if res == 1000 else 0.5)
