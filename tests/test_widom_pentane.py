"""The reference's pentane Widom fixture (pregen run of 11 trajectory frames,
60 united-atom pentanes in a 100 A box at 336 K) rerun with its own input
options -- kappa_ins = kappa_dih = 4, the CBMC atom-pair energy table with 1000
bins, Cell_List_Overlap and adaptive r_min with U_max = 300 kT -- against the
reference's output: the per-frame averages of widom_var (.spec1.wprp, 90,000
insertions each) and the shifted chemical potential of the log (-39.0826
kJ/mol).  Both sides are Monte Carlo estimates, so the comparison is
statistical: the spread of one insertion's widom_var, measured here, gives the
standard error of both averages."""
import math

import numpy as np

import helpers
from oracle import oracle

KBOLTZ = 0.8314472
N_REF = 90000
OPTIONS = {"energy_table_res": 1000, "sector_overlap": True, "rmin_u_max": 300.0}


def run_frames(open_ctx, n_ins, frames, seed, options=OPTIONS):
    out = []
    for f in frames:
        s = helpers.pentane_widom_system(f)
        lam3 = helpers.de_broglie(s) ** 3
        with open_ctx(s) as o:
            o.system_total_energy(1)
            if options:
                o.set_cbmc_options(**options)
            r, tr = o.widom_insert(1, [1], n_ins, 4, 4, seed=seed + f, trace=True)
        w = tr["widom_var"].ravel()
        out.append((r[0]["widom_sum"] / lam3, r[0]["n_insertions"], float(w.std() / w.mean()), r[0]["n_overlaps"]))
    return out


def check_against_reference(res, frames, n_ins):
    d = helpers.golden("widom_pentane.npz")
    zs = []
    for (wsum, n, spread, _), f in zip(res, frames):
        ours, ref = wsum / n, d["widom_var_mean"][f]
        sigma = ref * spread * math.sqrt(1.0 / n_ins + 1.0 / N_REF)
        zs.append((ours - ref) / sigma)
    zs = np.array(zs)
    assert np.all(np.abs(zs) < 4.5), zs
    assert np.mean(zs ** 2) < 3.0, zs
    T = 336.0
    tot = sum(r[0] for r in res) / sum(r[1] for r in res)
    mu = -KBOLTZ * T * 0.01 * math.log(tot)
    ref_tot = np.mean(d["widom_var_mean"][list(frames)])
    spread = np.mean([r[2] for r in res])
    sig_mu = KBOLTZ * T * 0.01 * spread * math.sqrt(1.0 / (n_ins * len(frames)) + 1.0 / (N_REF * len(frames)))
    assert abs(mu - (-KBOLTZ * T * 0.01 * math.log(ref_tot))) < 4.5 * sig_mu
    if len(frames) == 11:  # the log's value is over all frames
        assert abs(mu - float(d["mu_prime_kjmol"])) < 4.5 * sig_mu, (mu, float(d["mu_prime_kjmol"]), sig_mu)
    return zs


def test_oracle_pentane_widom_statistics():
    frames = range(11)
    res = run_frames(oracle.open_system, 20000, frames, seed=100)
    check_against_reference(res, frames, 20000)
    assert all(r[3] == 0 for r in res)  # the reference logged no overlapping insertion


def test_options_change_trials_only_slightly():
    # the table and the r_min overlap change trial energies, not the estimator:
    # with and without them the same seeds give averages within statistical noise
    frames = [0, 5]
    a = run_frames(oracle.open_system, 4000, frames, seed=7, options=None)
    b = run_frames(oracle.open_system, 4000, frames, seed=7)
    for (wa, n, sp, _), (wb, _, _, _) in zip(a, b):
        assert abs(wa / wb - 1.0) < 4.0 * sp / math.sqrt(n)
