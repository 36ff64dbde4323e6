"""CBMC options on the GPU (cass_set_cbmc_options): the atom-pair energy table
(energy_table N), the r_min^2 overlap test of Widom growth (Cell_List_Overlap)
and adaptive r_min (Rcutoff_Low adaptive U), against the oracle and against
the reference's own pentane Widom statistics."""
import numpy as np
import pytest

import cassandra_gb300 as cg
import test_widom_pentane as pent
from cassandra_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

OPTS = {"energy_table_res": 1000, "sector_overlap": True, "rmin_u_max": 300.0}


def _butane(sizes, seed=9):
    return workloads.widom_batch_system(nboxes=len(sizes), sizes=sizes, seed=seed, nconfig=200)


def _open(ctx, nb, **opts):
    for b in range(1, nb + 1):
        ctx.system_total_energy(b)
    ctx.set_cbmc_options(**opts)
    return ctx


def test_table_trial_and_molecule_energies_match_oracle():
    s = _butane([300, 500], seed=8)
    rng = np.random.default_rng(4)
    L = s.boxes[1].length[0]
    frag = np.array([[0.0, 0.0, 0.0], [1.54, 0.0, 0.0], [-0.63, 1.40, 0.0]])
    xyz = np.array([frag + (rng.random(3) - 0.5) * L for _ in range(200)])
    m = s.molecules
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        with oracle.open_system(s) as o, cg.open_system(s, precision=prec) as g:
            for res in (1000, 64):
                _open(o, 2, energy_table_res=res)
                _open(g, 2, energy_table_res=res)
                eo, oo = o.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=True)
                eg, og = g.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=True)
                assert np.array_equal(oo, og) and (~oo).sum() > 20
                assert np.allclose(eg, eo, rtol=1e-10, atol=1e-9)
                for k in [k for k in range(len(m.im)) if m.ibox[k] == 2][:20]:
                    a = o.mol_inter_energy(m.im[k], m.is_[k], cbmc=True)
                    b = g.mol_inter_energy(m.im[k], m.is_[k], cbmc=True)
                    assert a[2] == b[2]
                    assert abs(a[0] - b[0]) <= 1e-10 * (abs(a[0]) + 1.0) and b[1] == 0.0
            # switching the table off restores the exact pair energies
            _open(o, 2)
            _open(g, 2)
            eo, _ = o.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=True)
            eg, _ = g.cbmc_trial_energies(2, 2, [2, 1, 3], xyz, cbmc=True)
            assert np.allclose(eg, eo, rtol=1e-10 if prec == abi.PREC_FP64 else 1e-4, atol=1e-6 * np.abs(eo).max())


def test_widom_fp64_with_options_matches_oracle_per_insertion():
    s = _butane([250, 600])
    with oracle.open_system(s) as o, cg.open_system(s, precision=abi.PREC_FP64) as g:
        _open(o, 2, **OPTS)
        _open(g, 2, **OPTS)
        ro, to = o.widom_insert(2, [1, 2], 512, 12, 12, seed=31, trace=True)
        rg, tg = g.widom_insert(2, [1, 2], 512, 12, 12, seed=31, trace=True)
        # without the options the same seeds give other selections: the options are in effect
        _open(o, 2)
        r0, t0 = o.widom_insert(2, [1, 2], 512, 12, 12, seed=31, trace=True)
    assert np.array_equal(to["overlap"], tg["overlap"])
    assert np.array_equal(to["selected_trial"], tg["selected_trial"])
    ok = to["overlap"] == 0
    assert ok.sum() > 0.3 * ok.size
    assert np.allclose(tg["widom_var"][ok], to["widom_var"][ok], rtol=1e-8, atol=0)
    assert np.allclose(tg["ln_pbias"][ok], to["ln_pbias"][ok], rtol=1e-10, atol=1e-10)
    assert not np.array_equal(t0["selected_trial"], to["selected_trial"])
    for a, b in zip(ro, rg):
        assert a["n_overlaps"] == b["n_overlaps"]
        assert abs(b["widom_sum"] - a["widom_sum"]) <= 1e-8 * abs(a["widom_sum"])


def test_widom_mixed_with_options_matches_fp64():
    s = _butane([300, 700], seed=21)
    with cg.open_system(s, precision=abi.PREC_FP64) as d, cg.open_system(s, precision=abi.PREC_MIXED) as m:
        _open(d, 2, **OPTS)
        _open(m, 2, **OPTS)
        rd, td = d.widom_insert(2, [1, 2], 2048, 12, 12, seed=5, trace=True)
        rm, tm = m.widom_insert(2, [1, 2], 2048, 12, 12, seed=5, trace=True)
    same = (td["overlap"] == tm["overlap"]) & (td["selected_trial"] == tm["selected_trial"])
    # FP32 r^2 can put a pair in the neighbouring table bin or across an r_min
    assert same.mean() > 0.95
    for a, b in zip(rd, rm):
        assert abs(b["widom_sum"] / a["widom_sum"] - 1.0) < 0.02


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_pentane_widom_statistics_on_gpu(prec):
    frames = range(11)
    res = pent.run_frames(lambda x: cg.open_system(x, precision=prec), 90000, frames, seed=500 + prec)
    pent.check_against_reference(res, frames, 90000)
    nov = sum(r[3] for r in res)
    if prec == abi.PREC_FP64:
        assert nov == 0  # as the reference logged
    else:  # FP32 geometry can put a trial atom across r_min
        assert nov <= 1e-5 * 90000 * len(frames), nov


def test_gcmc_fp64_with_table_matches_oracle():
    s = workloads.gcmc_system(nboxes=2, length=25.0, max_per_box=300)
    out = []
    for open_ctx in (oracle.open_system, lambda x: cg.open_system(x, precision=abi.PREC_FP64)):
        with open_ctx(s) as g:
            _open(g, 2, energy_table_res=500)
            out.append(g.gcmc([1, 2], 600, 1, [-22.0, -26.0], [[1.0], [1.0]], [[0.5], [0.5]], seed=4))
    for a, b in zip(*out):
        for k in ("n_insert_accepted", "n_delete_accepted", "n_regrow_accepted", "n_translate_accepted",
                  "n_molecules"):
            assert a[k] == b[k], (k, a[k], b[k])
        assert abs(a["energy"]["total"] - b["energy"]["total"]) <= 1e-9 * (abs(a["energy"]["inter_vdw"]) + 1.0)
