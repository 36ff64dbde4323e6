"""The CPU oracle's NVT translate / rotate sweeps (move_translate.f90,
move_rotate.f90): energy bookkeeping, determinism, independence of boxes and
the step-size adaptation."""
import numpy as np

import mc_helpers
from oracle import oracle


def _run(system, boxes, nsweeps, seed, prob_translate=1.0, nupdate=0, max_rot=0.0):
    with oracle.open_system(system) as o:
        for b in boxes:
            o.system_total_energy(b)
        ns = len(system.species)
        res, md, mr = o.mc_sweeps(boxes, nsweeps, [[0.8] * ns] * len(boxes), [[max_rot] * ns] * len(boxes),
                                  seed=seed, prob_translate=prob_translate, nupdate=nupdate)
        return res, md, mr, mc_helpers.positions(o, system)


def test_lj_bookkeeping_matches_recomputed_energy():
    s = mc_helpers.lj_small()
    res, md, mr, xyz = _run(s, [1, 2], 5, seed=7)
    again = mc_helpers.recomputed_totals(oracle.fns(), s, xyz, [1, 2])
    for r, e in zip(res, again):
        assert r["n_translate"] == 1000
        assert 0 < r["n_translate_accepted"] < r["n_translate"]
        assert abs(r["energy"]["total"] - e["total"]) <= 1e-9 * abs(e["inter_vdw"]) + 1e-6
        assert abs(r["energy"]["inter_vdw"] - e["inter_vdw"]) <= 1e-9 * abs(e["inter_vdw"]) + 1e-6


def test_water_bookkeeping_with_ewald_and_rotation():
    s = mc_helpers.water_small()
    res, md, mr, xyz = _run(s, [1], 3, seed=11, prob_translate=0.5, max_rot=0.4)
    (e,) = mc_helpers.recomputed_totals(oracle.fns(), s, xyz, [1])
    r = res[0]
    assert r["n_translate"] + r["n_rotate"] == 3 * 64
    assert r["n_rotate_accepted"] > 0 and r["n_translate_accepted"] > 0
    for k in ("total", "inter_q", "reciprocal", "inter_vdw"):
        assert abs(r["energy"][k] - e[k]) <= 1e-9 * abs(e["inter_q"]) + 1e-6, k


def test_deterministic_and_boxes_independent():
    s = mc_helpers.lj_small()
    a = _run(s, [1, 2], 2, seed=3)
    b = _run(s, [1, 2], 2, seed=3)
    c = _run(s, [2], 2, seed=3)
    assert a[0] == b[0]
    assert np.array_equal(a[3], b[3])
    assert a[0][1] == c[0][0]


def test_step_adaptation():
    s = mc_helpers.lj_small(nboxes=1)
    res, md, mr, _ = _run(s, [1], 2, seed=5, nupdate=50)
    # 400 trials, 8 updates: max_disp = min(rcut, 2 * ratio * max_disp) each time
    assert md[0, 0] != 0.8 and 0.0 < md[0, 0] <= 12.0
