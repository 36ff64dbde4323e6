"""Device NVT sweeps (cass_mc_sweeps) against the CPU oracle's chains.

The FP64 kernel draws the same lfsr258 numbers in the same order as the
oracle, so over short runs both chains make the same decisions; energies and
coordinates then agree to FP64 summation-order differences.  The mixed kernel
(FP32 pair loop and phases, FP64 bookkeeping) follows its own chain; its
running energy must match an FP64 recomputation of its final configuration.
"""
import numpy as np
import pytest

import cassandra_gb300 as cg
import mc_helpers
from cassandra_gb300 import abi
from oracle import oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9


def _chain(open_ctx, system, boxes, nsweeps, seed, prob_translate=1.0, max_rot=0.0, nupdate=0):
    with open_ctx(system) as ctx:
        for b in boxes:
            ctx.system_total_energy(b)
        ns = len(system.species)
        res, md, mr = ctx.mc_sweeps(boxes, nsweeps, [[0.8] * ns] * len(boxes), [[max_rot] * ns] * len(boxes),
                                    seed=seed, prob_translate=prob_translate, nupdate=nupdate)
        return res, md, mr, mc_helpers.positions(ctx, system)


def _gpu(precision):
    return lambda s: cg.open_system(s, precision=precision)


@pytest.mark.parametrize("kind", ["lj", "water"])
def test_fp64_chain_matches_oracle(kind):
    if kind == "lj":
        s, boxes, kw = mc_helpers.lj_small(), [1, 2], dict(nsweeps=4, seed=9, nupdate=100)
    else:
        s, boxes, kw = mc_helpers.water_small(), [1], dict(nsweeps=3, seed=4, prob_translate=0.5, max_rot=0.4,
                                                             nupdate=40)
    ro, mdo, mro, xo = _chain(oracle.open_system, s, boxes, **kw)
    rg, mdg, mrg, xg = _chain(_gpu(abi.PREC_FP64), s, boxes, **kw)
    for a, b in zip(ro, rg):
        for k in ("n_translate", "n_translate_accepted", "n_rotate", "n_rotate_accepted", "n_overlap"):
            assert a[k] == b[k], (k, a[k], b[k])
        scale = abs(a["energy"]["inter_vdw"]) + abs(a["energy"]["inter_q"]) + 1.0
        for k, v in a["energy"].items():
            assert abs(b["energy"][k] - v) <= FP64_TOL * scale, (k, v, b["energy"][k])
    assert np.allclose(mdg, mdo, rtol=1e-12) and np.allclose(mrg, mro, rtol=1e-12)
    assert np.max(np.abs(xg - xo)) < 1e-8


@pytest.mark.parametrize("kind", ["lj", "water"])
def test_mixed_bookkeeping_matches_fp64_recompute(kind):
    if kind == "lj":
        s, boxes, kw = mc_helpers.lj_small(), [1, 2], dict(nsweeps=20, seed=2)
    else:
        s, boxes, kw = mc_helpers.water_small(), [1], dict(nsweeps=10, seed=6, prob_translate=0.5, max_rot=0.4)
    res, _, _, xyz = _chain(_gpu(abi.PREC_MIXED), s, boxes, **kw)
    start = mc_helpers.recomputed_totals(oracle.fns(), s, s.molecules.flat_xyz(), boxes)
    again = mc_helpers.recomputed_totals(oracle.fns(), s, xyz, boxes)
    for r, e0, e in zip(res, start, again):
        assert r["n_translate_accepted"] > 0
        # FP32 pair energies and phases, FP64 bookkeeping: the running energy
        # follows the FP32 energy surface, within 1e-6 of the largest energy
        # scale the chain saw (the random start holds overlapping pairs)
        scale = max(abs(x["inter_vdw"]) + abs(x["inter_q"]) + abs(x["reciprocal"]) for x in (e0, e))
        assert abs(r["energy"]["total"] - e["total"]) <= 1e-6 * scale, (r["energy"]["total"], e["total"], scale)


def test_mc_state_after_sweeps_drives_widom_and_energies():
    s = mc_helpers.lj_small(nboxes=1)
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        g.system_total_energy(1)
        res, _, _ = g.mc_sweeps([1], 2, [[0.8]], [[0.0]], seed=1)
        e_run = res[0]["energy"]["total"]
        e_new, _ = g.system_total_energy(1)
    assert abs(e_new["total"] - e_run) <= FP64_TOL * abs(e_new["inter_vdw"])


def test_mc_errors():
    s = mc_helpers.lj_small()
    with cg.open_system(s, precision=abi.PREC_FP64) as g:
        with pytest.raises(abi.CassError) as e:
            g.mc_sweeps([1], 1, [[0.8]], [[0.0]], seed=1)
        assert e.value.code == abi.CASS_ESTATE
        g.system_total_energy(1)
        with pytest.raises(abi.CassError):
            g.mc_sweeps([1, 1], 1, [[0.8], [0.8]], [[0.0], [0.0]], seed=1)
