"""Box sharding of the batched Widom workload over ranks (one GPU per rank).

The reference's only exchange on this path is the sum of the Widom
accumulators over the OpenMP threads that shared a frame's insertions
(widom_insert.f90:255-263, ``REDUCTION(+: widom_sum, n_overlaps, ...)``).
Here the units are whole boxes: every rank runs ``cass_widom_insert`` on its
own boxes, and the per-box accumulators are merged on the host with one small
all-reduce of a [boxes x 5] FP64 array in which each box has exactly one
non-zero contribution.  The merge is therefore exact, and because insertion k
of box b draws from its own lfsr258 stream seeded by (seed, b, k), the merged
result is identical, bit for bit, to a one-rank run over all boxes.

The engine is anything with the ``widom_insert`` method of
``cassandra_gb300.abi.Context`` (a GPU context, or the CPU oracle in tests).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

FIELDS = ("widom_sum", "prefactor", "n_insertions", "n_overlaps", "n_trials")
_INT_FIELDS = {"n_insertions", "n_overlaps", "n_trials"}


def assign_boxes(boxes: Sequence[int], world: int, weights: Sequence[float] | None = None) -> list[list[int]]:
    """Deterministic split of `boxes` over `world` ranks: heaviest box first to the
    least-loaded rank (ties to the lower rank); each rank's list keeps the input order.
    `weights` (e.g. atoms per box) default to 1."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = [1.0] * len(boxes) if weights is None else [float(x) for x in weights]
    if len(w) != len(boxes):
        raise ValueError("one weight per box")
    load = [0.0] * world
    owner = [0] * len(boxes)
    for i in sorted(range(len(boxes)), key=lambda k: (-w[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += w[i]
    return [[b for b, o in zip(boxes, owner) if o == r] for r in range(world)]


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is part of the environment
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def merge_box_results(boxes: Sequence[int], mine: Sequence[int], results: Sequence[dict]) -> list[dict]:
    """All-reduce the per-box accumulators of this rank's boxes (`mine`, with their
    `results` in the same order) into the results of every box in `boxes`."""
    index = {b: k for k, b in enumerate(boxes)}
    buf = np.zeros((len(boxes), len(FIELDS)), dtype=np.float64)
    for b, r in zip(mine, results):
        buf[index[b]] = [float(r[f]) for f in FIELDS]
    dist = _dist()
    if dist is not None and dist.get_world_size() > 1:
        import torch
        t = torch.from_numpy(buf)
        if dist.get_backend() == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        buf = t.cpu().numpy()
    return [{f: (int(v) if f in _INT_FIELDS else float(v)) for f, v in zip(FIELDS, row)} for row in buf]


def widom_sharded(engine, is_: int, boxes: Sequence[int], n_insertions: int, kappa_ins: int, kappa_dih: int,
                  seed: int, weights: Sequence[float] | None = None) -> tuple[list[dict], list[int]]:
    """Widom insertions into `boxes`, this rank's share on `engine`, merged over the
    ranks of the default process group (one rank without one).  Returns the per-box
    results of every box (in the order of `boxes`) and the boxes this rank ran."""
    dist = _dist()
    world = dist.get_world_size() if dist is not None else 1
    rank = dist.get_rank() if dist is not None else 0
    mine = assign_boxes(boxes, world, weights)[rank]
    res = engine.widom_insert(is_, mine, n_insertions, kappa_ins, kappa_dih, seed) if mine else []
    return merge_box_results(boxes, mine, res), mine
