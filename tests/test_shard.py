"""Box sharding of the batched Widom workload (cassandra_gb300/shard.py) on two
gloo ranks, with the FP64 oracle as each rank's engine: the per-box Widom
accumulators merged over the ranks equal, bit for bit, those of one rank that
ran every box.  The reference reduces the same accumulators over its OpenMP
threads (widom_insert.f90:255-263)."""
import os
import pickle
import socket

import numpy as np
import pytest

from cassandra_gb300 import shard, workloads

SIZES = [200, 320, 260, 230, 280]
BOXES = [1, 2, 3, 4, 5]
N_INS, KAPPA, SEED = 48, 6, 11


def _system():
    return workloads.widom_batch_system(nboxes=len(SIZES), sizes=SIZES, seed=3, nconfig=40)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_path):
    import torch.distributed as dist

    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = _system()
        with oracle.open_system(s) as o:
            mine = shard.assign_boxes(BOXES, world, SIZES)[rank]
            for b in mine:
                o.system_total_energy(b)
            res, ran = shard.widom_sharded(o, 2, BOXES, N_INS, KAPPA, KAPPA, SEED, weights=SIZES)
        with open(f"{out_path}.{rank}", "wb") as f:
            pickle.dump((res, ran), f)
    finally:
        dist.destroy_process_group()


def test_assign_boxes_balanced_and_deterministic():
    parts = shard.assign_boxes(BOXES, 2, SIZES)
    assert sorted(b for p in parts for b in p) == BOXES
    assert parts == shard.assign_boxes(BOXES, 2, SIZES)
    loads = [sum(SIZES[b - 1] for b in p) for p in parts]
    assert max(loads) - min(loads) <= max(SIZES)
    assert shard.assign_boxes([1, 2], 3) == [[1], [2], []]
    with pytest.raises(ValueError):
        shard.assign_boxes([1], 0)


def test_two_gloo_ranks_match_one_rank_bit_for_bit(tmp_path):
    import torch.multiprocessing as mp

    from oracle import oracle
    oracle.build()
    out = str(tmp_path / "res")
    mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    merged = []
    ran = []
    for r in range(2):
        with open(f"{out}.{r}", "rb") as f:
            res, mine = pickle.load(f)
        merged.append(res)
        ran.append(mine)
    assert merged[0] == merged[1]
    assert sorted(ran[0] + ran[1]) == BOXES and not set(ran[0]) & set(ran[1])
    s = _system()
    with oracle.open_system(s) as o:
        for b in BOXES:
            o.system_total_energy(b)
        single = o.widom_insert(2, BOXES, N_INS, KAPPA, KAPPA, SEED)
    for a, b in zip(merged[0], single):
        for k in shard.FIELDS:
            assert a[k] == b[k], (k, a[k], b[k])
    assert all(r["n_insertions"] == N_INS for r in single)
    assert np.isfinite([r["widom_sum"] for r in single]).all()
