"""Replica bookkeeping for N > 1 GPUs, on CPU: two `gloo` ranks reduce the
timing the way the bench does (max of the device times, sum of the units),
and the cost partition of independent circuits is deterministic, complete
and balanced."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from afquantumsim_gb300 import circuits, replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, units = replicas.reduce_timing(10.0 + 5.0 * rank, 480 * (rank + 1))
        # every rank computes the same split of a sweep and takes its own slice
        items = circuits.vqe_sweep(64, seed=5)
        costs = [len(ops) * (1 << n) for n, ops in items]
        mine = replicas.partition(costs, world)[rank]
        got = [None] * world
        dist.all_gather_object(got, mine)
        out[rank] = (ms, units, replicas.rank_seed(3, rank), got)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_partition():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True,
                       start_method="spawn")
    res = dict(out)
    assert set(res) == {0, 1}
    for r in range(world):
        ms, units, seed, slices = res[r]
        assert ms == 15.0  # the slowest rank's time
        assert units == 480 * 1 + 480 * 2  # all ranks' gate applications
        assert seed == 3 + r
    s0, s1 = res[0][3], res[1][3]
    assert s0 == s1  # every rank saw the same split
    flat = sorted(s0[0] + s0[1])
    assert flat == list(range(64)) and not set(s0[0]) & set(s0[1])


def test_reduce_timing_single_rank_is_identity():
    assert replicas.reduce_timing(3.5, 7) == (3.5, 7.0)


def test_partition_balanced_and_deterministic():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(1, 1 << 20, size=500))
    for world in (1, 2, 3, 8):
        parts = replicas.partition(costs, world)
        assert parts == replicas.partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(500))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT bound: no rank exceeds the mean by more than the largest item
        assert max(loads) <= sum(costs) / world + max(costs)
    with pytest.raises(ValueError):
        replicas.partition(costs, 0)
