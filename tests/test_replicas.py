"""Replica sharding and bookkeeping over two gloo ranks on the CPU (no GPU)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from gbpowspec.replicas import gather_rows, max_over_ranks, rank_seed, shard, world


def test_shard_is_disjoint_and_covering():
    for n in (0, 1, 7, 256):
        for size in (1, 2, 3, 8):
            parts = [shard(n, r, size) for r in range(size)]
            allidx = np.concatenate(parts) if parts else np.array([])
            assert sorted(allidx.tolist()) == list(range(n))
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_single_process_defaults():
    assert world() == (0, 1)
    assert max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    out = gather_rows(np.ones((2, 3)), np.array([3, 1]), 5)
    assert np.all(out[[1, 3]] == 1.0) and np.all(np.isnan(out[[0, 2, 4]]))
    assert rank_seed(7, 0) != rank_seed(7, 1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, size, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    try:
        r, s = world()
        idx = shard(10, r, s)
        # each rank "times" its own share; the job time is the slowest rank's
        t = max_over_ranks([1.0 + r, 10.0 - r])
        rows = np.stack([np.full(3, float(i)) for i in idx])
        full = gather_rows(rows, idx, 10)
        q.put((r, idx.tolist(), t, None if full is None else full[:, 0].tolist()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_time_and_gather():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        r, idx, t, full = q.get(timeout=120)
        got[r] = (idx, t, full)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0][0] == [0, 2, 4, 6, 8] and got[1][0] == [1, 3, 5, 7, 9]
    assert got[0][1] == got[1][1] == [2.0, 10.0]
    assert got[0][2] == [float(i) for i in range(10)]
    assert got[1][2] is None
