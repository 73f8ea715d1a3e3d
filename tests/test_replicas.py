"""Replicas over several ranks (CPU, gloo, world size 2): sharding of the chains and the reductions of results."""
import os
import socket

import numpy as np
import pytest

from jellyfysh_gb300 import replicas

torch = pytest.importorskip("torch")


def test_shards_cover_every_chain_once_and_balance_the_work():
    rng = np.random.default_rng(0)
    work = rng.integers(32, 2049, size=4096) * 128.0
    for world in (1, 2, 3, 8):
        blocks = [replicas.shard(work, world, r) for r in range(world)]
        assert blocks[0][0] == 0 and blocks[-1][1] == len(work)
        assert all(blocks[r][1] == blocks[r + 1][0] for r in range(world - 1))
        loads = [work[a:b].sum() for a, b in blocks]
        assert max(loads) - min(loads) <= 2 * work.max()
    assert replicas.shard([], 2, 1) == (0, 0)
    with pytest.raises(ValueError):
        replicas.shard(work, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r processed 1000 (r + 1) events in 10 (r + 1) ms
        events, ms, rate = replicas.timed_throughput(1000.0 * (rank + 1), 10.0 * (rank + 1))
        histogram = replicas.sum_over_ranks(np.arange(5, dtype=np.float64) * (rank + 1))
        first, last = replicas.shard([1.0] * 10, world, rank)
        results.put((rank, events, ms, rate, histogram.tolist(), first, last))
    finally:
        dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    context = mp.get_context("spawn")
    results = context.Queue()
    port = _free_port()
    processes = [context.Process(target=_rank, args=(r, 2, port, results)) for r in range(2)]
    for p in processes:
        p.start()
    for p in processes:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(results.get(timeout=10) for _ in range(2))
    for rank, events, ms, rate, histogram, first, last in got:
        assert events == 3000.0 and ms == 20.0 and rate == pytest.approx(150000.0)
        assert histogram == [0.0, 3.0, 6.0, 9.0, 12.0]
    assert [(g[5], g[6]) for g in got] == [(0, 5), (5, 10)]
