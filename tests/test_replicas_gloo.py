"""Multi-rank host path on CPU: two gloo ranks shard a global batch of small
oracle solves, time them, and reduce with MAX -- the same replica logic the
benchmark uses across GPUs (no data-path collective)."""

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from jaxfun_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import spectral as O

    info = replicas.rank_info()
    mine = replicas.shard(10, info.rank, info.world)
    V = O.Space1D("legendre", 10, True)
    K, M = V.stiffness_matrix(), V.mass_matrix()
    sols = {}
    for i in mine:
        b = np.random.default_rng(replicas.seed_base(0) + i).standard_normal((8, 8))
        sols[i] = O.kron_solve([(1.0, [K, M]), (1.0, [M, K])], b)
    t_local = 0.1 * (rank + 1)  # a deterministic stand-in for the measured time
    t = replicas.max_time(t_local, dist)
    gathered = [None] * world
    dist.all_gather_object(gathered, sols)
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        out.put((t, replicas.throughput(len(mine), world, t), sorted(merged)))
    dist.destroy_process_group()


def test_shard_partition():
    for total in (0, 1, 7, 10, 1024):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(total, r, world) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(total))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    t, thr, keys = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert t == pytest.approx(0.2)  # MAX over ranks
    assert thr == pytest.approx(2 * 5 / 0.2)
    assert keys == list(range(10))  # every problem solved exactly once
