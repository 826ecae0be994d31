"""Batched QR sharded over ranks: cost-balanced partition and the final
gather, with world_size 2 over gloo on CPU (the per-rank factorization here is
the oracle's LAPACK, standing in for each rank's GPU)."""
import os
import socket

import numpy as np
import pytest

from hqrrp_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_partition_is_complete_deterministic_and_balanced():
    rng = np.random.default_rng(0)
    m = np.exp(rng.uniform(np.log(64), np.log(1024), 4096)).astype(int)
    shapes = [(int(a), int(np.exp(rng.uniform(np.log(32), np.log(min(a, 512)))))) for a in m]
    for world in (1, 2, 4, 8):
        parts = shard.partition_by_cost(shapes, world)
        assert sorted(i for p in parts for i in p) == list(range(len(shapes)))
        assert parts == shard.partition_by_cost(shapes, world)
        loads = shard.shard_loads(shapes, parts)
        assert max(loads) <= 1.01 * min(loads)


def _worker(rank, world, port, shapes, seed, q):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o = oracle.Oracle()
        parts = shard.partition_by_cost(shapes, world)
        mine = parts[rank]
        local = []
        for i in mine:
            m, n = shapes[i]
            A = oracle.gaussian(m, n, seed + i)
            Af, jp, tau, info = o.dgeqp3(A)
            local.append((jp.tolist(), float(np.abs(np.diag(Af[:min(m, n)])).sum())))
        merged = shard.gather_to_root(local, mine, world, rank)
        if rank == 0:
            q.put(sorted(merged.items()))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_shard_and_gather():
    import torch.multiprocessing as mp
    import oracle
    shapes = [(80 + 7 * i, 40 + 3 * (i % 9)) for i in range(12)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, shapes, 11, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [k for k, _ in got] == list(range(len(shapes)))
    o = oracle.Oracle()
    for i, (jp, dsum) in got:
        m, n = shapes[i]
        Af, jo, _, _ = o.dgeqp3(oracle.gaussian(m, n, 11 + i))
        assert jp == jo.tolist()
        assert abs(dsum - np.abs(np.diag(Af[:min(m, n)])).sum()) <= 1e-10 * dsum
