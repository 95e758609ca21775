"""CPU, world_size 2 over gloo: sharding of a batch of systems, max-over-ranks
timing and the gather of per-rank results (the multi-GPU layout of the
batched path, with SciPy standing in for the per-rank GPU solve)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mpdok_gb300.replicas import gather_results, max_over_ranks, shard_imbalance, shard_systems


def test_shard_covers_every_system_once_and_balances():
    rng = np.random.default_rng(3)
    sizes = list(rng.integers(500, 8001, size=256))
    for world in (1, 2, 4, 8):
        parts = shard_systems(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        assert shard_imbalance(sizes, parts) < 1.02
    assert sum(1 for p in shard_systems([10, 20], 4) if p) == 2  # more ranks than systems: some idle
    with pytest.raises(ValueError):
        shard_systems([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import scipy.linalg as sl
    from oracle import batch_ref as R
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(0)
        sizes = [int(n) for n in rng.integers(20, 80, size=7)]
        systems = [(rng.uniform(0, 1, (n, 2)), float(rng.uniform(3, 6)), rng.standard_normal((n, 2))) for n in sizes]
        mine = shard_systems(sizes, world)[rank]
        local = {}
        for i in mine:
            X, eps, B = systems[i]
            local[i] = R.solve(X, eps, 1e-3, B)[0]
        allres = gather_results(local)
        t = max_over_ranks(float(rank + 1))
        if rank == 0:
            ok = sorted(allres) == list(range(len(sizes))) and t == float(world)
            for i, (X, eps, B) in enumerate(systems):
                A = R.rbf(X, eps, 1e-3)
                ok = ok and np.allclose(allres[i], sl.solve(A, B), rtol=1e-9, atol=1e-12)
            q.put(bool(ok))
    finally:
        dist.destroy_process_group()


def test_two_rank_shard_gather_and_max_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True
