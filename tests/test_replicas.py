"""Replica sharding across ranks: world-size-2 gloo processes on the CPU split
a batch of impacts by particle count, run their shares (a host stand-in for the
GPU runner) and gather the results on rank 0."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from deorbit_gb300 import ic, replicas


def test_partition_is_a_balanced_cover():
    sizes = ic.batch_sizes(256)
    for world in (1, 2, 3, 8):
        parts = replicas.partition(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in map(np.asarray, parts)]
        assert max(loads) - min(loads) <= int(sizes.max())
    assert replicas.partition(sizes, 4) == replicas.partition(list(sizes), 4)  # deterministic


def test_request_shards_cover_the_stream():
    reqs = list(range(23))
    shards = [replicas.shard_requests(reqs, r, 3) for r in range(3)]
    assert sorted(x for s in shards for x in s) == reqs


def host_runner(scenarios, steps):
    return [{"n": sc.n, "checksum": float(sc.pos.sum() + steps)} for sc in scenarios]


def _worker(rank, world, port, scs, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local = replicas.run_shard(scs, 3, rank, world, runner=host_runner)
        out = replicas.gather(local, rank, world)
        if rank == 0:
            q.put(out)
        else:
            assert out is None
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.timeout(120)
def test_gloo_world2_gathers_every_impact():
    scs = ic.batch_impacts(count=10, lo=300, hi=2000)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, scs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=100)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == host_runner(scs, 3)
