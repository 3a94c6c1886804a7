"""Data-parallel replicas across GPUs.

Impacts are independent, so N GPUs run N engine contexts (one process per
GPU) on disjoint shares of a batch or of a request stream, with no collective
on the data path.  The only exchange is the gather of results at the end
(torch.distributed object gather: gloo on CPU, NCCL on GPUs).

Shares are balanced by particle count (a deterministic longest-first split),
since a step's cost grows with the particles it covers, and every rank
computes the same split from the same inputs, so no coordination is needed to
agree on it.
"""
from __future__ import annotations

RESULT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "u", "rho", "D")


def partition(sizes, world):
    """Item indices per rank, balanced in total size: items taken largest
    first (ties by index), each to the least-loaded rank (ties by rank).
    Deterministic; every item lands on exactly one rank; each list ascending."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(i)
        loads[r] += int(sizes[i])
    return [sorted(p) for p in parts]


def shard_requests(requests, rank, world):
    """A request stream split round-robin in arrival order (each GPU serves
    its own queue; each sub-stream keeps the arrival process's statistics)."""
    return [r for i, r in enumerate(requests) if i % world == rank]


def gpu_runner(scenarios, steps, device=0, precision=None, fields=RESULT_FIELDS):
    """Run a share of impacts in one context for `steps` device-controlled
    steps; returns one {field: array} per impact, in order."""
    from . import ic, sph

    ctx = sph.Context(sph.MIXED if precision is None else precision, device)
    try:
        mids = {}
        ids = [ic.to_context(ctx, sc, material_ids=mids) for sc in scenarios]
        if ids:
            ctx.init()
            ctx.run(steps)
        return [{k: ctx.read(b, k) for k in fields} for b in ids]
    finally:
        ctx.close()


def run_shard(scenarios, steps, rank, world, runner=None, **kw):
    """This rank's share of `scenarios`: {item index: result}."""
    idx = partition([sc.n for sc in scenarios], world)[rank]
    out = (runner or gpu_runner)([scenarios[i] for i in idx], steps, **kw)
    return dict(zip(idx, out))


def gather(local, rank, world, dst=0):
    """Merge every rank's {index: result} on rank `dst` (others get None);
    the merged results are returned as a list in index order."""
    import torch.distributed as dist

    if world == 1:
        return [local[i] for i in sorted(local)]
    objs = [None] * world if rank == dst else None
    dist.gather_object(local, objs, dst=dst)
    if rank != dst:
        return None
    merged = {}
    for part in objs:
        overlap = merged.keys() & part.keys()
        if overlap:
            raise RuntimeError(f"items computed on two ranks: {sorted(overlap)[:5]}")
        merged.update(part)
    return [merged[i] for i in sorted(merged)]
