"""Autotuner for the neighbour-search shape of the SPH engine.

Chooses, per (GPU, precision, workload class), the traversal cell width (as a
multiple of h_init), the neighbour-list builder (one thread per particle, one
warp per column run or one warp per particle) and the thread-block size, by timing a few KDK steps of
a representative workload with CUDA events on the engine stream.  Results are
cached in a JSON file so a run pays for the search once per class.

A workload class is (strength on/off, particles per impact rounded to a power
of two); classes share a configuration because the cost drivers -- particles
per cell and neighbours per particle -- depend on those and not on geometry.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.environ.get("DEORBIT_SPH_TUNE_CACHE", os.path.join(HERE, "_tune", "autotune.json"))

CELL_FACTORS = (0.75, 1.0, 1.5)
# graded lattices: h spans an order of magnitude, and cells sized for the finest
# particles make the coarse ones search hundreds of columns
GRADED_CELL_FACTORS = (1.5, 2.0, 3.0, 4.0)
# (cell factor, z cell factor) pairs also tried there: flatter cells shorten the
# column chords of the list build at the price of more cells to sort
GRADED_FLAT_CELLS = ((3.0, 0.5), (4.0, 0.5), (3.0, 0.33))
# (cell factor, z cell factor) pairs also tried with the per-thread builder on
# uniform lattices: slightly flatter cells shorten the chords of the list build
FLAT_CELLS = ((1.0, 0.75), (0.85, 0.75), (1.0, 0.6))
SLACKS = (0.03, 0.06)
BLOCKS = (128, 256)
LIST_MODES = (2, 1, 0)


def gpu_name(device=0) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "unknown-gpu"


def workload_class(sc, per_impact_n=None) -> str:
    n = per_impact_n if per_impact_n is not None else sc.n
    strength = int(bool(sc.params.get("damage_on", 0)) or any(m.get("G", 0) > 0 for m in sc.materials))
    return f"s{strength}_n2^{int(round(math.log2(max(n, 2))))}"


SHIPPED = os.path.join(HERE, "tuned_gb300.json")   # measured on GB300, committed


def _load():
    """Runtime cache over the shipped table (runtime entries win)."""
    out = {}
    for path in (SHIPPED, CACHE):
        try:
            with open(path) as f:
                out.update(json.load(f))
        except Exception:
            pass
    return out


def _save(d):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    try:
        with open(SHIPPED) as f:
            shipped = json.load(f)
    except Exception:
        shipped = {}
    d = {k: v for k, v in d.items() if shipped.get(k) != v}
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def key(precision, cls, device=0) -> str:
    return f"{gpu_name(device)}|p{precision}|{cls}"


def measure(sc, precision, cfg, device=0, steps=3, warmup=2) -> float:
    """ms per KDK step of `sc` (one scenario, or a list run as one batch)
    under configuration cfg (dict of engine options)."""
    from . import ic, sph

    ctx = sph.Context(precision, device)
    try:
        ctx.set_tuning(cfg.get("block", 0), cfg.get("cell_factor", 0.0))
        ctx.set_option("cell_factor_z", cfg.get("cell_factor_z", 1.0))
        ctx.set_option("slack", cfg.get("slack", 0.08))
        ctx.set_option("list_mode", cfg.get("list_mode", 1))
        mids = {}
        for one in (sc if isinstance(sc, (list, tuple)) else [sc]):
            ic.to_context(ctx, one, material_ids=mids)
        ctx.init()
        for _ in range(warmup):
            ctx.run(1)
        ctx.event_record(0)
        ctx.run(steps)
        ctx.event_record(1)
        return ctx.event_elapsed(0, 1) / steps
    finally:
        ctx.close()


def tune(sc, precision, device=0, steps=3, warmup=2, candidates=None, force=False, verbose=False):
    """Search the candidates on `sc` (a scenario, or a list of scenarios run
    as one batch and classed by their mean size), cache and return
    (best_cfg, table)."""
    if isinstance(sc, (list, tuple)):
        cls = workload_class(sc[0], sum(x.n for x in sc) // len(sc))
    else:
        cls = workload_class(sc)
    k = key(precision, cls, device)
    cache = _load()
    if not force and k in cache:
        return cache[k]["best"], cache[k]["table"]
    if candidates is None:
        candidates = [dict(list_mode=lm, slack=sl, cell_factor=f, block=b)
                      for lm, sl, f, b in itertools.product(LIST_MODES, SLACKS, CELL_FACTORS, BLOCKS)
                      if not (lm == 1 and b != 128)]
        candidates += [dict(list_mode=0, slack=sl, cell_factor=f, cell_factor_z=fz, block=b)
                       for sl, (f, fz), b in itertools.product(SLACKS, FLAT_CELLS, BLOCKS)]
    table = []
    for cfg in candidates:
        t0 = time.perf_counter()
        try:
            ms = measure(sc, precision, cfg, device, steps, warmup)
        except Exception as e:  # a shape that cannot run is skipped, not fatal
            ms = float("inf")
            cfg = dict(cfg, error=str(e))
        table.append(dict(cfg, ms_per_step=ms))
        if verbose:
            print(f"  {cfg} -> {ms:.3f} ms/step ({time.perf_counter() - t0:.1f} s)", flush=True)
    best = min(table, key=lambda r: r["ms_per_step"])
    best = {k2: best[k2] for k2 in ("list_mode", "slack", "cell_factor", "cell_factor_z", "block") if k2 in best}
    n = sum(x.n for x in sc) if isinstance(sc, (list, tuple)) else sc.n
    cache[k] = {"best": best, "table": table, "n": n, "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
    _save(cache)
    return best, table


def lookup(sc, precision, device=0, per_impact_n=None):
    """Cached best configuration for this workload class, or None."""
    cache = _load()
    e = cache.get(key(precision, workload_class(sc, per_impact_n), device))
    return None if e is None else e["best"]


def apply(ctx, sc, precision, device=0, per_impact_n=None, default=None):
    """Configure a fresh context from the cache (or `default`)."""
    cfg = lookup(sc, precision, device, per_impact_n) or default
    if cfg:
        ctx.set_tuning(int(cfg.get("block", 0)), float(cfg.get("cell_factor", 0.0)))
        ctx.set_option("cell_factor_z", float(cfg.get("cell_factor_z", 1.0)))
        ctx.set_option("slack", cfg.get("slack", 0.08))
        ctx.set_option("list_mode", cfg.get("list_mode", 1))
    return cfg


def ship(device=0, verbose=True, only=None):
    """Re-measure the table shipped for this GPU model (tuned_gb300.json on a
    GB300): the 1,048,576-particle grazing impact in both forms, the batched
    class (32 impacts of the 256-impact sweep run as one batch) and the
    16,777,216-particle graded run (cell factors only).  Returns the entries."""
    from . import ic

    out = {}
    runs = [(ic.grazing(), 1, None), (ic.grazing(), 0, None),
            (ic.batch_impacts(256)[:32], 1, None),
            (ic.large_graded(), 1, [dict(list_mode=0, slack=0.03, cell_factor=f, block=128)
                                    for f in GRADED_CELL_FACTORS] +
             [dict(list_mode=0, slack=0.03, cell_factor=f, cell_factor_z=fz, block=128)
              for f, fz in GRADED_FLAT_CELLS])]
    if only is not None:  # re-measure some entries, keep the others
        runs = [runs[i] for i in only]
        try:
            with open(SHIPPED) as f:
                out = json.load(f)
        except Exception:
            out = {}
    for sc, prec, cands in runs:
        best, table = tune(sc, prec, device, candidates=cands, force=True, verbose=verbose)
        cls = workload_class(sc[0], sum(x.n for x in sc) // len(sc)) if isinstance(sc, list) else workload_class(sc)
        out[key(prec, cls, device)] = dict(_load()[key(prec, cls, device)],
                                           source="autotune.ship on GB300")
        if verbose:
            print(key(prec, cls, device), "->", best, flush=True)
    with open(SHIPPED if "GB300" in gpu_name(device) else CACHE + ".ship.json", "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    return out


if __name__ == "__main__":
    import sys
    ship(only=[int(a) for a in sys.argv[1:]] or None)
