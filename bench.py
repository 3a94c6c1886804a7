"""Benchmark of the SPH step loop on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload grazing|halfspace] [--n PARTICLES]

Workload (default): the grazing strength + damage impact, 1,048,576 particles
(1 km iron sphere at 3 deg, 8 km/s into a granite slab; von Mises iron, Collins
granite, multi-flaw damage), seeded synthetic inputs.  A step is one KDK step
of the whole workload (sph.hpp:357-377) with the CFL dt computed on the device.

value   particle-steps/s of the mixed form (FP32 pairs / EOS / stress, FP64
        positions and energies), state resident in HBM, CUDA events on the
        engine stream around exactly K steps.
e2e     the same metric through the C ABI with host buffers: every step
        writes the carried state from pinned host memory, steps, and reads it
        back (a drop-in caller that keeps System's vectors on the host), as
        one sph_step_fields call per step; e2e.separate_calls times the same
        steps as sph_write_fields + sph_timestep + sph_step + sph_read_fields.
plain_fp64  the FP64 plain form on the same workload (the 4x comparison).
accuracy_vs_oracle  both GPU forms against the FP64 CPU oracle on a bounded
        sample of the workload (per-field rel-L2, pass / fail at 1e-4).
cpu_baseline  the FP64 CPU oracle on host cores (reference thread cap of 16)
        over the same workload (2 steps), with the precision-matched ratio
        (plain FP64 GPU over CPU) beside the mixed one.
--impl reference  times that CPU oracle as the reference arm on the same
        workload (--cpu-sample N: a cropped sample instead).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s batched vs plain GPU at ≤1e-4 FP64 rel err; p50/p99 latency"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle of one launch: compulsory reads of the
# particle's own state and writes of its results, plus the list entries the
# kernel must write or read; neighbour re-reads and sort scratch excluded.
# Kernel of each single-kernel class and its algorithmic bytes per particle
# in the mixed form: (fixed bytes, list bytes per list entry).  The neighbour
# list is written once per step by k_list_thread and read by every k_density
# and k_force launch; its length (own + reverse entries per particle) is read
# from the engine after the profiled steps.
KERNEL_OF_CLASS = {"list_density": "k_list_thread", "density": "k_density", "force": "k_force",
                   "eos": "k_eos", "damage": "k_damage", "finish": "k_finish"}
ALG_BYTES = {
    # k_list_thread: reads pf 16, cpk 4, refbin 8, imp 2; writes count 4 and 4 B per entry
    "list_density": (34, 4),
    # k_density: reads pf 16, cpk 4, imp 2, count 4, h, mass; writes rho, h, pf.w 4; reads 4 B per entry
    "density": (16 + 4 + 2 + 4 + 2 * 4 + 2 * 4 + 4, 4),
    # k_force: reads pf 16, cpk 4, imp 2, mat 1, count 4, the packed record
    # (h, rho, csig, P/rho^2, dscale/rho^2, dscale, Rart, P, m/rho, mass: 10 x 4),
    # vel 3 x 4, S 6 x 4, u 8; writes acc 3, dudt 1, dSdt 6, eps_work 1 (x 4); reads 4 B per entry
    "force": (16 + 4 + 2 + 1 + 4 + 10 * 4 + 3 * 4 + 6 * 4 + 8 + (3 + 1 + 6 + 1) * 4, 4),
    # k_eos: reads rho, u 8, mat 1, D, S 6; writes P, cs, packed record 40
    "eos": (4 + 8 + 1 + 4 + 24 + 8 + 40, 0),
    "damage": (4 + 4 + 4 + 8 + 4 + 4, 0),
    "finish": (8 * 4 + 6 * 4 + 6 * 4, 0),
}
# FP32 flops executed per list entry (per iteration for k_density), from the
# ncu instruction counters of the mixed kernels (2 x FFMA + FADD + FMUL over
# the entries processed; captures in profiles/): the numerator of the FP32
# issue fraction beside the HBM one.
FLOPS_PER_ENTRY = {"force": 169, "density": 34}
# FP32 lanes per SM of compute capability 10.x (sm_100 / sm_103): the FP32
# issue peak is SMs x lanes x 2 flops (FMA) x the maximum SM clock, both read
# from the device at run time
FP32_LANES_PER_SM = 128


def fp32_peak_tflops(device, sm_max_mhz):
    import torch
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    return sms * FP32_LANES_PER_SM * 2 * sm_max_mhz * 1e6 / 1e12, sms
# Compulsory state traffic of one particle-step, strength + damage, from the
# engine's layout: (bytes per field, access) with access "rw" for carried state
# read and written once, "r" read-only, "w" written once.  Positions,
# velocities and internal energy are FP64 in both forms; the rest is FP64 in
# the plain form and FP32 in the mixed one.  Lists, neighbour re-reads and sort
# scratch are excluded.
def state_layout(real_bytes):
    R = real_bytes
    return {"pos": (24, "rw"), "vel": (24, "rw"), "u": (8, "rw"), "h": (R, "rw"), "acc": (3 * R, "rw"),
            "dudt": (R, "rw"), "S": (6 * R, "rw"), "D": (R, "rw"), "dSdt": (6 * R, "rw"),
            "mass": (R, "r"), "eps_act": (R, "r"), "mat": (1, "r"), "fixed": (1, "r"), "rho": (R, "w")}


def step_bytes(real_bytes):
    return sum(b * (2 if a == "rw" else 1) for b, a in state_layout(real_bytes).values())


# frozen per form (a unit test recomputes them from state_layout)
STEP_BYTES = {8: 426, 4: 270}


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload(name, n):
    from deorbit_gb300 import ic
    if name == "halfspace":
        return ic.impact_halfspace()
    return ic.grazing(n_total=n)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.lines = []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                out, _ = self.p.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def time_form(sph, ic, sc, precision, steps, warmup, device, options=None):
    """Init (untimed), W warm-up steps, then exactly K timed steps in the
    production mode (captured CUDA graphs, no per-kernel events); then K more
    steps with per-kernel CUDA events for the kernel breakdown (not timed).
    options: engine options set after the tuned ones."""
    from deorbit_gb300 import autotune
    ctx = sph.Context(precision, device)
    autotune.apply(ctx, sc, precision, device)
    for k, v in (options or {}).items():
        ctx.set_option(k, v)
    b = ic.to_context(ctx, sc)
    ctx.init()
    ctx.run(max(warmup, 3))  # also captures the step graphs
    ctx.synchronize()
    l0 = ctx.launches()
    ctx.event_record(0)
    ctx.run(steps)
    ctx.event_record(1)
    ms = ctx.event_elapsed(0, 1)
    ctx.synchronize()
    l1 = ctx.launches()
    ctx.set_profiling(True)
    ctx.kernel_stats_reset()
    ctx.run(steps)
    ctx.synchronize()
    kst = ctx.kernel_stats()
    ctx.set_profiling(False)
    return ctx, b, ms, kst, l1 - l0


def mixed_error(sph, ic, sc, steps, device):
    """rel-L2 of the mixed form against the FP64 form after `steps` steps with
    the same dt sequence (taken from the FP64 form)."""
    c64 = sph.Context(sph.FP64, device)
    b64 = ic.to_context(c64, sc)
    c32 = sph.Context(sph.MIXED, device)
    b32 = ic.to_context(c32, sc)
    c64.init()
    c32.init()
    for _ in range(steps):
        dt = c64.timestep(b64)
        c64.step(dt)
        c32.step(dt)
    out = {}
    for grp, names in (("pos", ["x", "y", "z"]), ("vel", ["vx", "vy", "vz"]), ("u", ["u"]), ("rho", ["rho"]),
                       ("P", ["P"]), ("S", ["Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"]), ("D", ["D"])):
        a = np.concatenate([c32.read(b32, k) for k in names])
        r = np.concatenate([c64.read(b64, k) for k in names])
        nr = np.linalg.norm(r)
        out[grp] = float(np.linalg.norm(a - r) / nr) if nr > 0 else float(np.linalg.norm(a - r))
    c64.close()
    c32.close()
    return out


ACC_FIELDS = (("pos", ["x", "y", "z"]), ("vel", ["vx", "vy", "vz"]), ("u", ["u"]), ("rho", ["rho"]),
              ("P", ["P"]), ("S", ["Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"]), ("D", ["D"]))


def _group_errors(get_a, get_r, mask=None):
    out = {}
    for grp, names in ACC_FIELDS:
        a = np.concatenate([get_a(k) if mask is None else get_a(k)[mask] for k in names])
        r = np.concatenate([get_r(k) if mask is None else get_r(k)[mask] for k in names])
        nr = np.linalg.norm(r)
        out[grp] = float(np.linalg.norm(a - r) / nr) if nr > 0 else float(np.linalg.norm(a - r))
    return out


def accuracy_vs_oracle(sph, ic, sc, steps, device, tol=1e-4):
    """Both GPU forms against the FP64 CPU oracle on the same input (a bounded
    sample of the workload) after `steps` steps on the oracle's dt sequence:
    rel-L2 per field group, pass / fail against `tol`, and the particles whose
    damage differs by a flaw activation taken one step apart ("flips"), with the
    damage-switched fields over the particles without a flip."""
    from oracle import oracle as O

    S = O.from_scenario(sc, threads=min(os.cpu_count() or 1, 16))
    S.init()
    dts = []
    for _ in range(steps):
        dts.append(S.timestep())
        S.step(dts[-1])
    names = [k for _, ks in ACC_FIELDS for k in ks]
    ref = {k: S.field(k) for k in names}
    S.close()
    out = {"sample": f"{sc.n} particles cropped around the impact point, {steps} steps on the oracle's dt "
                     f"sequence", "tol": tol}
    for prec, name in ((sph.FP64, "fp64"), (sph.MIXED, "mixed")):
        ctx = sph.Context(prec, device)
        b = ic.to_context(ctx, sc)
        ctx.init()
        for dt in dts:
            ctx.step(dt)
        got = {k: ctx.read(b, k) for k in names}
        ctx.close()
        errs = _group_errors(got.__getitem__, ref.__getitem__)
        flip = np.abs(got["D"] - ref["D"]) > 1e-6
        rec = {"rel_l2": errs, "pass": sorted(k for k, v in errs.items() if v <= tol),
               "fail": sorted(k for k, v in errs.items() if not v <= tol), "damage_flips": int(flip.sum())}
        if flip.any():
            e2 = _group_errors(got.__getitem__, ref.__getitem__, mask=~flip)
            rec["rel_l2_without_flips"] = {"S": e2["S"], "D": e2["D"]}
        out[name] = rec
    return out


def e2e_rate(sph, ctx, b, n, steps, warmup, fused=True):
    """Steps through the C ABI with the carried state crossing the boundary
    from / to pinned host buffers every step: one sph_step_fields call per
    step (fused), or sph_write_fields + sph_timestep + sph_step +
    sph_read_fields."""
    names = ["x", "y", "z", "vx", "vy", "vz", "u", "hh", "D", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"]
    pinned = True
    try:
        import torch
        bufs = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k in names}
    except Exception:
        pinned = False
        bufs = {k: np.empty(n) for k in names}
    outs = [bufs[k] for k in names]
    ctx.read_many(b, names, outs)

    def one():
        if fused:  # inputs and outputs are the same pinned buffers
            ctx.step_fields(b, bufs, names, outs)
            return
        ctx.write_many(b, bufs)          # the step's inputs, pinned host -> device
        dt = ctx.timestep(b)
        ctx.step(dt)
        ctx.read_many(b, names, outs)    # the step's state, device -> pinned host

    for _ in range(warmup):
        one()
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    ctx.synchronize()
    el = time.perf_counter() - t0
    nbytes = 8 * n * len(names)
    return n * steps / el, el, nbytes, pinned


def cpu_rate(ic, sc, steps, threads=0):
    from oracle import oracle as O

    S = O.from_scenario(sc, threads=threads)
    S.init()
    t0 = time.perf_counter()
    for _ in range(steps):
        S.step(S.timestep())
    el = time.perf_counter() - t0
    return sc.n * steps / el, el, S.threads()


def plain_single_rate(sph, ic, scs, steps, device):
    """The plain form: one impact per context, FP64, host-driven
    timestep()/step() (the reference's System loop), impacts one after the
    other.  Returns particle-steps/s over the sample."""
    tot_ps, tot_s = 0, 0.0
    for sc in scs:
        ctx = sph.Context(sph.FP64, device)
        b = ic.to_context(ctx, sc)
        ctx.init()
        ctx.step(ctx.timestep(b))  # warm-up
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.step(ctx.timestep(b))
        ctx.synchronize()
        tot_s += time.perf_counter() - t0
        tot_ps += sc.n * steps
        ctx.close()
    return tot_ps / tot_s


def batched_section(sph, ic, device, steps, warmup, count=256):
    """The batched sweep: `count` impacts of uneven size in one context, every
    step one launch sequence over all of them (captured CUDA graphs), each
    impact with its own CFL dt."""
    from deorbit_gb300 import autotune
    scs = ic.batch_impacts(count)
    n_tot = sum(sc.n for sc in scs)
    out = {"workload": f"{count} impacts, iron into granite, strength + damage, N log-uniform 5k-80k",
           "n_particles": n_tot, "steps": steps}
    for prec, name in ((sph.MIXED, "mixed"), (sph.FP64, "fp64_batched")):
        ctx = sph.Context(prec, device)
        autotune.apply(ctx, scs[0], prec, device, per_impact_n=n_tot // count)
        mids = {}
        for sc in scs:
            ic.to_context(ctx, sc, material_ids=mids)
        ctx.init()
        ctx.run(max(warmup, 3))
        ctx.synchronize()
        l0 = ctx.launches()
        ctx.event_record(0)
        ctx.run(steps)
        ctx.event_record(1)
        ms = ctx.event_elapsed(0, 1)
        out[name] = {"value": n_tot * steps / (ms / 1000.0), "ms_per_step": ms / steps,
                     "gpu_launches": ctx.launches() - l0}
        # the kernels' own device time per step (CUDA events around every launch,
        # K further steps): what the graph-replayed step spends beyond it is the
        # most one persistent launch of the whole step could remove
        ctx.set_profiling(True)
        ctx.kernel_stats_reset()
        ctx.run(steps)
        ctx.synchronize()
        kst = ctx.kernel_stats()
        ctx.set_profiling(False)
        ksum = sum(v[0] for v in kst.values()) / steps
        out[name]["kernel_sum_ms_per_step"] = ksum
        out[name]["launches_per_step"] = out[name]["gpu_launches"] / steps
        out[name]["beyond_kernels_ms_per_step"] = ms / steps - ksum
        ctx.close()
    sample = scs[:: max(1, count // 8)][:8]
    out["plain_fp64_single"] = {"value": plain_single_rate(sph, ic, sample, steps, device),
                                "sample": f"{len(sample)} of the impacts, one at a time, {steps} steps each"}
    out["speedup_vs_plain_fp64_single"] = out["mixed"]["value"] / out["plain_fp64_single"]["value"]
    out["speedup_vs_fp64_batched"] = out["mixed"]["value"] / out["fp64_batched"]["value"]
    out["value"] = out["mixed"]["value"]
    return out


def large_section(sph, ic, device, steps, warmup, n_total=1 << 24):
    """The large graded run (mixed form), plus the mixed-vs-FP64 error on its
    1/64-particle replica (same geometry, 4x the spacing)."""
    from deorbit_gb300 import autotune
    t0 = time.perf_counter()
    sc = ic.large_graded(n_total)
    t_ic = time.perf_counter() - t0
    ctx = sph.Context(sph.MIXED, device)
    autotune.apply(ctx, sc, sph.MIXED, device)
    ic.to_context(ctx, sc)
    ctx.init()
    ctx.run(max(warmup, 3))
    ctx.synchronize()
    ctx.event_record(0)
    ctx.run(steps)
    ctx.event_record(1)
    ms = ctx.event_elapsed(0, 1)
    ctx.close()
    rep = ic.large_graded(n_total // 64)
    return {"workload": f"graded grazing slab 40x20x5 km, iron sphere r=500 m at 2 deg, 8 km/s, "
                        f"{sc.n} particles, surface spacing {sc.dx:.1f} m growing 6% per layer",
            "n_particles": sc.n, "value": sc.n * steps / (ms / 1000.0), "ms_per_step": ms / steps,
            "ic_build_s": t_ic,
            "replica_mixed_vs_fp64_rel_l2": mixed_error(sph, ic, rep, steps, device),
            "replica_vs_oracle": accuracy_vs_oracle(sph, ic, rep, steps, device),
            "replica_particles": rep.n}


def halfspace_section(sph, ic, device, steps=200):
    """The plain FP64 half-space impact (57,344 particles, 45 deg, 8 km/s,
    hydro-only, CFL 0.3) for its full 200 steps: the FP64 GPU solver with the
    host-driven timestep()/step() loop, and the CPU oracle (the reference's
    algorithm, thread cap 16) on the same input, with the FP64 fields' rel-L2
    between them at the end."""
    sc = ic.impact_halfspace()
    ctx = sph.Context(sph.FP64, device)
    b = ic.to_context(ctx, sc)
    ctx.init()
    ctx.synchronize()
    t0 = time.perf_counter()
    dts = []
    for _ in range(steps):
        dt = ctx.timestep(b)
        ctx.step(dt)
        dts.append(dt)
    ctx.synchronize()
    t_gpu = time.perf_counter() - t0
    names = ["x", "y", "z", "vx", "vy", "vz", "u", "rho", "P"]
    gpu = ctx.read_many(b, names)
    ctx.close()
    threads = min(os.cpu_count() or 1, 16)
    from oracle import oracle as O

    S = O.from_scenario(sc, threads=threads)
    S.init()
    t0 = time.perf_counter()
    for dt in dts:   # the GPU run's dt sequence (equal to the oracle's to 1e-9)
        S.step(dt)
    t_cpu = time.perf_counter() - t0
    err = {}
    for k in names:
        r = S.field(k)
        err[k] = float(np.linalg.norm(gpu[k] - r) / max(np.linalg.norm(r), 1e-300))
    return {"workload": "half-space impact, 48x48x24 granite + iron sphere r = 8 dx, 45 deg, 8 km/s, "
                        "hydro-only, CFL 0.3", "n_particles": sc.n, "steps": steps,
            "gpu_fp64": {"value": sc.n * steps / t_gpu, "ms_per_step": 1000 * t_gpu / steps,
                         "loop": "host-driven timestep()/step()"},
            "cpu_oracle": {"value": sc.n * steps / t_cpu, "cores": threads, "nproc": os.cpu_count()},
            "fp64_vs_oracle_rel_l2": err}


# Compulsory state traffic of one grid cell-step (FP64): the 14 Runge-Kutta
# fields (rho, momentum, energy, deviatoric stress, damage, tracer, vibration)
# read and written once, the fluidization ratio read once.
EULER_STEP_BYTES = 14 * 8 * 2 + 8


def euler_section(device, steps, warmup, N=256, cpu_n=64, acc_n=32, form=0, cpu=True, acc=True, e2e=True):
    """The Euler grid solver (hydrocodes/euler/hydro_cpu.cpp step_rk2) on the
    3-D half-space impact: N^3 cells of 50 m, basalt sphere at 30 deg, ROCK
    yield, tensile damage, gravity, near-void cells.  Device loop (dt on the
    device, steps replayed from a CUDA graph) timed with events; e2e through
    the C ABI with every field written from and read back to pinned host
    memory each step; the CPU oracle (the reference's algorithm, serial like
    the reference) on a cropped grid; rel-L2 against the oracle."""
    import torch
    from deorbit_gb300 import euler as E, grid_ic as GI
    from oracle import euler as EO

    case = GI.impact3d(N)
    g = E.from_case(case, device=device, form=form)
    g.run(case.cfl, case.t_end, max(warmup, 3))
    g.synchronize()
    l0 = g.launches()
    g.event_record(0)
    s, t = g.run(case.cfl, case.t_end, steps)
    g.event_record(1)
    ms = g.event_elapsed(0, 1)
    launches = g.launches() - l0
    # e2e: host buffers every step
    names = E.FIELDS
    el = None
    if e2e:
        host = {k: torch.empty(case.n, dtype=torch.float64).pin_memory().numpy() for k in names}
        g.read_many(names, [host[k] for k in names])
        t0 = time.perf_counter()
        for _ in range(steps):
            g.write_many(host)
            g.run(case.cfl, case.t_end, 1)
            g.read_many(names, [host[k] for k in names])
        el = time.perf_counter() - t0
    g.close()
    nbytes = len(names) * 8 * case.n
    hbm, hbm_kind = peaks()
    value = case.n * s / (ms / 1000.0)
    out = {"workload": f"3-D half-space impact, {N}^3 cells of 50 m, basalt sphere r = {N // 16} cells at 30 deg, "
                       "8 km/s; ROCK yield, tensile damage, gravity 3.71, near-void < 100 kg/m^3",
           "cells": case.n, "steps": s, "ms_per_step": ms / max(s, 1), "value": value, "unit": "cell-steps/s",
           "form": "mixed (FP32 fluxes and sources, FP64 state)" if form else "fp64 (reference operation order)",
           "dtype": "f32+f64" if form else "f64", "gpu_launches": launches,
           "e2e": None if el is None else {"value": case.n * steps / el, "unit": "cell-steps/s",
                                           "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                                           "pinned_host": True},
           "step_roofline": {"alg_bytes_per_cell_step": EULER_STEP_BYTES,
                             "achieved_gbs": EULER_STEP_BYTES * value / 1e9,
                             "frac": EULER_STEP_BYTES * value / 1e9 / hbm, "peak_kind": f"{hbm_kind} copy bandwidth"}}
    if cpu:  # CPU oracle on a smaller grid of the same workload (serial, as the reference)
        small = GI.impact3d(cpu_n)
        o = EO.from_case(small)
        o.run(small.cfl, small.t_end, 1)
        t0 = time.perf_counter()
        so, _ = o.run(small.cfl, small.t_end, 2)
        el = time.perf_counter() - t0
        o.close()
        out["cpu_baseline"] = {"value": small.n * so / el, "unit": "cell-steps/s", "cores": 1, "kind": "port",
                               "sample": f"the same impact on {cpu_n}^3 cells, {so} steps after one warm-up step"}
    if not acc:
        return out
    # parity on a small grid of the same workload
    acc = GI.impact3d(acc_n)
    keys = ("r", "mu", "mw", "E", "Sxx", "Sxy", "D")
    a = E.from_case(acc, device=device, form=form)
    a.run(acc.cfl, acc.t_end, 10)
    got = {k: a.read(k) for k in keys}
    a.close()
    o = EO.from_case(acc)
    o.run(acc.cfl, acc.t_end, 10)
    out["vs_oracle_rel_l2"] = {k: float(np.linalg.norm(got[k] - o.field(k)) / max(np.linalg.norm(o.field(k)), 1e-300))
                               for k in keys}
    out["vs_oracle_sample"] = f"{acc_n}^3 cells, 10 steps"
    o.close()
    return out


def crater_visc_section(device, steps=20, warmup=3, cpu_steps=3):
    """The reference driver's crater mode at its default size (hydro_cpu.cpp:
    557-597: a = 500 m, U = 12 km/s, 5 cells per radius, a 30 x 22 radii
    cylindrical domain) with shock-activated fluidization and the implicit
    fluidization viscosity (its argument 16; eta = 1e9 Pa s): device time per
    step of both forms (steps issued directly: the viscosity's cooperative
    launch is not replayed from a graph), conjugate-gradient iterations per
    step, and the serial CPU oracle on the same grid."""
    from deorbit_gb300 import euler as E, grid_ic as GI
    from oracle import euler as EO

    case = GI.crater(cppr=5, Rfac=30.0, Zfac=22.0, tdec=2.0, eta_af=1e9, visc_imp=1)
    out = {"workload": f"axisymmetric crater, {case.shape[0]} x {case.shape[2]} cells of {case.dx:.0f} m, "
                       "12 km/s, fluidization with the implicit viscosity (eta 1e9 Pa s)", "cells": case.n}
    for form, name in ((E.FP64, "fp64"), (E.MIXED, "mixed")):
        g = E.from_case(case, device=device, form=form)
        g.run(case.cfl, case.t_end, warmup)
        g.synchronize()
        it0, l0 = g.visc_iters(), g.launches()
        g.event_record(0)
        s, _ = g.run(case.cfl, case.t_end, steps)
        g.event_record(1)
        ms = g.event_elapsed(0, 1)
        out[name] = {"ms_per_step": ms / max(s, 1), "value": case.n * s / (ms / 1000.0), "unit": "cell-steps/s",
                     "cg_iters_per_step": (g.visc_iters() - it0) / max(s, 1),
                     "gpu_launches_per_step": (g.launches() - l0) / max(s, 1)}
        g.close()
    o = EO.from_case(case)
    EO.run_case(o, case, warmup)
    t0 = time.perf_counter()
    so, _ = EO.run_case(o, case, cpu_steps)
    el = time.perf_counter() - t0
    o.close()
    out["cpu_baseline"] = {"value": case.n * so / el, "unit": "cell-steps/s", "ms_per_step": 1e3 * el / so,
                           "cores": 1, "kind": "port", "sample": f"the same crater, {so} steps after {warmup}"}
    return out


def crater_sweep_section(device, tend=3.0, form=0):
    """The crater mode as a parameter sweep (impactor radius 300-600 m x speed
    8 / 12 km/s at the mode's default domain of 30 x 22 radii and 5 cells per
    radius, fixed end time): one run alone, then all eight at once through
    crater.run_many (a grid, stream and host thread each).  Wall-clock times
    of the whole driver loop, host measurements included."""
    from deorbit_gb300 import crater

    def setups():
        return [crater.setup(a=a, U=U, tend=tend) for a in (300.0, 400.0, 500.0, 600.0) for U in (8000.0, 12000.0)]

    one = setups()[5]
    crater.run(crater.setup(a=one.a, U=one.U, tend=0.2), form=form, device=device)  # warm-up: library, graphs
    t0 = time.perf_counter()
    r1 = crater.run(one, form=form, device=device)
    el1 = time.perf_counter() - t0
    sts = setups()
    t0 = time.perf_counter()
    res = crater.run_many(sts, form=form, device=device)
    el = time.perf_counter() - t0
    cell_steps = sum(st.case.n * r["steps"] for st, r in zip(sts, res))
    single = one.case.n * r1["steps"] / el1
    return {"workload": f"crater mode sweep: a 300-600 m x U 8 / 12 km/s, default domain, t_end {tend} s, "
                        + ("mixed" if form else "fp64") + " form",
            "runs": len(sts), "cells": [st.case.n for st in sts], "steps": [r["steps"] for r in res],
            "alone": {"cells": one.case.n, "steps": r1["steps"], "wall_s": el1, "value": single,
                      "unit": "cell-steps/s"},
            "concurrent": {"wall_s": el, "value": cell_steps / el, "unit": "cell-steps/s",
                           "speedup_vs_alone": cell_steps / el / single}}


def serving_section(device, rates=(4.0, 8.0, 16.0), count=200, steps=300):
    """Poisson request streams through the continuous-batching server."""
    from deorbit_gb300 import serve, sph
    out = {"workload": f"{count} requests per rate, N log-uniform 10k-500k, half strength + damage, "
                       f"{steps} steps each, 160 GB admission budget", "rates": []}
    for rate in rates:
        reqs = serve.poisson_requests(count, rate, steps=steps)
        srv = serve.Server(sph.MIXED, device, hbm_budget_bytes=160e9, chunk=4)
        from deorbit_gb300 import autotune
        autotune.apply(srv.ctx, reqs[0][1], sph.MIXED, device)
        base = srv.now()
        for t, sc, st in reqs:
            srv.submit(sc, st, arrival=base + t)
        srv.serve(timeout=900)
        rep = srv.report()
        srv.close()
        rep["rate_per_s"] = rate
        out["rates"].append(rep)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="grazing", choices=["grazing", "halfspace"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="particles of the CPU legs (0: the whole workload)")
    ap.add_argument("--acc-sample", type=int, default=1 << 17,
                    help="particles of the accuracy-vs-oracle sample")
    ap.add_argument("--acc-steps", type=int, default=10)
    ap.add_argument("--no-acc", action="store_true")
    ap.add_argument("--force-staging", type=int, default=None,
                    help="mixed form: force-pass record staging (engine option force_staging)")
    ap.add_argument("--host-direct", type=int, default=None,
                    help="mixed form: 1 lets kernels reach host field buffers directly over the "
                         "CPU-GPU link (engine option host_direct; default: device staging copies)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-halfspace", action="store_true")
    ap.add_argument("--no-euler", action="store_true")
    ap.add_argument("--euler-n", type=int, default=256)
    ap.add_argument("--only-euler", action="store_true",
                    help="run only the Euler grid section (both forms) and print its JSON")
    args = ap.parse_args()
    rank, world, local = rank_info()
    if args.only_euler:
        out = {f: euler_section(local, args.steps, args.warmup, args.euler_n, form=i, cpu=not args.no_cpu,
                                acc=not args.no_acc, e2e=not args.no_e2e)
               for i, f in enumerate(("fp64", "mixed"))}
        out["crater_visc"] = crater_visc_section(local)
        out["crater_sweep"] = crater_sweep_section(local)
        print(json.dumps(out), flush=True)
        return

    from deorbit_gb300 import ic

    sc = workload(args.workload, args.n)
    sample_n = min(args.cpu_sample, sc.n) if args.cpu_sample > 0 else sc.n
    wl = {"workload": f"{args.workload} impact, strength+damage" if args.workload == "grazing"
          else "halfspace impact, hydro only", "n_particles": sc.n, "dx_m": sc.dx,
          "materials": "granite (Collins, multi-flaw) + iron (von Mises)" if args.workload == "grazing"
          else "granite + iron, hydro only", "l2": "working set > 129 MB L2 (no flush needed)"}

    if args.impl == "reference":
        # the reference's own CPU path is the oracle port here (the reference
        # tree is not on this machine); rank 0 only
        if rank != 0:
            return
        from oracle import oracle as O

        sample = ic.crop(sc, sample_n)
        t_init = time.perf_counter()
        S = O.from_scenario(sample, threads=min(os.cpu_count() or 1, 16))
        S.init()
        t_init = time.perf_counter() - t_init
        for _ in range(args.warmup):
            S.step(S.timestep())
        t0 = time.perf_counter()
        for _ in range(args.steps):
            S.step(S.timestep())
        el = time.perf_counter() - t0
        v = sample.n * args.steps / el
        what = (f"the whole {sc.n}-particle workload" if sample.n == sc.n else
                f"{sample.n} particles cropped from the {sc.n}-particle workload around the impact point")
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": dict(wl, sample=sample.n),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": S.threads(), "nproc": os.cpu_count(),
                                 "kind": "port",
                                 "sample": f"{what}, {args.steps} KDK steps after init and {args.warmup} "
                                           f"warm-up steps (init {t_init:.1f} s)"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    from deorbit_gb300 import sph

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- mixed form (headline)
    barrier()
    with ClockSampler(device) as clk:
        opts = {} if args.force_staging is None else {"force_staging": args.force_staging}
        if args.host_direct is not None:
            opts["host_direct"] = args.host_direct
        ctx, b, ms, kst, launches = time_form(sph, ic, sc, sph.MIXED, args.steps, args.warmup, device, opts)
    list_entries = ctx.get_option("list_entries")
    barrier()
    ms = max_over_ranks(ms)
    value = world * sc.n * args.steps / (ms / 1000.0)

    # ---- e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        r, el, nbytes, pinned = e2e_rate(sph, ctx, b, sc.n, args.steps, min(args.warmup, 2))
        el = max_over_ranks(el)
        _, el_sep, _, _ = e2e_rate(sph, ctx, b, sc.n, args.steps, min(args.warmup, 2), fused=False)
        el_sep = max_over_ranks(el_sep)
        e2e = {"value": world * sc.n * args.steps / el, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes + 8, "pinned_host": pinned,
               "api": "sph_step_fields (one call per step; copies overlap the step)",
               "separate_calls": {"value": world * sc.n * args.steps / el_sep,
                                  "api": "sph_write_fields + sph_timestep + sph_step + sph_read_fields",
                                  "host_path": "direct (kernels over the CPU-GPU link)"
                                  if ctx.get_option("host_direct") else "device staging copies"}}
    ctx.close()

    # ---- plain FP64 form
    c64, b64, ms64, kst64, _ = time_form(sph, ic, sc, sph.FP64, args.steps, args.warmup, device)
    c64.close()
    ms64 = max_over_ranks(ms64)
    value64 = world * sc.n * args.steps / (ms64 / 1000.0)

    # ---- batched sweep and serving streams (rank 0 of a replica run)
    batched = serving = None
    if rank == 0 and not args.no_batch:
        batched = batched_section(sph, ic, device, args.steps, args.warmup, args.batch_count)
    if rank == 0 and not args.no_serve:
        serving = serving_section(device)
    large = None
    if rank == 0 and not args.no_large:
        large = large_section(sph, ic, device, args.steps, args.warmup)
    halfspace = None
    if rank == 0 and world == 1 and not args.no_halfspace:
        halfspace = halfspace_section(sph, ic, device)
    euler = None
    if rank == 0 and world == 1 and not args.no_euler:
        euler = {"fp64": euler_section(device, args.steps, args.warmup, args.euler_n),
                 "mixed": euler_section(device, args.steps, args.warmup, args.euler_n, form=1, cpu=False),
                 "crater_visc": crater_visc_section(device),
                 "crater_sweep": crater_sweep_section(device)}

    # ---- accuracy of the mixed form against FP64 (same dt sequence), and of
    # both forms against the oracle on a bounded sample
    err = mixed_error(sph, ic, sc, args.steps, device) if rank == 0 else None
    acc = None
    if rank == 0 and not args.no_acc:
        acc = accuracy_vs_oracle(sph, ic, ic.crop(sc, min(args.acc_sample, sc.n)), args.acc_steps, device)

    # ---- roofline of the dominant mixed-form kernel (largest total time of
    # the classes that hold one kernel; per-launch time from CUDA events)
    hbm, hbm_kind = peaks()
    dom = max((k for k in kst if k in KERNEL_OF_CLASS), key=lambda k: kst[k][0])
    tot_ms, nl = kst[dom]
    avg_ms = tot_ms / max(nl, 1)
    fixed, per_entry = ALG_BYTES[dom]
    alg = fixed + per_entry * list_entries / sc.n
    achieved = alg * sc.n / (avg_ms / 1000.0) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if os.path.exists(tfile):
        for line in open(tfile):
            f = line.split()
            if len(f) >= 4 and not line.startswith("#") and f[0] == KERNEL_OF_CLASS[dom] + "_mixed":
                # bytes per particle measured on a smaller case, scaled to this launch
                traffic = (float(f[2]) + float(f[3])) * sc.n / float(f[1])
    fp32 = None
    clocks = clk.summary()
    if dom in FLOPS_PER_ENTRY:
        iters = 2 if dom == "density" else 1
        fl = FLOPS_PER_ENTRY[dom] * list_entries * iters
        tf = fl / (avg_ms / 1000.0) / 1e12
        mhz = clocks.get("sm_max_mhz") or 2070.0
        peak32, sms = fp32_peak_tflops(device, mhz)
        fp32 = {"flops_per_launch": fl, "achieved_tflops": tf, "peak_tflops": peak32,
                "peak_kind": f"{sms} SMs x {FP32_LANES_PER_SM} lanes x 2 x {mhz:.0f} MHz (device properties and "
                             f"the sampled maximum SM clock)", "frac": tf / peak32}
    roof = {"kernel": KERNEL_OF_CLASS[dom] + "<float>", "bound": "hbm", "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
            "peak_kind": f"{hbm_kind} copy bandwidth", "alg_bytes_per_launch": alg * sc.n,
            "alg_bytes_per_particle": alg, "list_entries_per_particle": list_entries / sc.n,
            "avg_launch_ms": avg_ms, "launches": nl, "fp32_issue": fp32}
    step_bytes = STEP_BYTES[4] * sc.n
    step_roof = {"alg_bytes_per_particle_step": STEP_BYTES[4],
                 "achieved_gbs": step_bytes / (ms / args.steps / 1000.0) / 1e9}
    step_roof["frac"] = step_roof["achieved_gbs"] / hbm

    # ---- CPU baseline (rank 0, N = 1): oracle on a cropped sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sample = ic.crop(sc, sample_n)
        v, el, thr = cpu_rate(ic, sample, 2, threads=min(os.cpu_count() or 1, 16))
        what = (f"the whole {sc.n}-particle workload" if sample.n == sc.n else
                f"{sample.n} particles cropped from the {sc.n}-particle workload around the impact point")
        cpu = {"value": v, "unit": UNIT, "cores": thr, "nproc": os.cpu_count(), "kind": "port",
               "sample": f"{what}, 2 KDK steps after init ({el:.1f} s)",
               "plain_fp64_gpu_over_cpu": value64 / v, "mixed_gpu_over_cpu": value / v}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": dict(wl, form="mixed (FP32 pairs/EOS/stress, FP64 positions/energies)",
                               parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
                "roofline": roof, "step_roofline": step_roof, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clocks,
                "plain_fp64": {"value": value64, "ms_per_step": ms64 / args.steps,
                               "kernel_ms": {k: v[0] for k, v in kst64.items()}},
                "speedup_vs_plain_fp64": value / value64,
                "mixed_vs_fp64_rel_l2": err,
                "accuracy_vs_oracle": acc,
                "kernel_ms": {k: v[0] for k, v in kst.items()},
                "batched": batched, "serving": serving, "large": large, "halfspace": halfspace,
                "euler": euler}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
