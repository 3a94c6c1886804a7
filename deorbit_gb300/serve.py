"""Continuous-batching server for impact runs on one GPU (Python front end
of the library's native server, sph_serve_* in the C ABI).

Requests (a Scenario and a step count) arrive over time.  The server keeps one
engine context; a request is admitted as soon as it has arrived and its
particles fit the device-memory budget next to the resident ones -- judged from
the engine's own allocations and its per-particle footprint at the current
neighbour-list capacity, which grows when an impact compresses -- initialised in
place while the others keep their state, then advanced together with every
other resident impact: one kernel launch per phase covers all of them, each with
its own CFL dt and step limit.  A finished request's fields are read back and its
slot and memory released, which admits the next one.  Flaw seeding of queued
requests (the multi-flaw law draws ~N ln N thresholds) runs on the server's
worker thread while the GPU advances the residents.  Results of a request do
not depend on what else is resident (all per-particle work is confined to the
particle's own impact and reductions are order-independent), so a request gives
the same result alone and in the mix.

Latency is measured from arrival (submit time) to the moment its results are
in host memory.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time

import numpy as np

from . import ic, sph

RESULT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "u", "rho", "P", "D")


@dataclasses.dataclass
class Request:
    rid: int
    scenario: ic.Scenario
    steps: int
    arrival: float            # seconds since the server clock started
    admitted: float | None = None
    finished: float | None = None
    impact: int | None = None
    result: dict | None = None
    failed: bool = False

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Server:
    def __init__(self, precision=sph.MIXED, device=0, hbm_budget_bytes=160e9, chunk=4,
                 fields=RESULT_FIELDS, ctx=None):
        self.precision = precision
        # ctx: an engine context to serve from (default: a new one on `device`)
        self.ctx = ctx if ctx is not None else sph.Context(precision, device)
        self.fields = tuple(fields)
        self.h = C.c_void_p()
        sph.check(sph.lib().sph_serve_create(self.ctx.h, float(hbm_budget_bytes), int(chunk),
                                             ",".join(self.fields).encode(), C.byref(self.h)))
        self.requests = {}
        self.done = []
        self.mat_ids = {}

    # ------------------------------------------------------------ clock
    def now(self):
        t = C.c_double()
        sph.check(sph.lib().sph_serve_now(self.h, C.byref(t)))
        return t.value

    # ------------------------------------------------------------ requests
    def submit(self, scenario: ic.Scenario, steps: int, arrival: float | None = None) -> Request:
        sc = scenario
        ids = []
        for d in sc.materials:  # materials are added to the context once and shared
            key = tuple(sorted(d.items()))
            if key not in self.mat_ids:
                self.mat_ids[key] = self.ctx.add_material(ic._material_struct(sph.Material, d))
            ids.append(self.mat_ids[key])
        mat = np.ascontiguousarray(np.asarray(ids if ids else [0], np.int32)[sc.mat])
        prm = sph.params(**sc.params)
        keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in (
            ("x", sc.pos[:, 0]), ("y", sc.pos[:, 1]), ("z", sc.pos[:, 2]), ("vx", sc.vel[:, 0]),
            ("vy", sc.vel[:, 1]), ("vz", sc.vel[:, 2]), ("mass", sc.mass), ("u", sc.u))}
        fixed = np.ascontiguousarray(sc.fixed, dtype=np.uint8)
        q = sph.Request()
        q.params = C.pointer(prm)
        for a in range(3):
            q.lo[a], q.hi[a], q.periodic[a] = float(sc.lo[a]), float(sc.hi[a]), int(sc.periodic[a])
        q.n = sc.n
        for k, v in keep.items():
            setattr(q, k, _dp(v))
        q.mat = mat.ctypes.data_as(C.POINTER(C.c_int32))
        q.fixed = fixed.ctypes.data_as(C.POINTER(C.c_uint8))
        h0 = None
        if sc.h0 is not None:
            h0 = np.ascontiguousarray(sc.h0, dtype=np.float64)
            q.h0 = _dp(h0)
        kind, seed = sc.flaws if sc.flaws is not None else (None, 0)
        q.flaws = sph.SERVE_FLAWS[kind]
        q.flaw_dx, q.flaw_seed = float(sc.dx), int(seed) & 0xffffffff
        q.steps = int(steps)
        q.arrival = -1.0 if arrival is None else float(arrival)
        rid = C.c_int64()
        sph.check(sph.lib().sph_serve_submit(self.h, C.byref(q), C.byref(rid)))  # copies the arrays
        rec = sph.ServeRecord()
        sph.check(sph.lib().sph_serve_request_info(self.h, rid.value, C.byref(rec)))
        r = Request(rid.value, sc, int(steps), rec.arrival)
        self.requests[r.rid] = r
        return r

    def _collect(self, rid):
        r = self.requests[rid]
        rec = sph.ServeRecord()
        sph.check(sph.lib().sph_serve_request_info(self.h, rid, C.byref(rec)))
        r.admitted, r.finished, r.impact = rec.admitted, rec.finished, rec.impact
        if rec.state == sph.SERVE_DONE:
            r.result = {}
            for k in self.fields:
                out = np.empty(r.scenario.n)
                sph.check(sph.lib().sph_serve_result(self.h, rid, k.encode(), _dp(out)))
                r.result[k] = out
        else:
            r.failed = True
        sph.check(sph.lib().sph_serve_release(self.h, rid))
        self.done.append(r)

    def step(self, max_wait_s=0.01):
        """One serving round: admit what has arrived, advance the residents by
        one chunk, retire; returns the requests finished in this round."""
        cap = 256
        ids = (C.c_int64 * cap)()
        nd = C.c_int32()
        sph.check(sph.lib().sph_serve_poll(self.h, float(max_wait_s), ids, cap, C.byref(nd)))
        fin = [ids[i] for i in range(min(nd.value, cap))]
        for rid in fin:
            self._collect(rid)
        return [self.requests[rid] for rid in fin]

    def serve(self, timeout=None):
        """Run until every submitted request is done (requests with future
        arrival times are admitted when the clock reaches them)."""
        t0 = time.perf_counter()
        while len(self.done) < len(self.requests):
            if timeout is not None and time.perf_counter() - t0 > timeout:
                raise TimeoutError("serving did not drain in time")
            self.step()
            for rid, r in self.requests.items():  # requests the server could not prepare
                if r.finished is None and not r.failed:
                    rec = sph.ServeRecord()
                    sph.check(sph.lib().sph_serve_request_info(self.h, rid, C.byref(rec)))
                    if rec.state == sph.SERVE_FAILED:
                        self._collect(rid)
        return self.done

    def report(self):
        st = sph.ServeSummary()
        sph.check(sph.lib().sph_serve_stats(self.h, C.byref(st)))
        return {
            "requests": int(st.done),
            "p50_latency_s": st.p50_latency_s if st.done else None,
            "p99_latency_s": st.p99_latency_s if st.done else None,
            "mean_latency_s": st.mean_latency_s if st.done else None,
            "throughput_particle_steps_per_s": st.throughput or None,
            "gpu_busy_particle_steps_per_s": st.busy_throughput or None,
            "particle_steps": st.particle_steps,
            "peak_device_bytes": st.peak_device_bytes,
            "admit_wait_s": st.admit_wait_s,
            "host_s": st.host_s,
        }

    def close(self):
        if self.h:
            sph.check(sph.lib().sph_serve_destroy(self.h))
            self.h = C.c_void_p()
        self.ctx.close()


def poisson_requests(count, rate_per_s, seed=20261203, n_lo=10_000, n_hi=500_000, steps=300):
    """Request stream: log-uniform sizes, half hydro-only and half strength +
    damage, angle U[1, 10] deg, speed U[6, 10] km/s, Poisson arrival times."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), size=count)).astype(int)
    out = []
    for i in range(count):
        strength = bool(i % 2)
        sc = ic.sized_impact(int(sizes[i]), seed=int(seed + 17 * i), angle_deg=float(rng.uniform(1, 10)),
                             speed=float(rng.uniform(6000, 10000)), ratio=float(rng.uniform(0.1, 0.3)),
                             strength=strength)
        out.append((float(t[i]), sc, steps))
    return out
