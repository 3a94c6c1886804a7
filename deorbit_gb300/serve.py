"""Continuous-batching server for impact runs on one GPU.

Requests (a Scenario and a step count) arrive over time.  The server keeps one
engine context; a request is admitted as soon as its particles fit the HBM
budget next to the resident ones, initialised in place while the others keep
their state, then advanced together with every other resident impact -- one
kernel launch per phase covers all of them, each with its own CFL dt and step
limit.  A finished request's fields are read back and its slot and memory
released, which admits the next one.  Results of a request do not depend on
what else is resident (all per-particle work is confined to the particle's own
impact and reductions are order-independent), so a request gives the same
result alone and in the mix.

Latency is measured from arrival (submit time) to the moment its results are
in host memory.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np

from . import ic, sph

# Device bytes per resident particle of the mixed form at the default list
# capacity (carried state double-buffered, derived fields, geometry, lists,
# sort buffers); the FP64 form needs about 1.6x.
BYTES_PER_PARTICLE = {sph.MIXED: 1500, sph.FP64: 2400}

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

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


class Server:
    def __init__(self, precision=sph.MIXED, device=0, hbm_budget_bytes=160e9, chunk=4,
                 fields=RESULT_FIELDS, bytes_per_particle=None, ctx=None):
        self.precision = precision
        # ctx: an engine context to serve from (default: a new one on `device`)
        self.ctx = ctx if ctx is not None else sph.Context(precision, device)
        self.budget = float(hbm_budget_bytes)
        self.bpp = bytes_per_particle or BYTES_PER_PARTICLE[precision]
        self.chunk = int(chunk)
        self.fields = fields
        self.pending = collections.deque()
        self.active = {}
        self.done = []
        self.mat_ids = {}
        self.t0 = time.perf_counter()
        self.particle_steps = 0
        self.busy_time = 0.0

    # ------------------------------------------------------------ clock
    def now(self):
        return time.perf_counter() - self.t0

    # ------------------------------------------------------------ requests
    def submit(self, scenario: ic.Scenario, steps: int, arrival: float | None = None) -> Request:
        r = Request(len(self.pending) + len(self.active) + len(self.done), scenario, int(steps),
                    self.now() if arrival is None else float(arrival))
        self.pending.append(r)
        return r

    def resident_particles(self):
        return sum(r.scenario.n for r in self.active.values())

    def _admit(self, now):
        admitted = []
        while self.pending and self.pending[0].arrival <= now:
            r = self.pending[0]
            need = (self.resident_particles() + r.scenario.n) * self.bpp
            if self.active and need > self.budget:
                break  # wait for memory to free up (FIFO admission)
            self.pending.popleft()
            b = ic.to_context(self.ctx, r.scenario, material_ids=self.mat_ids)
            self.ctx.set_step_limit(b, r.steps)
            r.impact = b
            r.admitted = now
            self.active[b] = r
            admitted.append(r)
        if admitted:
            self.ctx.init()  # initialises only the newly admitted impacts
        return admitted

    def _retire(self):
        finished = []
        for b, r in list(self.active.items()):
            if self.ctx.info(b).steps >= r.steps:
                r.result = {k: self.ctx.read(b, k) for k in self.fields}
                r.finished = self.now()
                self.ctx.remove(b)
                del self.active[b]
                self.done.append(r)
                finished.append(r)
        return finished

    def step(self):
        """Admit what has arrived, advance all residents by one chunk, retire."""
        self._admit(self.now())
        if not self.active:
            return 0
        steps = min(self.chunk, min(r.steps - self.ctx.info(b).steps for b, r in self.active.items()))
        steps = max(steps, 1)
        n = self.resident_particles()
        t = time.perf_counter()
        self.ctx.run(steps)
        self.ctx.synchronize()
        self.busy_time += time.perf_counter() - t
        self.particle_steps += n * steps
        self._retire()
        return steps

    def serve(self, timeout=None):
        """Run until every submitted request is done (requests with future
        arrival times are admitted when the clock reaches them)."""
        while self.pending or self.active:
            if timeout is not None and self.now() > timeout:
                raise TimeoutError("serving did not drain in time")
            if not self.active and self.pending and self.pending[0].arrival > self.now():
                time.sleep(min(0.01, self.pending[0].arrival - self.now()))
                continue
            self.step()
        return self.done

    def report(self):
        lat = np.array([r.latency for r in self.done if r.latency is not None])
        wall = max((r.finished for r in self.done), default=0.0) - min((r.arrival for r in self.done), default=0.0)
        return {
            "requests": len(self.done),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "mean_latency_s": float(lat.mean()) if lat.size else None,
            "throughput_particle_steps_per_s": self.particle_steps / wall if wall > 0 else None,
            "gpu_busy_particle_steps_per_s": self.particle_steps / self.busy_time if self.busy_time else None,
            "particle_steps": self.particle_steps,
        }

    def close(self):
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
