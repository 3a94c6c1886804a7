"""Host logic of the continuous-batching server (deorbit_gb300/serve.py) on the
CPU: FIFO admission under the HBM budget, arrival times, step limits, retirement
and the latency report -- against a stand-in engine context that counts steps
(the GPU path itself is covered by tests/test_gpu_serving.py)."""
import types

import numpy as np
import pytest

from deorbit_gb300 import ic, serve


class CountingContext:
    """Counts steps per impact the way the engine's step limits do."""

    def __init__(self):
        self.impacts = {}
        self.next_id = 0
        self.inits = 0
        self.runs = []

    def add(self, n):
        b = self.next_id
        self.next_id += 1
        self.impacts[b] = {"n": n, "steps": 0, "limit": 0}
        return b

    def set_step_limit(self, b, steps):
        self.impacts[b]["limit"] = steps

    def init(self):
        self.inits += 1

    def run(self, steps):
        self.runs.append((steps, sorted(self.impacts)))
        for d in self.impacts.values():
            d["steps"] = min(d["limit"], d["steps"] + steps)

    def synchronize(self):
        pass

    def info(self, b):
        return types.SimpleNamespace(steps=self.impacts[b]["steps"])

    def read(self, b, name):
        return np.zeros(self.impacts[b]["n"])

    def remove(self, b):
        del self.impacts[b]

    def close(self):
        pass


@pytest.fixture
def server(monkeypatch):
    ctx = CountingContext()
    monkeypatch.setattr(ic, "to_context", lambda c, sc, material_ids=None: c.add(sc.n))
    srv = serve.Server(ctx=ctx, hbm_budget_bytes=2500 * 100, bytes_per_particle=100, chunk=4)
    return srv, ctx


def scenario(n):
    return types.SimpleNamespace(n=n)


def test_fifo_admission_within_budget(server):
    srv, ctx = server
    a = srv.submit(scenario(1000), 6, arrival=0.0)
    b = srv.submit(scenario(1000), 6, arrival=0.0)
    c = srv.submit(scenario(1000), 6, arrival=0.0)   # 3000 particles > the 2500 budget
    srv.step()
    assert a.admitted is not None and b.admitted is not None and c.admitted is None
    assert set(ctx.impacts) == {a.impact, b.impact}
    srv.serve(timeout=10.0)
    assert c.admitted is not None and c.admitted >= max(a.finished, b.finished)
    assert [r.rid for r in srv.done] == [0, 1, 2]


def test_oversized_request_runs_alone(server):
    srv, ctx = server
    big = srv.submit(scenario(10_000), 3, arrival=0.0)   # larger than the whole budget
    small = srv.submit(scenario(10), 3, arrival=0.0)
    srv.step()
    assert big.admitted is not None and small.admitted is None
    srv.serve(timeout=10.0)
    assert small.admitted >= big.finished


def test_step_limits_and_chunks(server):
    srv, ctx = server
    r1 = srv.submit(scenario(100), 5, arrival=0.0)
    r2 = srv.submit(scenario(100), 9, arrival=0.0)
    srv.serve(timeout=10.0)
    # chunks never overshoot the nearest limit: 4, 1 (r1 done), 4 (r2 done)
    assert [s for s, _ in ctx.runs] == [4, 1, 4]
    assert srv.particle_steps == 100 * 4 * 2 + 100 * 1 * 2 + 100 * 4
    assert r1.result is not None and set(r1.result) == set(serve.RESULT_FIELDS)
    assert not ctx.impacts  # every impact released


def test_future_arrivals_wait_for_the_clock(server):
    srv, ctx = server
    late = srv.submit(scenario(100), 2, arrival=srv.now() + 0.05)
    assert srv.step() == 0 and late.admitted is None
    srv.serve(timeout=10.0)
    assert late.admitted >= late.arrival
    rep = srv.report()
    assert rep["requests"] == 1 and rep["p50_latency_s"] >= 0.0 and rep["particle_steps"] == 200


def test_poisson_stream_shape():
    reqs = serve.poisson_requests(16, rate_per_s=4.0, n_lo=2000, n_hi=4000, steps=5)
    t = [a for a, _, _ in reqs]
    assert all(np.diff(t) > 0) and len(reqs) == 16
    assert all(1500 <= sc.n <= 5000 for _, sc, _ in reqs)
    assert all(steps == 5 for _, _, steps in reqs)
