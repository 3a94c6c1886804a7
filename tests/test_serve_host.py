"""Host logic of the native continuous-batching server (sph_serve_* in
libdeorbit_sph.so, deorbit_gb300/csrc/serve.cpp) on the CPU: FIFO admission
under the device-memory budget, an oversized request served alone, arrival
times, chunks that never overshoot a step limit, retirement with results kept
in host memory, release, the latency report, and flaw seeding on the server's
worker thread -- driven by tests/serve_harness.cpp against a stand-in engine
that counts steps (the GPU path itself is covered by tests/test_gpu_serving.py)."""
import os
import subprocess

import numpy as np
import pytest

from deorbit_gb300 import serve

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "deorbit_gb300", "_lib")


@pytest.fixture(scope="module")
def harness(cuda_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("serve") / "serve_harness")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "deorbit_gb300", "csrc"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "serve_harness.cpp"), "-o", exe, "-L", LIBDIR, "-ldeorbit_sph",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    def run(case):
        p = subprocess.run([exe, case], capture_output=True, text=True, timeout=60)
        assert p.returncode == 0, p.stdout + p.stderr
        return {line.split()[0]: line.split()[1:] for line in p.stdout.splitlines() if line.strip()}
    return run


def test_fifo_admission_within_budget(harness):
    o = harness("fifo")
    # two of three 1000-particle requests fit the 2500-particle budget
    assert o["after_first_poll"][:3] == ["1", "1", "0"] and o["resident"] == ["2"]
    assert o["order"] == ["0", "1", "2"] and o["third_admitted_after"] == ["1"]


def test_oversized_request_runs_alone(harness):
    o = harness("oversized")
    assert o["after_first_poll"] == ["2", "0"]   # larger than the budget: admitted alone, the next waits
    assert o["small_after_big"] == ["1"]


def test_step_limits_and_chunks(harness):
    o = harness("chunks")
    # chunks never overshoot the nearest limit: 4, 1 (first done), 4 (second done)
    assert o["runs"] == ["4", "1", "4"]
    assert o["particle_steps"] == [str(100 * 4 * 2 + 100 * 1 * 2 + 100 * 4)]
    assert o["done"] == ["2"] and o["residents_left"] == ["0"]   # every impact released
    assert o["result_fields"] == ["0", "1"]   # kept fields read back in host memory
    assert o["unkept_field_rc"] == ["-1"] and o["released_rc"] == ["-1"]


def test_future_arrivals_wait_for_the_clock(harness):
    o = harness("future")
    assert o["not_yet"] == ["0"] and o["runs"] == ["0"]
    assert o["admitted_after_arrival"] == ["1"] and o["done"] == ["1"] and o["p50_nonneg"] == ["1"]
    assert o["particle_steps"] == ["200"]


def test_flaws_seeded_before_admission(harness):
    o = harness("seeding")
    # multi-flaw: ceil(N ln N) thresholds for 500 particles; single: eps_act only
    assert o["flaws"] == [str(int(np.ceil(500 * np.log(500)))), "0"]


def test_poisson_stream_shape():
    reqs = serve.poisson_requests(16, rate_per_s=4.0, n_lo=2000, n_hi=4000, steps=5)
    t = [a for a, _, _ in reqs]
    assert all(np.diff(t) > 0) and len(reqs) == 16
    assert all(1500 <= sc.n <= 5000 for _, sc, _ in reqs)
    assert all(steps == 5 for _, _, steps in reqs)
