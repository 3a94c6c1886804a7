"""Continuous batching: requests admitted while others run, by HBM budget, give
the same result alone and in the mix (bit-identical: per-particle work is
confined to its own impact and reductions are order-independent)."""
import numpy as np
import pytest

from deorbit_gb300 import ic

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(cuda_lib):
    """Through the native server (sph_serve_* of the C ABI): requests arriving
    while others run are admitted, advanced together and retired; each result is
    bit-identical to the same request run alone."""
    from deorbit_gb300 import serve, sph
    reqs = [ic.sized_impact(2500 + 1500 * i, seed=90 + i, angle_deg=5 + 3 * i, speed=7000 + 500 * i,
                            ratio=0.2, strength=bool(i % 2)) for i in range(4)]
    steps = [6, 9, 5, 7]
    srv = serve.Server(sph.MIXED, hbm_budget_bytes=160e9, chunk=2)
    for i, (sc, st) in enumerate(zip(reqs, steps)):
        srv.submit(sc, st, arrival=0.0 if i < 2 else 0.01 * i)
    done = srv.serve(timeout=120)
    rep = srv.report()
    srv.close()
    assert rep["requests"] == 4 and rep["p99_latency_s"] >= rep["p50_latency_s"] > 0
    assert rep["peak_device_bytes"] > 0
    by_id = {r.rid: r for r in done}
    # overlap happened: some request was admitted while another was resident
    adm = sorted((r.admitted, r.finished) for r in done)
    assert any(a2 < f1 for (a1, f1), (a2, f2) in zip(adm, adm[1:]))
    for i, (sc, st) in enumerate(zip(reqs, steps)):
        ctx = sph.Context(sph.MIXED)
        b = ic.to_context(ctx, sc)
        ctx.init()
        ctx.run(st)
        for k in serve.RESULT_FIELDS:
            assert np.array_equal(ctx.read(b, k), by_id[i].result[k]), (i, k)
        ctx.close()


def test_serving_admits_by_device_bytes(cuda_lib):
    """Admission compares the engine's own device footprint with the budget: a
    budget that holds one request's allocations makes the second wait until the
    first has finished and released its memory."""
    from deorbit_gb300 import serve, sph
    reqs = [ic.sized_impact(3000, seed=70 + i, angle_deg=10, speed=7000, ratio=0.2) for i in range(2)]
    probe = sph.Context(sph.MIXED)
    b = ic.to_context(probe, reqs[0])
    probe.init()
    one = probe.get_option("device_bytes")
    bpp = probe.get_option("bytes_per_particle")
    probe.close()
    assert one > bpp * reqs[0].n > 0
    srv = serve.Server(sph.MIXED, hbm_budget_bytes=one * 1.02, chunk=2)
    r0 = srv.submit(reqs[0], 4, arrival=0.0)
    r1 = srv.submit(reqs[1], 4, arrival=0.0)
    srv.serve(timeout=120)
    srv.close()
    assert r1.admitted >= r0.finished


def test_replica_shards_equal_one_context(cuda_lib):
    """Splitting a batch across replicas changes nothing: each shard run in its
    own context gives bit-identical results to the whole batch in one."""
    from deorbit_gb300 import replicas
    scs = ic.batch_impacts(count=6, lo=1500, hi=4000)
    whole = replicas.gpu_runner(scs, 4)
    merged = {}
    for rank in range(2):
        merged.update(replicas.run_shard(scs, 4, rank, 2))
    assert sorted(merged) == list(range(len(scs)))
    for i, w in enumerate(whole):
        for k in w:
            assert np.array_equal(w[k], merged[i][k]), (i, k)
