"""Edge cases of the step loop on the GPU: empty impacts, neighbour-list
overflow (the consumers' traversal fallback and the capacity growth), a box
periodic on all three axes, a particle that leaves the domain (clamped bins,
sph.hpp:142-146), flattened traversal cells, and removing an impact in the
middle of a batch.  FP64 parity
with the oracle where the oracle applies (rel-L2 <= 1e-9), bit-identity with an
undisturbed run otherwise."""
import os

import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O

from parity import field_errors, read_all

pytestmark = pytest.mark.gpu

NAMES = ["x", "y", "z", "vx", "vy", "vz", "u", "rho", "hh", "P"]


def run_pair(sc, steps, **opts):
    from deorbit_gb300 import sph
    ctx = sph.Context(sph.FP64)
    for k, val in opts.items():
        ctx.set_option(k, val)
    b = ic.to_context(ctx, sc)
    orc = O.from_scenario(sc, threads=min(os.cpu_count() or 1, 16))
    ctx.init()
    orc.init()
    for _ in range(steps):
        dt = orc.timestep()
        assert abs(ctx.timestep(b) - dt) <= 1e-9 * dt
        orc.step(dt)
        ctx.step(dt)
    errs = field_errors(read_all(ctx, b, NAMES), {k: orc.field(k) for k in NAMES}, NAMES)
    info = ctx.info(b)
    cap = ctx.get_option("list_capacity")
    ctx.close()
    return errs, info, cap


def test_empty_impacts(cuda_lib):
    from deorbit_gb300 import sph
    sc = ic.sheared_cube(L=6)
    ctx = sph.Context(sph.MIXED)
    e0 = ctx.impact_create(sph.params(h_init=1.3 * sc.dx), sc.lo, sc.hi)
    b = ic.to_context(ctx, sc)
    e1 = ctx.impact_create(sph.params(h_init=1.3 * sc.dx), sc.lo, sc.hi)
    ctx.init()
    ctx.run(3)
    ctx.step(ctx.timestep(b))
    got = read_all(ctx, b, NAMES)
    assert ctx.n(e0) == 0 and ctx.n(e1) == 0
    ctx.close()
    alone = sph.Context(sph.MIXED)
    b1 = ic.to_context(alone, sc)
    alone.init()
    alone.run(3)
    alone.step(alone.timestep(b1))
    ref = read_all(alone, b1, NAMES)
    alone.close()
    for k in NAMES:
        assert np.array_equal(got[k], ref[k]), k
    only_empty = sph.Context(sph.FP64)
    only_empty.impact_create(sph.params(h_init=1.0), (0, 0, 0), (1, 1, 1))
    only_empty.init()
    only_empty.run(2)
    only_empty.close()


def test_list_overflow_matches_oracle(cuda_lib, oracle_lib):
    """eta 2.6: ~600 neighbours per particle, far past the default list
    capacity (160): the first steps take the traversal fallback, the capacity
    then grows; results stay those of the oracle."""
    sc = ic.sheared_cube(L=8)
    sc.params = dict(sc.params, eta=2.6, h_init=2.6 * sc.dx)
    errs, info, cap = run_pair(sc, 3)
    assert max(errs.values()) < 1e-9, errs
    assert cap > 160


def test_fully_periodic_box_matches_oracle(cuda_lib, oracle_lib):
    n, dx = 9, 1.0
    rng = np.random.default_rng(5)
    pos = ic.lattice(n, n, n, dx) + rng.uniform(-0.05, 0.05, size=(n ** 3, 3))
    vel = rng.normal(0.0, 30.0, size=(n ** 3, 3))
    mats = [ic.basalt()]
    sc = ic.Scenario("periodic_box", pos, vel, np.full(n ** 3, mats[0]["rho0"] * dx ** 3),
                     np.full(n ** 3, 1.0e5), np.zeros(n ** 3, np.int32), np.zeros(n ** 3, np.uint8),
                     np.zeros(3), np.full(3, n * dx), np.ones(3, np.int32),
                     dict(eta=1.3, h_init=1.3 * dx, eps_as=0.3), mats, dx)
    errs, _, _ = run_pair(sc, 6)
    assert max(errs.values()) < 1e-9, errs


def test_escaping_particle_matches_oracle(cuda_lib, oracle_lib):
    """A particle shot out of the domain: its bins clamp to the border cells,
    as in the reference's binof."""
    sc = ic.impact_halfspace(nx=10, ny=10, nz=5, r_cells=2.0)
    k = int(np.argmax(sc.pos[:, 2]))
    sc.vel[k] = (0.0, 0.0, 4.0e5)   # leaves through the top within a few steps
    errs, info, _ = run_pair(sc, 8)
    assert max(errs.values()) < 1e-9, errs


@pytest.mark.parametrize("cfz", [0.5, 0.25])
def test_flat_z_cells_match_oracle(cuda_lib, oracle_lib, cfz):
    """Traversal cells cell_factor_z times as high as wide: the same pairs,
    found over shorter column chords."""
    sc = ic.impact_halfspace(nx=12, ny=12, nz=6, r_cells=2.0)
    errs, _, _ = run_pair(sc, 4, cell_factor_z=cfz)
    assert max(errs.values()) < 1e-9, errs


def test_remove_in_the_middle(cuda_lib):
    from deorbit_gb300 import sph
    scs = ic.batch_impacts(count=3, lo=1500, hi=3000)
    ctx = sph.Context(sph.MIXED)
    mids = {}
    ids = [ic.to_context(ctx, s, material_ids=mids) for s in scs]
    ctx.init()
    ctx.run(3)
    ctx.remove(ids[1])
    ctx.run(3)
    got = [read_all(ctx, b, NAMES) for b in (ids[0], ids[2])]
    ctx.close()
    for s, g in zip((scs[0], scs[2]), got):
        alone = sph.Context(sph.MIXED)
        b = ic.to_context(alone, s)
        alone.init()
        alone.run(3)
        alone.run(3)
        ref = read_all(alone, b, NAMES)
        alone.close()
        for k in NAMES:
            assert np.array_equal(g[k], ref[k]), k


def test_flaw_pool_through_admissions_and_retirements(cuda_lib):
    """Multi-flaw thresholds live in one device pool with a segment per impact:
    impacts retired and admitted over several cycles (reusing particle ids and
    growing, then compacting, the pool) keep exactly the thresholds and the
    damage they have alone."""
    from deorbit_gb300 import sph
    scs = ic.batch_impacts(count=9, lo=1200, hi=2600, seed=7)
    ctx = sph.Context(sph.MIXED)
    mids = {}
    live = {}
    for s in scs[:3]:
        live[ic.to_context(ctx, s, material_ids=mids)] = s
    ctx.init()
    ctx.run(2)
    for cyc, s in enumerate(scs[3:]):
        ctx.remove(sorted(live)[cyc % len(live)])
        live.pop(sorted(live)[cyc % len(live)])
        b = ic.to_context(ctx, s, material_ids=mids)
        live[b] = s
        ctx.init()
        ctx.run(2)
    ctx.run(2)
    got = {b: (ctx.flaws(b), read_all(ctx, b, NAMES + ["D"])) for b in live}
    ctx.close()
    for b, s in live.items():
        alone = sph.Context(sph.MIXED)
        a = ic.to_context(alone, s)
        alone.init()
        ptr, eps = alone.flaws(a)
        assert len(eps) > 0
        assert np.array_equal(got[b][0][0], ptr) and np.array_equal(got[b][0][1], eps), b
        if s is scs[-1]:  # admitted last: two rounds of two steps in the mix
            alone.run(2)
            alone.run(2)
            ref = read_all(alone, a, NAMES + ["D"])
            for k in ref:
                assert np.array_equal(got[b][1][k], ref[k]), k
        alone.close()
