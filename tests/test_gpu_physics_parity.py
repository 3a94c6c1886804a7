"""CUDA solver vs the FP64 CPU oracle on the physics of the strength + damage
workloads, on small seeded versions of them:

  grazing   iron sphere into a granite slab at 3 deg, 8 km/s, the sphere touching
            the surface from the start: granite with Collins pressure-dependent
            yield, iron with von Mises yield, Benz-Asphaug multi-flaw damage and
            artificial stress eps_as = 0.3 (the 1,048,576-particle grazing
            impact's physics at ~16k particles)
  graded    a crop of the graded slab (per-particle reference smoothing length
            h0 = 1.3 x the local lattice spacing, growing with depth), same
            physics

Tolerances:
  FP64      rel-L2 <= 1e-9 per field after 20 steps, stress and damage included,
            with the CFL dt agreeing to 1e-9 every step; the device's multi-flaw
            CSR equal to the oracle's bit for bit
  mixed     rel-L2 <= 1e-4 per field after 20 steps (the mixed-form target), on
            the oracle's dt sequence; the device's flaw thresholds equal to the
            oracle's rounded to FP32
"""
import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O

from parity import rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ["x", "y", "z", "vx", "vy", "vz", "u", "rho", "hh", "P", "cs", "csig", "sigmax",
          "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz", "D"]
FP64_TOL = 1e-9
MIXED_TOL = 1e-4
STEPS = 20


def grazing_small():
    return ic.grazing(n_total=16384, gap=0.25)


def graded_crop():
    return ic.crop(ic.large_graded(1 << 18), 30000)


SCENARIOS = {"grazing": grazing_small, "graded": graded_crop}


@pytest.fixture(scope="module")
def sph_mod(cuda_lib, oracle_lib):
    from deorbit_gb300 import sph
    return sph


_oracle_runs = {}


def oracle_run(which):
    """Oracle trajectory of a scenario: its dt sequence and final fields."""
    if which not in _oracle_runs:
        sc = SCENARIOS[which]()
        orc = O.from_scenario(sc, threads=16)
        orc.init()
        dts = []
        for _ in range(STEPS):
            dts.append(orc.timestep())
            orc.step(dts[-1])
        _oracle_runs[which] = (sc, dts, {k: orc.field(k) for k in FIELDS}, orc.flaws())
        orc.close()
    return _oracle_runs[which]


def gpu_run(sph, sc, precision, dts):
    ctx = sph.Context(precision)
    b = ic.to_context(ctx, sc)
    ctx.init()
    dt_err = 0.0
    for dt in dts:
        if precision == sph.FP64:
            dt_err = max(dt_err, abs(ctx.timestep(b) - dt) / dt)
        ctx.step(dt)
    out = {k: ctx.read(b, k) for k in FIELDS}
    flaws = ctx.flaws(b)
    ctx.close()
    return out, flaws, dt_err


@pytest.mark.parametrize("which", ["grazing", "graded"])
def test_fp64_matches_oracle(sph_mod, which):
    sc, dts, orc, oflaws = oracle_run(which)
    assert np.count_nonzero(orc["D"]) > 0, "the scenario must exercise damage"
    gpu, flaws, dt_err = gpu_run(sph_mod, sc, sph_mod.FP64, dts)
    assert dt_err <= 1e-9, dt_err
    errs = {k: rel_l2(gpu[k], orc[k]) for k in FIELDS}
    print(which, "fp64", {k: f"{v:.1e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if not v <= FP64_TOL}
    assert not bad, bad
    assert np.array_equal(flaws[0], oflaws[0]) and np.array_equal(flaws[1], oflaws[1])


@pytest.mark.parametrize("which", ["grazing", "graded"])
def test_mixed_matches_oracle(sph_mod, which):
    sc, dts, orc, oflaws = oracle_run(which)
    gpu, flaws, _ = gpu_run(sph_mod, sc, sph_mod.MIXED, dts)
    errs = {k: rel_l2(gpu[k], orc[k]) for k in FIELDS}
    flips = int(np.count_nonzero(np.abs(gpu["D"] - orc["D"]) > 1e-6))
    print(which, "mixed", {k: f"{v:.1e}" for k, v in errs.items()}, "D differs at", flips)
    assert np.array_equal(flaws[0], oflaws[0])
    assert np.array_equal(flaws[1], oflaws[1].astype(np.float32).astype(np.float64))
    bad = {k: v for k, v in errs.items() if not v <= MIXED_TOL}
    assert not bad, bad


def test_scenarios_exercise_the_extensions():
    """The scenarios switch on what they are meant to test (host-side check)."""
    g = grazing_small()
    assert g.materials[0]["yield_model"] == 1 and g.materials[0]["Y0"] == 1.0e7
    assert g.params["flaw_model"] == 1 and g.params["eps_as"] == 0.3 and g.flaws[0] == "multi"
    c = graded_crop()
    assert c.h0 is not None and np.unique(np.round(c.h0, 6)).size >= 3
