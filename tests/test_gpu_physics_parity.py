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
  mixed     on the oracle's dt sequence, after 20 steps: rel-L2 <= 1e-4 per field
            (the mixed-form target) for every field damage does not switch; the
            device's flaw thresholds equal to the oracle's rounded to FP32.
            Damage is an integer step function of sigma_max / E (the number of
            flaws whose threshold it exceeds, with D capped at n_act / n_f), so a
            particle whose sigma_max sits within FP32 rounding of a threshold
            activates a flaw one step earlier or later than in FP64 and its D
            differs by ~1 / n_f for good (a "flip").  One flip among 30,000
            particles is ~3e-4 of D's rel-L2.  The test therefore asserts D and S
            (which D scales) at 1e-4 over the particles without a flip, and that
            flips stay below 1 in 1,000 particles.
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
    switched = ("D", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz")
    bad = {k: v for k, v in errs.items() if k not in switched and not v <= MIXED_TOL}
    assert not bad, bad
    keep = np.abs(gpu["D"] - orc["D"]) <= 1e-6
    errs_kept = {k: rel_l2(gpu[k][keep], orc[k][keep]) for k in switched}
    print(which, "mixed, particles without a flip", {k: f"{v:.1e}" for k, v in errs_kept.items()})
    bad = {k: v for k, v in errs_kept.items() if not v <= MIXED_TOL}
    assert not bad, bad
    assert flips <= sc.n // 1000, flips


def test_scenarios_exercise_the_extensions():
    """The scenarios switch on what they are meant to test (host-side check)."""
    g = grazing_small()
    assert g.materials[0]["yield_model"] == 1 and g.materials[0]["Y0"] == 1.0e7
    assert g.params["flaw_model"] == 1 and g.params["eps_as"] == 0.3 and g.flaws[0] == "multi"
    c = graded_crop()
    assert c.h0 is not None and np.unique(np.round(c.h0, 6)).size >= 3
