"""The Sod shock tube gate (the reference's sod.cpp + analyze_sod.py criteria):
ideal gas, artificial conductivity, periodic y / z, frozen ends, run to
t = 0.2 and compared with the exact Riemann solution -- binned density and
pressure RMS error < 0.05 over 100 bins in [-0.45, 0.45], shock front within 3
bins of the exact one.  Plus FP64 parity with the oracle on the same tube.

The exact solution is this file's own implementation of the standard exact
Riemann solver for the Euler equations of an ideal gas (Toro, "Riemann Solvers
and Numerical Methods for Fluid Dynamics", ch. 4): Newton iteration on the
star-region pressure, then sampling of the self-similar solution at x / t."""
import math
import os

import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O

from parity import field_errors, read_all

GAMMA = 1.4
LEFT = (1.0, 0.0, 1.0)     # rho, u, p
RIGHT = (0.125, 0.0, 0.1)
T_END = 0.2


class ExactRiemann:
    def __init__(self, left, right, g=GAMMA):
        self.g = g
        self.L, self.R = left, right
        self.cL = math.sqrt(g * left[2] / left[0])
        self.cR = math.sqrt(g * right[2] / right[0])
        self.p_star, self.u_star = self._star()

    def _branch(self, p, state, c):
        """Velocity change across the wave of one side and its derivative."""
        rho, _, pk = state
        g = self.g
        if p > pk:  # shock
            a = 2.0 / ((g + 1.0) * rho)
            b = (g - 1.0) / (g + 1.0) * pk
            q = math.sqrt(a / (p + b))
            return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (p + b))
        r = p / pk  # rarefaction
        return 2.0 * c / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0), r ** (-(g + 1.0) / (2.0 * g)) / (rho * c)

    def _star(self):
        p = 0.5 * (self.L[2] + self.R[2])
        for _ in range(200):
            fl, dl = self._branch(p, self.L, self.cL)
            fr, dr = self._branch(p, self.R, self.cR)
            step = (fl + fr + self.R[1] - self.L[1]) / (dl + dr)
            p_new = max(p - step, 1e-12)
            if abs(p_new - p) <= 1e-14 * p:
                p = p_new
                break
            p = p_new
        fl, _ = self._branch(p, self.L, self.cL)
        fr, _ = self._branch(p, self.R, self.cR)
        return p, 0.5 * (self.L[1] + self.R[1]) + 0.5 * (fr - fl)

    def shock_speed_right(self):
        g, (rho, u, pk) = self.g, self.R
        return u + self.cR * math.sqrt((g + 1.0) / (2.0 * g) * self.p_star / pk + (g - 1.0) / (2.0 * g))

    def sample(self, s):
        """(rho, u, p) at similarity coordinate s = x / t."""
        g, ps, us = self.g, self.p_star, self.u_star
        left = s <= us
        rho, u, pk = self.L if left else self.R
        c = self.cL if left else self.cR
        sgn = -1.0 if left else 1.0      # waves move left (-) or right (+)
        if ps > pk:  # shock on this side
            ws = u + sgn * c * math.sqrt((g + 1.0) / (2.0 * g) * ps / pk + (g - 1.0) / (2.0 * g))
            if sgn * (s - ws) >= 0.0:
                return rho, u, pk
            ratio = ps / pk
            k = (g - 1.0) / (g + 1.0)
            return rho * (ratio + k) / (k * ratio + 1.0), us, ps
        head = u + sgn * c
        c_star = c * (ps / pk) ** ((g - 1.0) / (2.0 * g))
        tail = us + sgn * c_star
        if sgn * (s - head) >= 0.0:
            return rho, u, pk
        if sgn * (s - tail) <= 0.0:
            return rho * (ps / pk) ** (1.0 / g), us, ps
        # inside the fan
        cf = 2.0 / (g + 1.0) * (c - sgn * 0.5 * (g - 1.0) * (u - s))
        uf = 2.0 / (g + 1.0) * (-sgn * c + 0.5 * (g - 1.0) * u + s)
        return rho * (cf / c) ** (2.0 / (g - 1.0)), uf, pk * (cf / c) ** (2.0 * g / (g - 1.0))


def run_tube(sph, precision):
    sc = ic.sod_tube()
    ctx = sph.Context(precision)
    b = ic.to_context(ctx, sc)
    ctx.init()
    while ctx.info(b).t < T_END:
        ctx.run(50, T_END)
    f = read_all(ctx, b, ["x", "vx", "rho", "P"])
    moving = ctx.fixed(b) == 0
    t = ctx.info(b).t
    ctx.close()
    return {k: v[moving] for k, v in f.items()}, t


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_sod_against_exact_riemann(cuda_lib, precision):
    from deorbit_gb300 import sph
    f, t = run_tube(sph, precision)
    assert abs(t - T_END) < 1e-12
    ex = ExactRiemann(LEFT, RIGHT)
    nb, lo, hi = 100, -0.45, 0.45
    sel = (f["x"] >= lo) & (f["x"] < hi)
    idx = ((f["x"][sel] - lo) / (hi - lo) * nb).astype(int)
    cnt = np.bincount(idx, minlength=nb)
    occupied = cnt > 0
    mean = {k: np.bincount(idx, weights=f[k][sel], minlength=nb)[occupied] / cnt[occupied]
            for k in ("rho", "vx", "P")}
    xc = lo + (np.arange(nb)[occupied] + 0.5) / nb * (hi - lo)
    exact = np.array([ex.sample(x / T_END) for x in xc])
    rms = {k: float(np.sqrt(np.mean((mean[k] - exact[:, c]) ** 2))) for c, k in ((0, "rho"), (1, "vx"), (2, "P"))}
    # shock front: rightmost bin with binned density above 0.2
    above = np.nonzero(mean["rho"] > 0.2)[0]
    x_shock = xc[above[-1]]
    x_exact = ex.shock_speed_right() * T_END
    binw = (hi - lo) / nb
    assert abs(x_shock - x_exact) < 3 * binw, (x_shock, x_exact)
    assert rms["rho"] < 0.05 and rms["P"] < 0.05, rms


def test_exact_solver_known_values():
    """Toro's test 1 (the Sod problem): p* = 0.30313, u* = 0.92745."""
    ex = ExactRiemann(LEFT, RIGHT)
    assert abs(ex.p_star - 0.30313) < 1e-5 and abs(ex.u_star - 0.92745) < 1e-5
    # star densities either side of the contact and the shock speed
    assert abs(ex.sample(ex.u_star - 1e-9)[0] - 0.42632) < 1e-5
    assert abs(ex.sample(ex.u_star + 1e-9)[0] - 0.26557) < 1e-5
    assert abs(ex.shock_speed_right() - 1.75216) < 1e-5
    # undisturbed states outside the waves, a point inside the rarefaction fan
    assert ex.sample(-2.0) == LEFT and ex.sample(2.0) == RIGHT
    rho, u, p = ex.sample(-0.5)
    assert 0.42632 < rho < 1.0 and 0.0 < u < ex.u_star and ex.p_star < p < 1.0


@pytest.mark.gpu
def test_sod_fp64_matches_oracle(cuda_lib, oracle_lib):
    """Ideal EOS, artificial conductivity, periodic axes and frozen ends
    against the oracle: 40 steps with the oracle's dt."""
    from deorbit_gb300 import sph
    sc = ic.sod_tube()
    ctx = sph.Context(sph.FP64)
    b = ic.to_context(ctx, sc)
    orc = O.from_scenario(sc, threads=min(os.cpu_count() or 1, 16))
    ctx.init()
    orc.init()
    for _ in range(40):
        dt = orc.timestep()
        assert abs(ctx.timestep(b) - dt) <= 1e-9 * dt
        orc.step(dt)
        ctx.step(dt)
    names = ["x", "vx", "u", "rho", "P", "hh"]
    errs = field_errors(read_all(ctx, b, names), {k: orc.field(k) for k in names}, names)
    ctx.close()
    assert max(errs.values()) < 1e-9, errs
