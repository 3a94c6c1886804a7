"""The reference's CPU validation gates, applied to the oracle (CPU only):
eos_test.cpp:10-33 known answers, strength_test.cpp:56-121 (shear, yield,
elastic wave) and the Collins / Lundborg yield-surface gate of
hydrocodes/euler/hydro_cpu.cpp:541-556 for the oracle's extension."""
import numpy as np
import pytest

from deorbit_gb300 import ic


def test_eos_known_answers(oracle_lib):
    O = oracle_lib
    for m, lo, hi in ((O.iron(), 3900, 4200), (O.basalt(), 3000, 3300), (O.water(), 1450, 1520)):
        P0, c0 = O.eos(m, [m.rho0], [0.0])
        Pc, _ = O.eos(m, [1.1 * m.rho0], [0.0])
        assert abs(P0[0]) < 1e3
        assert lo < c0[0] < hi
        assert Pc[0] > 0


def basalt_block(O, x0, x1, dx, Lyz):
    S = O.OracleSystem()
    S.add_material(O.basalt())
    S.set_params(eta=1.3, h_init=1.3 * dx)
    S.set_domain((x0, 0, 0), (x1, Lyz, Lyz))
    nx, ny = int(round((x1 - x0) / dx)), int(round(Lyz / dx))
    pos = ic.lattice(nx, ny, ny, dx, (x0, 0.0, 0.0))
    S.add_many(pos, np.zeros_like(pos), O.basalt().rho0 * dx ** 3, 0.0, 0)
    return S, pos


def test_shear_rate(oracle_lib):
    O = oracle_lib
    S, pos = basalt_block(O, -0.2, 0.2, 0.02, 0.16)
    S.set_field("vx", pos[:, 1])
    S.set_field("vy", pos[:, 0])
    S.init()
    S.compute_strain_stress()
    best = np.argmin(((pos - [0, 0.08, 0.08]) ** 2).sum(1))
    ratio = S.field("dSxy")[best] / (2 * O.basalt().G * 1.0)
    assert 0.8 < ratio < 1.2


def test_von_mises_cap(oracle_lib):
    O = oracle_lib
    S = O.OracleSystem()
    S.add_material(O.basalt())
    S.add_many(np.zeros((1, 3)), np.zeros((1, 3)), 1.0, 0.0, 0)
    s = [1.0e9, -0.4e9, -0.6e9, 3.0e8, 1.0e8, -2.0e8]
    for k, v in zip(("Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"), s):
        S.set_field(k, [v])
    S.yield_limit(0)
    a = [S.field(k)[0] for k in ("Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz")]
    J2 = 0.5 * (a[0] ** 2 + a[1] ** 2 + a[2] ** 2) + (a[3] ** 2 + a[4] ** 2 + a[5] ** 2)
    assert abs(np.sqrt(3 * J2) - O.basalt().Y) / O.basalt().Y < 1e-6
    ratios = np.array(a) / np.array(s)
    assert np.ptp(ratios) < 1e-9


def test_collins_yield_surface(oracle_lib):
    """Extension gate: the capped stress follows Y_i(P) (intact) and Y_d(P)
    (damaged) on the analytic surface to 1e-6, as in hydro_cpu.cpp:541-556."""
    O = oracle_lib
    base = O.basalt()
    m = O.collins(base, Y0=1.0e7, mu_i=1.2, Ylim=2.5e9, Yd0=5.0e6, mu_d=0.6)
    for mu in (0.001, 0.005, 0.02, 0.05):
        for dam in (0.0, 1.0):
            S = O.OracleSystem()
            S.add_material(m)
            S.add_many(np.zeros((1, 3)), np.zeros((1, 3)), 1.0, 0.0, 0)
            rho = base.rho0 * (1 + mu)
            P = O.eos(m, [rho], [0.0])[0][0]
            S.set_field("P", [P])
            S.set_field("D", [dam])
            S.set_field("Sxy", [5.0e9])
            S.yield_limit(0)
            vm = np.sqrt(3.0) * abs(S.field("Sxy")[0])
            Yi = 1.0e7 + 1.2 * P / (1.0 + 1.2 * P / (2.5e9 - 1.0e7))
            Yd = min(5.0e6 + 0.6 * P, 2.5e9)
            Y = Yd if dam else Yi
            assert abs(vm - Y) / Y < 1e-6, (mu, dam)


@pytest.mark.slow
def test_elastic_wave_speed(oracle_lib):
    """strength_test.cpp:95-120: the right-going pulse travels at c_L (+-15%)."""
    O = oracle_lib
    S, pos = basalt_block(O, -0.6, 0.6, 0.01, 0.08)
    S.set_domain((-0.6, 0, 0), (0.6, 0.08, 0.08), (False, True, True))
    b = O.basalt()
    cL = np.sqrt((b.A + 4.0 / 3.0 * b.G) / b.rho0)
    S.set_field("vx", np.exp(-(pos[:, 0] ** 2) / 0.06 ** 2))
    S.set_fixed((np.abs(pos[:, 0]) > 0.55).astype(np.uint8))
    S.init()
    t, t1 = 0.0, 6.0e-5
    while t < t1:
        dt = min(S.timestep(), t1 - t)
        S.step(dt)
        t += dt
    x = S.field("x")
    v = np.abs(S.field("vx"))
    sel = x > 0.05
    xpk = x[sel][np.argmax(v[sel])]
    assert 0.85 < (xpk / t) / cL < 1.15
