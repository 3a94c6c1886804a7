"""The Euler grid oracle (oracle/euler_oracle.c) against the reference.

* Golden vectors: tests/golden/euler_gates.npz holds the reference solver's
  outputs (hydrocodes/euler/hydro_cpu.cpp compiled unmodified, see
  tests/golden/make_euler_golden.py) for the gate workloads run through the
  drivers' loop and for single operators; the oracle reproduces every field
  bit for bit.
* Physics gates: the reference's own pass/fail gates (hydro_cpu.cpp modes sod,
  tracer, shear, yield, vacuum, tensile, freefall, atmos, alimpact, friction;
  the CI list) evaluated on the oracle's full runs.
* The library's default settings equal the oracle's (and, where the reference
  tree is present, the reference's own).
* The reference's implicit-viscosity gates (visc_diff, visc_agree,
  visc_energy, vib_regen; tests/visc_gates.py) on the oracle.
"""
import json
import math
import os

import numpy as np
import pytest

from deorbit_gb300 import grid_ic as GI
from oracle import euler as EO
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "euler_gates.npz")


def _cases():
    z = np.load(GOLD)
    keys = sorted({k.split("/")[0] for k in z.files})
    return z, keys


def case_from(z, key):
    """The workload case a fixture was made from (fields, reference state, pin)."""
    meta = json.loads(str(z[f"{key}/meta"]))
    ins = {k.split("/")[-1]: z[k] for k in z.files if k.startswith(key + "/in/")}
    post = {k.split("/")[-1]: z[k] for k in z.files if k.startswith(key + "/post/")}
    case = GI.Case(key, tuple(meta["shape"]), meta["dx"], meta["material"], meta["params"], ins,
                   meta.get("cfl", 0.4), meta.get("t_end", 0.0), meta.get("set_ref", False), post,
                   meta.get("pin_floor", 0), meta.get("sponge_from", -1))
    return case, meta


def _grid_from(z, key):
    case, meta = case_from(z, key)
    return EO.from_case(case), meta, case


@pytest.mark.parametrize("key", _cases()[1])
def test_oracle_reproduces_reference_bit_for_bit(key):
    z = np.load(GOLD)
    g, meta, case = _grid_from(z, key)
    if meta["kind"] == "run":
        s, t = EO.run_case(g, case, meta["max_steps"])
        assert s == meta["steps"] and t == meta["t"]
        got = g.fields()
    else:
        if meta["op"] == "lop":
            g.lop()
            got = {f"rhs_{k}": g.rhs(k) for k in EO.RHS}
        else:
            getattr(g, meta["op"])(meta["arg"])
            got = g.fields()
        got["maxspeed"] = np.array([g.maxspeed()])
    assert g.visc_iters() == meta.get("visc_iters", 0)
    for k in z.files:
        if k.startswith(key + "/out/"):
            name = k.split("/")[-1]
            assert np.array_equal(got[name], z[k]), (key, name)
    g.close()


@pytest.mark.parametrize("gate", ["visc_diff", "visc_agree", "visc_energy", "vib_regen"])
def test_oracle_passes_viscosity_gates(gate):
    import visc_gates as VG
    ok, info = VG.GATES[gate](VG.OracleGrid)
    assert ok, info


def test_default_settings_agree():
    """Oracle defaults = hydro_cpu.cpp:17-36 (and the reference's own values
    when its shim is built); the C ABI's eu_params_default (no GPU needed)
    gives the same numbers."""
    orc = EO.default_params().as_dict()
    if EO.ref_available():
        assert EO.default_params(ref=True).as_dict() == orc
    from deorbit_gb300 import euler as E
    lib_p = E.default_params()
    for k, v in orc.items():
        assert getattr(lib_p, k) == v, k


def _run(case):
    g = EO.from_case(case)
    s, t = g.run(case.cfl, case.t_end)
    return g, s, t


def _exact_sod(S, gam=1.4):
    """Exact Riemann solution of Sod's problem at x/t = S (Toro, ch. 4)."""
    rL, uL, pL, rR, uR, pR = 1.0, 0.0, 1.0, 0.125, 0.0, 0.1
    cL, cR = math.sqrt(gam * pL / rL), math.sqrt(gam * pR / rR)
    G1, G2, G3, G4, G5, G6 = ((gam - 1) / (2 * gam), (gam + 1) / (2 * gam), 2 * gam / (gam - 1),
                              2 / (gam - 1), 2 / (gam + 1), (gam - 1) / (gam + 1))

    def fk(P, rk, pk, ck):
        if P > pk:
            A, B = G5 / rk, G6 * pk
            return (P - pk) * math.sqrt(A / (P + B))
        return G4 * ck * ((P / pk) ** G1 - 1)

    def fp(P, rk, pk, ck):
        if P > pk:
            A, B = G5 / rk, G6 * pk
            return math.sqrt(A / (B + P)) * (1 - (P - pk) / (2 * (B + P)))
        return (P / pk) ** (-G2) / (rk * ck)

    P = 0.5 * (pL + pR)
    for _ in range(100):
        Pn = abs(P - (fk(P, rL, pL, cL) + fk(P, rR, pR, cR) + uR - uL) / (fp(P, rL, pL, cL) + fp(P, rR, pR, cR)))
        if abs(Pn - P) < 1e-12:
            P = Pn
            break
        P = Pn
    us = 0.5 * (uL + uR) + 0.5 * (fk(P, rR, pR, cR) - fk(P, rL, pL, cL))
    if S <= us:
        SHL, STL = uL - cL, us - cL * (P / pL) ** G1
        if S < SHL:
            return rL, uL, pL
        if S > STL:
            return rL * (P / pL) ** (1 / gam), us, P
        u = G5 * (cL + (gam - 1) / 2 * uL + S)
        c = G5 * (cL + (gam - 1) / 2 * (uL - S))
        return rL * (c / cL) ** G4, u, pL * (c / cL) ** G3
    SR = uR + cR * math.sqrt(G2 * P / pR + G1)
    if S > SR:
        return rR, uR, pR
    return rR * ((P / pR + G6) / (G6 * P / pR + 1)), us, P


def test_gate_sod():
    """hydro_cpu.cpp:449-454: L1(rho) against the exact solution < 0.007."""
    case = GI.sod()
    g, s, t = _run(case)
    N = case.shape[0]
    x = (np.arange(N) + 0.5) * case.dx
    re = np.array([_exact_sod((xi - 0.5) / case.t_end)[0] for xi in x])
    assert t == case.t_end
    assert np.abs(g.field("r") - re).mean() < 0.007


def test_gate_tracer():
    """hydro_cpu.cpp:455-465: tracer mass conserved, centroid speed within 1%."""
    case = GI.tracer()
    x = (np.arange(case.shape[0]) + 0.5) * case.dx
    rc0 = case.fields["rc"]
    g, s, t = _run(case)
    rc1, r1 = g.field("rc"), g.field("r")
    cen0, cen1 = (rc0 * x).sum() / rc0.sum(), (rc1 * x).sum() / rc1.sum()
    assert abs(rc1.sum() - rc0.sum()) / rc0.sum() < 1e-6
    assert abs((cen1 - cen0) / t - 2.0) / 2.0 < 0.01
    cc = rc1 / r1
    assert cc.min() >= -1e-9 and cc.max() <= 1.0 + 1e-9


def test_gate_shear_and_yield():
    """hydro_cpu.cpp:682-703: elastic shear speed within 3%; the von Mises cap."""
    case = GI.shear()
    g, s, t = _run(case)
    N, dx = case.shape[0], case.dx
    vy = g.field("mv") / g.field("r")
    x0 = 0.3 * 400e3
    ip0 = int(x0 / dx)
    i = np.arange(ip0 + 3, N - 2)
    xpk = (i[np.argmax(vy[i])] + 0.5) * dx
    cs = math.sqrt(2.27e10 / 2700.0)
    assert abs((xpk - x0) / t - cs) / cs < 0.03
    case = GI.yield_pulse()
    g, s, t = _run(case)
    f = g.fields(["Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"])
    J2 = 0.5 * (f["Sxx"] ** 2 + f["Syy"] ** 2 + f["Szz"] ** 2) + f["Sxy"] ** 2 + f["Sxz"] ** 2 + f["Syz"] ** 2
    smax, Y = np.sqrt(3 * J2).max(), 3.5e8
    assert 0.9 * Y < smax <= 1.01 * Y


def test_gate_vacuum():
    """hydro_cpu.cpp:704-715: the Toro rarefaction fan into vacuum."""
    case = GI.vacuum()
    g, s, t = _run(case)
    gam, rL, pL = 1.4, 1.0, 1.0
    cL = math.sqrt(gam * pL / rL)
    x = (np.arange(case.shape[0]) + 0.5) * case.dx
    S = (x - 0.5) / t
    fan = (S > -cL) & (S < 2 * cL / (gam - 1))
    ua = np.where(S <= -cL, 0.0, np.where(fan, 2.0 / (gam + 1) * (cL + S), 0.0))
    cc = 2.0 / (gam + 1) * (cL - 0.5 * (gam - 1) * S)
    ra = np.where(S <= -cL, rL, np.where(fan, rL * np.abs(cc / cL) ** (2.0 / (gam - 1)), 0.0))
    r = g.field("r")
    sel = ra > 0.02
    assert np.abs(r[sel] - ra[sel]).mean() < 0.03
    assert np.abs(g.field("mu")[sel] / r[sel] - ua[sel]).mean() < 0.05
    assert r.min() > 0


def test_gate_tensile():
    """hydro_cpu.cpp:736-743: tensile damage grows past 0.9 and weakens Sxx."""
    case = GI.tensile()
    g, s, t = _run(case)
    D, Sxx = g.field("D")[20:80], g.field("Sxx")[20:80]
    assert D.max() > 0.9 and np.abs(Sxx).max() < 0.5 * 3.5e8


def test_gate_freefall_and_atmos():
    """hydro_cpu.cpp:721-735: v = -g t exactly enough; a still atmosphere."""
    case = GI.freefall()
    g, s, t = _run(case)
    v = g.field("mw") / g.field("r")
    assert np.abs(v + 9.8 * t).max() < 1e-3 * 9.8 * t
    case = GI.atmos()
    g, s, t = _run(case)
    v = g.field("mw") / g.field("r")
    cs = math.sqrt(1.4 * 1e5)
    assert np.abs(v[80:120]).max() < 0.02 * cs


def test_gate_alimpact():
    """hydro_cpu.cpp:744-752: peak shock pressure within 5% of the Tillotson
    Hugoniot (bisection on the shock speed as in hydro_cpu.cpp:440-446)."""
    case = GI.alimpact()
    g, s, t = _run(case)
    m = O.material_from_dict(case.material)
    Pmax = max(g.pcell(c) for c in range(case.n))
    rho0, up = 2700.0, 5000.0
    lo, hi = up * 1.0001, up * 30.0
    for _ in range(200):
        Us = 0.5 * (lo + hi)
        rho = rho0 * Us / (Us - up)
        Pm = rho0 * Us * up
        uint = 0.5 * Pm * (1.0 / rho0 - 1.0 / rho)
        if Pm - float(O.eos(m, np.array([rho]), np.array([uint]))[0][0]) < 0:
            lo = Us
        else:
            hi = Us
    Phug = rho0 * 0.5 * (lo + hi) * up
    assert abs(Pmax - Phug) / Phug < 0.05


def test_gate_friction():
    """hydro_cpu.cpp:541-556: the ROCK yield caps pure shear on the analytic
    intact (Lundborg) / damaged (friction) surfaces, to 1e-6."""
    m = O.material_from_dict(GI.ic.basalt())
    prm = {"rock": 1, "y_d0": 5.0e6}
    d = EO.default_params().as_dict()
    for mu in (0.001, 0.005, 0.02, 0.05):
        for dam in (0, 1):
            g = EO.OracleGrid(1, 1, 1, 500.0, material=m, params=prm)
            g.set_field("r", [2700.0 * (1.0 + mu)])
            g.set_field("D", [float(dam)])
            g.set_field("Sxy", [5.0e9])
            P = g.pcell(0)
            g.vonmises()
            f = g.fields(["Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"])
            J2 = 0.5 * (f["Sxx"] ** 2 + f["Syy"] ** 2 + f["Szz"] ** 2) + f["Sxy"] ** 2 + f["Sxz"] ** 2 + f["Syz"] ** 2
            vm = math.sqrt(3.0 * J2[0])
            Yi = d["y_i0"] + d["mu_i"] * P / (1.0 + d["mu_i"] * P / (d["y_m"] - d["y_i0"]))
            Yd = min(5.0e6 + d["mu_d"] * P, d["y_m"])
            Y = Yd if dam else Yi
            assert abs(vm - Y) / Y < 1e-6, (mu, dam)
            g.close()
