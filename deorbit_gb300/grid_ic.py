"""Workloads of the Eulerian grid hydrocode.

Each `Case` holds a grid shape, cell width, material, solver settings and the
initial fields, plus the CFL number and end time of its run.  The 1-D / 2-D /
3-D gate problems restate the initial conditions of the reference driver's
modes (hydrocodes/euler/hydro_cpu.cpp:449-905, cited per case); `impact3d`
is this repository's 3-D Cartesian half-space impact used as the grid
solver's throughput workload (seeded, synthetic, no dataset).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import ic

GAM = 1.4


@dataclass
class Case:
    name: str
    shape: tuple
    dx: float
    material: dict
    params: dict = field(default_factory=dict)
    fields: dict = field(default_factory=dict)
    cfl: float = 0.4
    t_end: float = 0.0
    set_ref: bool = False      # freeze `fields` as the hydrostatic reference (set_ref) ...
    post_ref: dict = field(default_factory=dict)  # ... then write these over them
    pin_floor: int = 0         # driver: the lowest pin_floor z-layers return to the reference each step
    sponge_from: int = -1      # driver: columns i >= sponge_from relax toward the reference each step
    driver_flags: int = 0      # driver: euler.DRIVER_* steps after each step

    @property
    def n(self):
        return self.shape[0] * self.shape[1] * self.shape[2]


def aluminum():
    """Material::aluminum (eos.hpp:48-49)."""
    return ic.tillotson(2700, 7.52e10, 6.5e10, 0.5, 1.63, 5, 5, 5.0e6, 3.0e6, 1.39e7)


def _centres(n, dx):
    return (np.arange(n, dtype=np.float64) + 0.5) * dx


def _zeros(n):
    return np.zeros(n, dtype=np.float64)


def sod(N=200):
    """hydro_cpu.cpp:449-454: Sod tube, ideal gas 1.4, t_end 0.2, CFL 0.4."""
    dx = 1.0 / N
    x = _centres(N, dx)
    r = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    return Case("sod", (N, 1, 1), dx, ic.ideal_gas(GAM), {}, {"r": r, "E": p / (GAM - 1)}, 0.4, 0.2)


def tracer(N=200):
    """hydro_cpu.cpp:455-465: a tracer blob advected by a uniform flow."""
    dx = 1.0 / N
    x = _centres(N, dx)
    rho0, p0, v0 = 1.0, 1.0, 2.0
    f = {"r": np.full(N, rho0), "mu": np.full(N, rho0 * v0),
         "E": np.full(N, p0 / (GAM - 1) + 0.5 * rho0 * v0 * v0),
         "rc": rho0 * np.where((x > 0.3) & (x < 0.5), 1.0, 0.0)}
    return Case("tracer", (N, 1, 1), dx, ic.ideal_gas(GAM), {}, f, 0.4, 0.15)


def sedov(N=64):
    """hydro_cpu.cpp:466-477: 3-D point blast, E0 = 1 in the central cell."""
    L, E0, rho0 = 2.0, 1.0, 1.0
    dx = L / N
    n = N * N * N
    E = np.full(n, 1e-4 / (GAM - 1))
    ic_ = N // 2
    E[(ic_ * N + ic_) * N + ic_] += E0 / (dx * dx * dx)
    return Case("sedov", (N, N, N), dx, ic.ideal_gas(GAM), {}, {"r": np.full(n, rho0), "E": E}, 0.3, 0.5)


def sedov_axi(Nr=64, Nz=128):
    """hydro_cpu.cpp:478-489: on-axis point blast in cylindrical (r, z)."""
    dx = 2.0 / 64
    E0, rho0 = 1.0, 1.0
    n = Nr * Nz
    E = np.full(n, 1e-4 / (GAM - 1))
    kc = Nz // 2
    E[kc] += E0 / (math.pi * dx * dx * dx)
    return Case("sedov_axi", (Nr, 1, Nz), dx, ic.ideal_gas(GAM), {"axisym": 1},
                {"r": np.full(n, rho0), "E": E}, 0.3, 0.5)


def _pulse(N, L, A):
    rho0 = 2700.0
    dx = L / N
    x = _centres(N, dx)
    x0, wid = 0.3 * L, 8e3
    vy = A * np.exp(-((x - x0) / wid) * ((x - x0) / wid))
    return dx, {"r": np.full(N, rho0), "mv": rho0 * vy, "E": 0.5 * rho0 * vy * vy}


def shear(N=800):
    """hydro_cpu.cpp:682-694: small elastic shear pulse in basalt."""
    m = ic.basalt()
    dx, f = _pulse(N, 400e3, 1.0)
    cs = math.sqrt(m["G"] / 2700.0)
    return Case("shear", (N, 1, 1), dx, m, {}, f, 0.3, 20e3 / cs)


def yield_pulse(N=400):
    """hydro_cpu.cpp:695-703: shear pulse driven past the von Mises surface."""
    m = ic.basalt()
    dx, f = _pulse(N, 400e3, 2000.0)
    cs = math.sqrt(m["G"] / 2700.0)
    return Case("yield", (N, 1, 1), dx, m, {}, f, 0.3, 15e3 / cs)


def vacuum(N=400):
    """hydro_cpu.cpp:704-715: expansion into vacuum with the vacuum-aware flux."""
    dx = 1.0 / N
    x = _centres(N, dx)
    left = x < 0.5
    r = np.where(left, 1.0, 1e-6)
    E = np.where(left, 1.0 / (GAM - 1), 1e-6 / (GAM - 1))
    return Case("vacuum", (N, 1, 1), dx, ic.ideal_gas(GAM), {"rho_vac": 1e-3}, {"r": r, "E": E}, 0.4, 0.10)


def bshock(N=400):
    """hydro_cpu.cpp:716-720: basalt shock tube (Tillotson)."""
    L = 400e3
    dx = L / N
    x = _centres(N, dx)
    rr = np.where(x < 0.5 * L, 3000.0, 2700.0)
    ee = np.where(x < 0.5 * L, 1e6, 0.0)
    return Case("bshock", (N, 1, 1), dx, ic.basalt(), {}, {"r": rr, "E": rr * ee}, 0.4, 4.0)


def freefall(N=50):
    """hydro_cpu.cpp:721-727: uniform gas under gravity."""
    return Case("freefall", (1, 1, N), 10.0, ic.ideal_gas(GAM), {"gz": 9.8},
                {"r": np.ones(N), "E": np.full(N, 1e5 / (GAM - 1))}, 0.4, 10.0)


def atmos(N=200):
    """hydro_cpu.cpp:728-735: isothermal atmosphere under gravity."""
    gz, P0, rho0 = 9.8, 1e5, 1.0
    H = P0 / (rho0 * gz)
    L = 4 * H
    dx = L / N
    z = _centres(N, dx)
    cs = math.sqrt(GAM * P0 / rho0)
    f = {"r": rho0 * np.exp(-z / H), "E": (P0 * np.exp(-z / H)) / (GAM - 1)}
    return Case("atmos", (1, 1, N), dx, ic.ideal_gas(GAM), {"gz": gz}, f, 0.4, 0.05 * L / cs)


def tensile(N=100):
    """hydro_cpu.cpp:736-743: a stretched basalt bar (tensile damage)."""
    L, rho0, rate = 10e3, 2700.0, 1e-2
    dx = L / N
    x = _centres(N, dx)
    vx = rate * (x - 0.5 * L)
    return Case("tensile", (N, 1, 1), dx, ic.basalt(), {},
                {"r": np.full(N, rho0), "mu": rho0 * vx, "E": 0.5 * rho0 * vx * vx}, 0.3, 0.1)


def alimpact(N=400):
    """hydro_cpu.cpp:744-752: symmetric Al-on-Al planar impact."""
    L, rho0, up = 2.0, 2700.0, 5000.0
    dx = L / N
    x = _centres(N, dx)
    vx = np.where(x < 0.5 * L, up, -up)
    return Case("alimpact", (N, 1, 1), dx, aluminum(), {},
                {"r": np.full(N, rho0), "mu": rho0 * vx, "E": 0.5 * rho0 * vx * vx}, 0.3, 3e-5)


def surface(N=64):
    """hydro_cpu.cpp:901-905: a basalt half-space with a near-void above."""
    L = 200e3
    dx = L / N
    z = _centres(N, dx)
    return Case("surface", (1, 1, N), dx, ic.basalt(), {},
                {"r": np.where(z < 0.5 * L, 2700.0, 0.27), "E": np.zeros(N)}, 0.4, 2.0)


def impact3d(N=64, a_cells=None, speed=8000.0, angle_deg=30.0, af=False, t_end=None):
    """3-D Cartesian impact: a basalt sphere (radius a_cells cells, default N/16)
    at speed (m/s) and angle_deg from vertical into a basalt half-space filling
    the lower half of an N^3 grid of 50 m cells, near-void (0.27 kg/m^3) above.
    Strength with the pressure-dependent ROCK yield, tensile damage, gravity
    3.71 m/s^2, near-void cells out of CFL and strength (rho < 100), and
    optionally shock-activated acoustic fluidization."""
    dx = 50.0
    a = float(a_cells if a_cells is not None else max(2.0, N / 16))
    n = N * N * N
    c = _centres(N, dx)
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    rho0 = 2700.0
    zs = 0.5 * N * dx
    r = np.where(Z < zs, rho0, 0.27)
    th = math.radians(angle_deg)
    cx, cy, cz = 0.5 * N * dx - 2.0 * a * dx * math.sin(th), 0.5 * N * dx, zs + (a + 1.0) * dx
    sphere = (X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2 < (a * dx) ** 2
    r = np.where(sphere, rho0, r)
    vx = np.where(sphere, speed * math.sin(th), 0.0)
    vz = np.where(sphere, -speed * math.cos(th), 0.0)
    f = {"r": r.reshape(-1), "mu": (r * vx).reshape(-1), "mw": (r * vz).reshape(-1),
         "E": (0.5 * r * (vx * vx + vz * vz)).reshape(-1), "rc": np.where(sphere, r, 0.0).reshape(-1)}
    prm = {"rock": 1, "gz": 3.71, "rho_cfl": 100.0}
    if af:
        prm.update(tdec=2.0, eta_af=1e7, c_act=0.1)
    if t_end is None:
        t_end = 4.0 * a * dx / speed
    return Case(f"impact3d_{N}", (N, N, N), dx, ic.basalt(), prm, f, 0.3, t_end)


def substrate(N=60):
    """hydro_cpu.cpp:847-859: a gravity-loaded lithostatic basalt substrate
    under the well-balanced reconstruction must stay at rest (t_end 200 s,
    the two deepest layers pinned to the reference after every step)."""
    gz, rho0, A, dx, zsurf = 3.71, 2700.0, 2.67e10, 500.0, 20e3
    z = _centres(N, dx)
    col = np.where(z < zsurf, rho0 * (1.0 + rho0 * gz * (zsurf - z) / A), 0.27)
    r = np.tile(col, N)  # (i, k) with k fastest
    return Case("substrate", (N, 1, N), dx, ic.basalt(), {"gz": gz, "damp": 1.0, "rho_cfl": 100.0},
                {"r": r, "E": np.zeros(N * N)}, 0.4, 200.0, set_ref=True, pin_floor=2)


def crater(cppr=4, Rfac=8.0, Zfac=8.0, a=500.0, U=12000.0, tdec=0.0, eta_af=0.0, gz=3.71, t_end=None,
           void_cons=0, void_amb=0.0, visc_imp=0):
    """hydro_cpu.cpp:557-597: the axisymmetric vertical impact crater -- a
    basalt sphere of radius a on the axis, tangent to the surface, at U m/s
    into a lithostatic basalt half-space under gravity, with the frozen
    pre-impact column as the well-balanced reference, ROCK yield, near-void
    and vacuum-aware faces, and (tdec > 0) shock-activated fluidization with
    the crater defaults (acoustic seeding, overburden relief); void_cons /
    void_amb select the conservative and ambient void resets (its arguments 17
    and 14), visc_imp the implicit fluidization viscosity (argument 16).  The
    driver's far-field floor pin and radial sponge are not part of the case."""
    rho0, Abulk = 2700.0, 2.67e10
    dx = a / cppr
    Nr, Nz = int(Rfac * a / dx + 0.5), int(Zfac * a / dx + 0.5)
    zsurf = Nz * dx - 5.0 * a
    rr = _centres(Nr, dx)[:, None]
    zz = _centres(Nz, dx)[None, :]
    r = np.where(zz < zsurf, rho0 * (1.0 + rho0 * gz * (zsurf - zz) / Abulk), 0.27) * np.ones_like(rr)
    zc = zsurf + a
    sph_ = np.sqrt(rr * rr + (zz - zc) * (zz - zc)) < a
    post = {"r": np.where(sph_, rho0, r).reshape(-1), "mw": np.where(sph_, -rho0 * U, 0.0).reshape(-1),
            "E": np.where(sph_, 0.5 * rho0 * U * U, 0.0).reshape(-1)}
    prm = {"axisym": 1, "rho_cfl": 100.0, "rho_vac": 100.0, "rock": 1, "gz": gz}
    if tdec > 0:
        prm.update(tdec=tdec, eta_af=eta_af, c_act=0.5, p_coh=1.0e6, p_act=1.0e8, af_seeddp=1, af_prel=1)
    if void_cons or void_amb:
        prm.update(void_cons=int(void_cons), void_amb=float(void_amb))
    if visc_imp:
        prm.update(visc_imp=1)
    if t_end is None:
        t_end = 2.0 * math.sqrt((Rfac * a) / gz)
    name = f"crater_{cppr}" + ("_vc" if void_cons else "") + ("_amb" if void_amb else "") + ("_vi" if visc_imp else "")
    return Case(name, (Nr, 1, Nz), dx, ic.basalt(), prm,
                {"r": r.reshape(-1), "E": np.zeros(Nr * Nz)}, 0.4, t_end, set_ref=True, post_ref=post)


def visc_mode(N=256, m=4, nu=1.0):
    """hydro_cpu.cpp:907-929 (visc_diff A): a fluidized ideal-gas slab of N
    unit cells, rho 1, eta = nu, carrying the transverse cosine mode
    v_y = cos(k x), v_z = v_y / 2 (k = m pi / L, the discrete Neumann
    eigenmode); the gate applies the implicit viscosity at 20x the explicit
    limit."""
    dx, rho0 = 1.0, 1.0
    kk = m * math.pi / (N * dx)
    vy = np.cos(kk * (np.arange(N) + 0.5) * dx)  # k (i + 1/2) dx, the reference's order
    mv, mw = rho0 * vy, 0.5 * rho0 * vy
    f = {"r": np.full(N, rho0), "af": np.ones(N), "mv": mv, "mw": mw,
         "E": 1e5 + 0.5 * (mv * mv + mw * mw) / rho0}
    return Case("visc_mode", (N, 1, 1), dx, ic.ideal_gas(GAM), {"visc_imp": 1, "eta_af": nu * rho0}, f, 0.4, 0.0)


def visc_axi(Nr=64, Nz=8, A0=1e-2, W0=3.0, nu=1.0):
    """hydro_cpu.cpp:930-944 (visc_diff B): cylindrical, v_r = A0 r (an exact
    null mode of the discrete operator) and v_z = W0 in a fluidized ideal gas."""
    dx, rho0 = 1.0, 1.0
    rr = _centres(Nr, dx)[:, None] * np.ones((1, Nz))
    mu, mw = rho0 * A0 * rr, rho0 * W0 * np.ones_like(rr)
    f = {"r": np.full(Nr * Nz, rho0), "af": np.ones(Nr * Nz), "mu": mu.reshape(-1), "mw": mw.reshape(-1),
         "E": (1e5 + 0.5 * (mu * mu + mw * mw) / rho0).reshape(-1)}
    return Case("visc_axi", (Nr, 1, Nz), dx, ic.ideal_gas(GAM), {"visc_imp": 1, "eta_af": nu * rho0, "axisym": 1},
                f, 0.4, 0.0)


def visc_slab(eta=1e8, A0=1.0, t_end=25.0, N=256, m=24, visc_imp=1):
    """hydro_cpu.cpp:947-987 (visc_agree, visc_energy): a fluidized basalt
    slab (af = 1, so no strength) of N 500 m cells carrying a transverse cosine
    shear mode of amplitude A0 m/s, viscosity eta, CFL 0.4; visc_imp 0 runs the
    Lop's explicit viscosity instead."""
    dx = 500.0
    rho0 = 2700.0
    kk = m * math.pi / (N * dx)
    vy = A0 * np.cos(kk * (np.arange(N) + 0.5) * dx)
    f = {"r": np.full(N, rho0), "af": np.ones(N), "mv": rho0 * vy, "E": 0.5 * rho0 * vy * vy}
    return Case(f"visc_slab_{'imp' if visc_imp else 'exp'}_{eta:.0e}", (N, 1, 1), dx, ic.basalt(),
                {"visc_imp": int(visc_imp), "eta_af": float(eta)}, f, 0.4, t_end)


def vib_slab(case=2, t_end=40.0, N=256, m=24):
    """hydro_cpu.cpp:988-1027 (vib_regen): a yielding-soft basalt slab
    (Y = 1 MPa) with vibrations vib0 = 10 m/s, a 10 m/s cosine shear mode,
    implicit viscosity 5e8 Pa s, decay time 2 s, no shock re-seeding; case 0
    without regeneration bookkeeping, 1 with it at C_REG = 0, 2 with
    C_REG = 1."""
    dx, A0, vib0 = 500.0, 10.0, 10.0
    mat = dict(ic.basalt())
    mat["Y"] = 1e6
    rho0 = mat["rho0"]
    kk = m * math.pi / (N * dx)
    vy = A0 * np.cos(kk * (np.arange(N) + 0.5) * dx)
    f = {"r": np.full(N, rho0), "vib": np.full(N, vib0), "Pmax": np.full(N, 1e30), "mv": rho0 * vy,
         "E": 0.5 * rho0 * vy * vy}
    prm = {"visc_imp": 1, "eta_af": 5e8, "tdec": 2.0, "c_act": 0.5, "p_act": 1e30, "p_coh": 1e6,
           "af_reg": int(case > 0), "c_reg": 0.0 if case < 2 else 1.0, "af_sat": 1e9}
    return Case(f"vib_slab_{case}", (N, 1, 1), dx, mat, prm, f, 0.4, t_end)


def bingham_heap(case=1, NX=112, NZ=20):
    """hydro_cpu.cpp:1028-1077 (bingham_slope): a fluidized triangular basalt
    heap (H 2 km, half-width 6 km) on an intact lithostatic substrate in x-z,
    gravity 3.71, ROCK yield, implicit viscosity 5e7 Pa s, voids reset to the
    ambient density, and the Bingham floor Y_B of the case: 0 static
    (2.5 x the peak flank stress), 1 arrest (0.2 x), 2 Newtonian control (0);
    run for 400 / 1200 / 600 s with the two deepest layers pinned to the
    reference."""
    rho0, Ab, gz, dx = 2700.0, 2.67e10, 3.71, 250.0
    z0, H, W = 1500.0, 2000.0, 6000.0
    xc = 0.5 * NX * dx
    taumax = rho0 * gz * H * (H / W)
    yb = (2.5 * math.sqrt(3.0) * taumax, 0.2 * math.sqrt(3.0) * taumax, 0.0)[case]
    x = _centres(NX, dx)[:, None]
    z = _centres(NZ, dx)[None, :]
    xx = np.abs(x - xc)
    zs = z0 + np.where(xx < W, H * (1.0 - xx / W), 0.0)
    r = np.where(z < zs, rho0 * (1.0 + rho0 * gz * (zs - z) / Ab), 0.27) * np.ones((NX, NZ))
    af = np.where(z > z0, 1.0, 0.0) * np.ones((NX, NZ))
    prm = {"gz": gz, "rock": 1, "rho_cfl": 100.0, "rho_vac": 100.0, "visc_imp": 1, "eta_af": 5e7,
           "void_amb": 0.27, "y_bingham": yb}
    return Case(f"bingham_{case}", (NX, 1, NZ), dx, ic.basalt(), prm,
                {"r": r.reshape(-1), "E": np.zeros(NX * NZ), "af": af.reshape(-1)}, 0.4,
                (400.0, 1200.0, 600.0)[case], set_ref=True, pin_floor=2)


def lame_hoop(Nr=40, edot=1e-6):
    """hydro_cpu.cpp:490-501 (lame A): a cylindrical basalt column in uniform
    radial expansion u = edot r, unstressed; one Lop gives the hoop strain
    rate's stress rates."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    mu = rho0 * edot * ((np.arange(Nr) + 0.5) * dx)
    return Case("lame_hoop", (Nr, 1, 1), dx, ic.basalt(), {"axisym": 1},
                {"r": np.full(Nr, rho0), "E": np.zeros(Nr), "mu": mu})


def lame_equilibrium(Nr=200, ia=20, ib=180):
    """hydro_cpu.cpp:502-516 (lame B): the deviatoric stress of a thick
    cylinder under internal pressure (S_rr = -B/r^2, S_thth = B/r^2) at rest;
    one Lop's radial momentum balance."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    ia_r = (ia + 0.5) * dx
    bc = 2.0e6 * ia_r * ia_r
    rr = (np.arange(Nr) + 0.5) * dx
    inside = (np.arange(Nr) >= ia) & (np.arange(Nr) <= ib)
    sxx = np.where(inside, -bc / (rr * rr), 0.0)
    syy = np.where(inside, bc / (rr * rr), 0.0)
    return Case("lame_equilibrium", (Nr, 1, 1), dx, ic.basalt(), {"axisym": 1},
                {"r": np.full(Nr, rho0), "E": np.zeros(Nr), "Sxx": sxx, "Syy": syy})


def af_visc_column(af, Nr=120, A=1e-9, eta=1e9):
    """hydro_cpu.cpp:519-529 (af_visc): u = A r^2 in a cylindrical basalt
    column, fluidized (af = 1) or not, explicit fluidization viscosity eta."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    r = (np.arange(Nr) + 0.5) * dx
    return Case(f"af_visc_{af}", (Nr, 1, 1), dx, ic.basalt(), {"axisym": 1, "eta_af": eta},
                {"r": np.full(Nr, rho0), "E": np.zeros(Nr), "mu": rho0 * A * r * r, "af": np.full(Nr, float(af))})


def vib_advect(N=200, v0=2000.0):
    """hydro_cpu.cpp:530-539 (vib_advect): a Gaussian vibration bump in basalt
    moving uniformly at v0 for 20 km (CFL 0.4)."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    x0, wid = 0.3 * N * dx, 8e3
    x = (np.arange(N) + 0.5) * dx
    return Case("vib_advect", (N, 1, 1), dx, ic.basalt(), {},
                {"r": np.full(N, rho0), "mu": np.full(N, rho0 * v0), "E": np.full(N, 0.5 * rho0 * v0 * v0),
                 "vib": np.exp(-((x - x0) / wid) * ((x - x0) / wid))}, 0.4, 20e3 / v0)


def af_shock(N=200, V=2000.0):
    """hydro_cpu.cpp:865-873 (af_activate A): the left half of a basalt bar
    moving at V into the right half, fluidization seeding on (TDEC 10 s,
    C_ACT 0.5), for 3 s."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    mu = np.where(np.arange(N) < N // 2, rho0 * V, 0.0)
    return Case("af_shock", (N, 1, 1), dx, ic.basalt(), {"tdec": 10.0, "c_act": 0.5, "eta_af": 0.0},
                {"r": np.full(N, rho0), "E": np.zeros(N), "mu": mu}, 0.4, 3.0)


def af_decay(M=50, vib0=80.0):
    """hydro_cpu.cpp:874-880 (af_activate B): basalt at rest with vibrations
    vib0 (TDEC 0.5 s, C_ACT 0.5), for 5 s."""
    dx, rho0 = 500.0, ic.basalt()["rho0"]
    return Case("af_decay", (M, 1, 1), dx, ic.basalt(), {"tdec": 0.5, "c_act": 0.5, "eta_af": 0.0},
                {"r": np.full(M, rho0), "E": np.zeros(M), "vib": np.full(M, vib0)}, 0.4, 5.0)


def collapse(af_on, NX=80, NZ=40):
    """hydro_cpu.cpp:883-900 (collapse): a lithostatic basalt step (14 km /
    10 km) under gravity 3.71 with its column as the reference, fluidized
    (af = 1, TDEC 1e6, explicit viscosity 1e9) or not, for 8 s with the two
    lowest layers held (stress included)."""
    rho0, A, gz, dx = 2700.0, 2.67e10, 3.71, 500.0
    zlo, zhi = 10e3, 14e3
    x = ((np.arange(NX) + 0.5) * dx)[:, None]
    z = ((np.arange(NZ) + 0.5) * dx)[None, :]
    zs = np.where(x < 0.5 * NX * dx, zhi, zlo)
    solid = z < zs
    r = np.where(solid, rho0 * (1.0 + rho0 * gz * (zs - z) / A), 0.27)
    prm = {"gz": gz, "rho_cfl": 100.0, "rho_vac": 100.0, "tdec": 1e6 if af_on else 0.0,
           "eta_af": 1e9 if af_on else 0.0}
    f = {"r": r.reshape(-1), "E": np.zeros(NX * NZ)}
    if af_on:
        f["af"] = np.where(solid, 1.0, 0.0).reshape(-1)
    return Case(f"collapse_{'af' if af_on else 'rigid'}", (NX, 1, NZ), dx, ic.basalt(), prm, f, 0.4, 8.0,
                set_ref=True, pin_floor=2, driver_flags=1)


def pierazzo2d(cppr=12.0, reach=12.0, U=5000.0, t_end=-1.0):
    """hydro_cpu.cpp:753-798 (pierazzo2d): Pierazzo et al. 2008's Al-on-Al
    benchmark, axisymmetric: an aluminium sphere of radius 1 m (no gravity:
    scale-free) at U into an aluminium half-space, strengthless, ambient gas
    above; CFL 0.3 until the shock has crossed 1.3 reach radii; the peak
    pressure of every cell recorded after each step."""
    mat = aluminum()
    a, dx, rho0 = 1.0, 1.0 / cppr, mat["rho0"]
    zsurf, zc = reach * a, reach * a + a
    nr, nz = int(reach * a / dx + 0.5), int((reach + 3.0) * a / dx + 0.5)
    r = ((np.arange(nr) + 0.5) * dx)[:, None]
    z = ((np.arange(nz) + 0.5) * dx)[None, :]
    proj = np.sqrt(r * r + (z - zc) * (z - zc)) < a
    dens = np.where(proj | (z < zsurf), rho0, 0.27) * np.ones((nr, nz))
    f = {"r": dens.reshape(-1), "mw": np.where(proj, -rho0 * U, 0.0).reshape(-1),
         "E": np.where(proj, 0.5 * rho0 * U * U, 0.0).reshape(-1)}
    c0 = math.sqrt(mat["A"] / rho0)
    return Case(f"pierazzo2d_{U:.0f}", (nr, 1, nz), dx, mat, {"axisym": 1}, f, 0.3,
                t_end if t_end > 0 else 1.3 * reach * a / c0, driver_flags=4)


def prater(cppr=10.0, U=7000.0, Y=414e6, G=27.6e9, Rfac=8.0, t_end=70e-6, rho_cfl=100.0):
    """hydro_cpu.cpp:799-846 (prater): Prater 1970's aluminium crater growth,
    axisymmetric: a 3.175 mm aluminium sphere at U into aluminium with von
    Mises strength Y and shear modulus G, vacuum-aware faces, CFL 0.3, the
    near-void cells reset to ambient gas after each step, for t_end."""
    mat = dict(aluminum())
    mat["Y"], mat["G"] = float(Y), float(G)
    a = 3.175e-3
    dx, rho0 = a / cppr, mat["rho0"]
    nr, nz = int(Rfac * a / dx + 0.5), int((Rfac + 3.0) * a / dx + 0.5)
    zsurf, zc = Rfac * a, Rfac * a + a
    r = ((np.arange(nr) + 0.5) * dx)[:, None]
    z = ((np.arange(nz) + 0.5) * dx)[None, :]
    proj = np.sqrt(r * r + (z - zc) * (z - zc)) < a
    dens = np.where(proj | (z < zsurf), rho0, 0.27) * np.ones((nr, nz))
    f = {"r": dens.reshape(-1), "mw": np.where(proj, -rho0 * U, 0.0).reshape(-1),
         "E": np.where(proj, 0.5 * rho0 * U * U, 0.0).reshape(-1)}
    return Case(f"prater_{cppr:g}", (nr, 1, nz), dx, mat, {"axisym": 1, "rho_vac": 100.0, "rho_cfl": float(rho_cfl)},
                f, 0.3, t_end, driver_flags=2)


GATES = {"sod": sod, "tracer": tracer, "sedov": sedov, "sedov_axi": sedov_axi, "shear": shear,
         "yield": yield_pulse, "vacuum": vacuum, "bshock": bshock, "freefall": freefall, "atmos": atmos,
         "tensile": tensile, "alimpact": alimpact, "surface": surface}
