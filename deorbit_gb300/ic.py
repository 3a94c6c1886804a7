"""Seeded synthetic initial conditions for the impact workloads.

Every workload is a `Scenario`: particle arrays in the reference's IC layout
(x y z vx vy vz mass u mat fixed, run_ic.cpp:4-6), a domain, the System
parameters (sph.hpp:86-92) and a material list.  The same Scenario feeds the
CUDA solver and the CPU oracle, so both see bit-identical inputs.

Workloads (sizes as named; all from numpy's seeded PCG64 generator):
  impact_halfspace  granite half-space lattice + iron sphere, hydro only
                    (48x48x24 + r = 8 dx sphere, 45 deg, 8 km/s, CFL 0.3)
  grazing           iron sphere of 1 km into a granite slab at a shallow angle,
                    strength (von Mises iron, Collins granite) + multi-flaw
                    damage; total particle count chosen exactly
  sheared_cube      the reference oracle-dump scenario (cpu_dump.cpp:12-40):
                    sheared, compressed basalt cube with an iron core, frac on
  batch             many independent impacts with log-uniform sizes
Materials: granite = the Tillotson set named for these workloads; its shear
modulus (24 GPa), Collins parameters (Y0 10 MPa, mu_i 1.5, Ylim 3.5 GPa, mu_d
0.6) and Weibull constants (m 9, k 4e35 m^-3) are this build's choices, as is
using the reference iron set (eos.hpp:42-43) for the impactor.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

MAT_FIELDS = "type yield_model gamma rho0 a b A B alpha beta u0 uiv ucv G Y Emod wm wk Y0 mu_i Ylim Yd0 mu_d".split()


def tillotson(rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, G=0.0, Y=0.0, wm=0.0, wk=0.0, **ext):
    """Material dict with the fields of eos.hpp:15-27 (Emod = 9AG/(3A+G), eos.hpp:37)."""
    m = dict(type=1, yield_model=0, gamma=1.4, rho0=rho0, a=a, b=b, A=A, B=B, alpha=alpha, beta=beta,
             u0=u0, uiv=uiv, ucv=ucv, G=G, Y=Y, Emod=(9.0 * A * G / (3.0 * A + G) if G > 0 else 0.0),
             wm=wm, wk=wk, Y0=0.0, mu_i=0.0, Ylim=0.0, Yd0=0.0, mu_d=0.0)
    m.update(ext)
    return m


def ideal_gas(gamma):
    """Ideal-gas material dict (eos.hpp:29): P = (gamma - 1) rho u."""
    m = {k: 0.0 for k in MAT_FIELDS}
    m.update(type=0, yield_model=0, gamma=gamma)
    return m


def iron(strength=True):
    """Reference iron set (eos.hpp:42-43); strength=False drops G and Y (hydro only)."""
    return tillotson(7800, 1.28e11, 1.05e11, 0.5, 1.5, 5, 5, 9.5e6, 2.4e6, 8.67e6,
                     *((7.75e10, 1.0e9) if strength else (0.0, 0.0)))


def basalt():
    return tillotson(2700, 2.67e10, 2.67e10, 0.5, 1.5, 5, 5, 4.87e8, 4.72e6, 1.82e7, 2.27e10, 3.5e8, 16.0, 1.0e61)


def granite(strength=True):
    """Granite Tillotson set (rho0 2680, A = B = 18 GPa, E0 16, Eiv 3.5, Ecv 18 MJ/kg,
    a 0.5, b 1.3, alpha = beta = 5) with this build's strength / flaw constants."""
    if not strength:
        return tillotson(2680, 1.8e10, 1.8e10, 0.5, 1.3, 5, 5, 1.6e7, 3.5e6, 1.8e7)
    return tillotson(2680, 1.8e10, 1.8e10, 0.5, 1.3, 5, 5, 1.6e7, 3.5e6, 1.8e7,
                     G=2.4e10, Y=3.5e9, wm=9.0, wk=4.0e35,
                     yield_model=1, Y0=1.0e7, mu_i=1.5, Ylim=3.5e9, Yd0=0.0, mu_d=0.6)


@dataclasses.dataclass
class Scenario:
    name: str
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    u: np.ndarray
    mat: np.ndarray
    fixed: np.ndarray
    lo: np.ndarray
    hi: np.ndarray
    periodic: np.ndarray
    params: dict
    materials: list
    dx: float
    flaws: tuple | None = None      # ("single" | "multi", seed)
    h0: np.ndarray | None = None

    @property
    def n(self):
        return int(self.pos.shape[0])


def lattice(nx, ny, nz, dx, origin=(0.0, 0.0, 0.0)):
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    return np.asarray(origin, float) + (p + 0.5) * dx


def sphere(R, dx, center):
    m = int(math.ceil(R / dx)) + 1
    g = (np.arange(-m, m) + 0.5) * dx
    i, j, k = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    p = p[(p * p).sum(1) < R * R]
    return p + np.asarray(center, float)


def _jitter(p, dx, frac, rng):
    return p + rng.uniform(-frac * dx, frac * dx, size=p.shape)


def impact_halfspace(nx=48, ny=48, nz=24, dx=10.0, r_cells=8.0, angle_deg=45.0, speed=8000.0,
                     jitter=0.01, cfl=0.3, seed=20261203):
    """Hydro-only iron sphere into a granite half-space (FP64 plain workload)."""
    rng = np.random.default_rng(seed)
    tgt = _jitter(lattice(nx, ny, nz, dx, (0.0, 0.0, -nz * dx)), dx, jitter, rng)
    R = r_cells * dx
    th = math.radians(angle_deg)
    cx = 0.5 * nx * dx - (R + dx) / math.tan(th) if angle_deg < 89 else 0.5 * nx * dx
    imp = _jitter(sphere(R, dx, (cx, 0.5 * ny * dx, R + dx)), dx, jitter, rng)
    pos = np.concatenate([tgt, imp])
    n_t = tgt.shape[0]
    vel = np.zeros_like(pos)
    vel[n_t:, 0] = speed * math.cos(th)
    vel[n_t:, 2] = -speed * math.sin(th)
    mat = np.r_[np.zeros(n_t, np.int32), np.ones(imp.shape[0], np.int32)]
    mats = [granite(strength=False), iron(strength=False)]
    mass = np.where(mat == 1, mats[1]["rho0"], mats[0]["rho0"]) * dx ** 3
    L = np.array([nx, ny, nz]) * dx
    lo = np.array([-0.25 * L[0], -0.25 * L[1], -L[2] - 0.25 * L[2]])
    hi = np.array([1.25 * L[0], 1.25 * L[1], 0.75 * L[2]])
    return Scenario("impact_halfspace", pos, vel, mass, np.zeros(pos.shape[0]), mat,
                    np.zeros(pos.shape[0], np.uint8), lo, hi, np.zeros(3, np.int32),
                    dict(eta=1.3, h_init=1.3 * dx, alpha=1.0, beta=2.0, eps=0.01, cfl=cfl,
                         eps_as=0.0, damage_on=0), mats, dx)


def grazing(n_total=1 << 20, radius=500.0, dx=None, angle_deg=3.0, speed=8000.0, jitter=0.01,
            aspect=(8.0, 4.0, 1.0), seed=20261203, flaws="multi", eps_as=0.3, cfl=0.2, gap=1.0):
    """Strength + damage grazing impact: iron sphere (von Mises, 1 GPa) into a
    granite slab (Collins yield, multi-flaw Weibull), exactly n_total particles.
    The sphere's lowest point starts `gap` lattice spacings above the surface."""
    rng = np.random.default_rng(seed)
    if dx is None:  # slab of aspect ax:ay:az (in sphere diameters) holding n_total
        vol = (n_total * 1.0) / 1.0
        D = 2 * radius
        ax, ay, az = aspect
        dx = (ax * ay * az * D ** 3 / vol) ** (1.0 / 3.0)
    R = radius
    imp = sphere(R, dx, (0.0, 0.0, 0.0))
    n_imp = imp.shape[0]
    n_slab = n_total - n_imp
    ax, ay, az = aspect
    D = 2 * R
    nz = max(2, int(round(az * D / dx)))
    ny = max(2, int(round(ay * D / dx)))
    nx = int(math.ceil(n_slab / (ny * nz)))
    slab = lattice(nx, ny, nz, dx, (0.0, -0.5 * ny * dx, -nz * dx))
    # drop surplus particles from the bottom of the far end (away from the track)
    order = np.lexsort((slab[:, 2], -slab[:, 0]))  # far x first, bottom first
    keep = np.ones(slab.shape[0], bool)
    keep[order[: slab.shape[0] - n_slab]] = False
    slab = slab[keep]
    th = math.radians(angle_deg)
    x0 = 0.15 * nx * dx
    cen = np.array([x0, 0.0, R + gap * dx])
    imp = imp + cen
    slab = _jitter(slab, dx, jitter, rng)
    imp = _jitter(imp, dx, jitter, rng)
    pos = np.concatenate([slab, imp])
    vel = np.zeros_like(pos)
    vel[n_slab:, 0] = speed * math.cos(th)
    vel[n_slab:, 2] = -speed * math.sin(th)
    mat = np.r_[np.zeros(n_slab, np.int32), np.ones(n_imp, np.int32)]
    mats = [granite(strength=True), iron(strength=True)]
    mass = np.where(mat == 1, mats[1]["rho0"], mats[0]["rho0"]) * dx ** 3
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    lo = np.array([-0.1 * Lx - 2 * R, -0.5 * Ly - 0.5 * Ly, -Lz - 0.5 * Lz])
    hi = np.array([1.1 * Lx, 0.5 * Ly + 0.5 * Ly, 4 * R + 0.5 * Lz])
    return Scenario("grazing", pos, vel, mass, np.zeros(pos.shape[0]), mat,
                    np.zeros(pos.shape[0], np.uint8), lo, hi, np.zeros(3, np.int32),
                    dict(eta=1.3, h_init=1.3 * dx, alpha=1.0, beta=2.0, eps=0.01, cfl=cfl,
                         eps_as=eps_as, damage_on=1, flaw_model=1 if flaws == "multi" else 0),
                    mats, dx, flaws=(flaws, 12345))


def sheared_cube(L=22, dx=30.0):
    """The reference's oracle-dump state builder (cpu_dump.cpp:12-31)."""
    lo = -L * dx / 2.0
    hi = L * dx / 2.0
    p = lattice(L, L, L, dx, (lo, lo, lo))
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    R = 5.0 * dx
    ir = (x * x + y * y + z * z) < R * R
    vel = np.stack([80.0 * (y / hi), np.zeros_like(x), -40.0 * (z / hi)], axis=1)
    u = 2.0e5 * (1.0 + x / hi)
    mats = [basalt(), iron()]
    mass = np.where(ir, 7800.0, 2700.0) * dx ** 3
    return Scenario("sheared_cube", p, vel, mass, u, ir.astype(np.int32), np.zeros(p.shape[0], np.uint8),
                    np.full(3, lo - dx), np.full(3, hi + dx), np.zeros(3, np.int32),
                    dict(eta=1.3, h_init=1.3 * dx, eps_as=0.3, damage_on=1), mats, dx, flaws=("single", 12345))


def periodic_bar(nx=24, ny=6, dx=0.01, seed=7):
    """Basalt bar, periodic in y and z, Gaussian velocity pulse, frozen ends
    (the wave-speed gate's geometry, strength_test.cpp:95-110, scaled down)."""
    x0, x1, Lyz = -nx * dx / 2, nx * dx / 2, ny * dx
    p = lattice(nx, ny, ny, dx, (x0, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    p = _jitter(p, dx, 0.05, rng)
    vel = np.zeros_like(p)
    vel[:, 0] = np.exp(-(p[:, 0] ** 2) / (0.06 * nx * dx / 1.2) ** 2)
    fixed = (np.abs(p[:, 0]) > 0.45 * nx * dx).astype(np.uint8)
    mats = [basalt()]
    mass = np.full(p.shape[0], mats[0]["rho0"] * dx ** 3)
    return Scenario("periodic_bar", p, vel, mass, np.zeros(p.shape[0]), np.zeros(p.shape[0], np.int32), fixed,
                    np.array([x0, 0.0, 0.0]), np.array([x1, Lyz, Lyz]), np.array([0, 1, 1], np.int32),
                    dict(eta=1.3, h_init=1.3 * dx), mats, dx)


def sod_tube(a_left=0.005, nx_left=100, ny_left=16, gamma=1.4):
    """3D Sod shock tube (the reference's first validation gate, sod.cpp:8-50):
    ideal gas, a thin slab periodic in y and z, density 1 / 0.125 and pressure
    1 / 0.1 across x = 0 from lattices of spacing a and 2a (equal masses),
    particles within 2 h_init of either end frozen; artificial viscosity
    alpha 1, beta 2 and conductivity alpha_u 1."""
    aL, aR = a_left, 2.0 * a_left
    nxR, nyR = nx_left // 2, ny_left // 2
    h_init = 1.3 * aL
    xfix = 2.0 * h_init
    rhoL, PL, PR = 1.0, 1.0, 0.1
    rhoR = 0.125
    m = rhoL * aL ** 3
    left = lattice(nx_left, ny_left, ny_left, aL, (-0.5, 0.0, 0.0))
    right = lattice(nxR, nyR, nyR, aR, (0.0, 0.0, 0.0))
    pos = np.concatenate([left, right])
    nL = left.shape[0]
    u = np.r_[np.full(nL, PL / ((gamma - 1.0) * rhoL)), np.full(right.shape[0], PR / ((gamma - 1.0) * rhoR))]
    fixed = ((pos[:, 0] < -0.5 + xfix) & (np.arange(pos.shape[0]) < nL)) | \
            ((pos[:, 0] > 0.5 - xfix) & (np.arange(pos.shape[0]) >= nL))
    mats = [ideal_gas(gamma)]
    Lyz = ny_left * aL
    return Scenario("sod_tube", pos, np.zeros_like(pos), np.full(pos.shape[0], m), u,
                    np.zeros(pos.shape[0], np.int32), fixed.astype(np.uint8),
                    np.array([-0.5, 0.0, 0.0]), np.array([0.5, Lyz, Lyz]), np.array([0, 1, 1], np.int32),
                    dict(eta=1.3, h_init=h_init, alpha=1.0, beta=2.0, eps=0.01, alpha_u=1.0, cfl=0.2),
                    mats, aL)


def _graded_layers(dx0, growth, L):
    """Depth layers of a slab graded in z: spacing dx0 * growth^k from the
    surface down; returns [(spacing, z_center, nx, ny)]."""
    Lx, Ly, Lz = L
    out, ztop, s = [], 0.0, dx0
    while ztop < Lz:
        nx, ny = int(Lx // s), int(Ly // s)
        out.append((s, -(ztop + 0.5 * s), nx, ny))
        ztop += s
        s *= growth
    return out


def large_graded(n_total=1 << 24, L=(40.0e3, 20.0e3, 5.0e3), radius=500.0, angle_deg=2.0, speed=8000.0,
                 growth=1.06, jitter=0.01, seed=20261203):
    """Large grazing run: iron sphere (radius 500 m) at 2 deg, 8 km/s into a
    40 x 20 x 5 km granite slab whose lattice spacing grows with depth by
    `growth` per layer (fine at the surface where the impactor runs, coarse at
    depth).  Exactly n_total particles; per-particle reference smoothing length
    h0 = 1.3 x the local spacing, mass = rho0 x spacing^3.  Strength + damage
    (Collins granite, multi-flaw with the surface spacing as flaw volume)."""
    rng = np.random.default_rng(seed)

    def count(dx0):
        n_imp = sphere(radius, dx0, (0.0, 0.0, 0.0)).shape[0]
        return n_imp + sum(nx * ny for _, _, nx, ny in _graded_layers(dx0, growth, L)), n_imp

    lo_dx, hi_dx = 1.0, 1000.0  # count decreases with dx0
    for _ in range(60):
        mid = math.sqrt(lo_dx * hi_dx)
        if count(mid)[0] >= n_total:
            lo_dx = mid
        else:
            hi_dx = mid
    dx0 = lo_dx
    layers = _graded_layers(dx0, growth, L)
    Lx, Ly, Lz = L
    slab, hsp = [], []
    for s, zc, nx, ny in layers:
        i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        xy = np.stack([(i.ravel() + 0.5) * s, (j.ravel() + 0.5) * s - 0.5 * ny * s], axis=1)
        p = np.concatenate([xy, np.full((xy.shape[0], 1), zc)], axis=1)
        slab.append(_jitter(p, s, jitter, rng))
        hsp.append(np.full(p.shape[0], s))
    slab = np.concatenate(slab)
    sp = np.concatenate(hsp)
    imp = sphere(radius, dx0, (0.0, 0.0, 0.0))
    n_imp = imp.shape[0]
    n_slab = n_total - n_imp
    # drop the surplus from the bottom of the far end (away from the track)
    order = np.lexsort((slab[:, 2], -slab[:, 0]))
    keep = np.ones(slab.shape[0], bool)
    keep[order[: slab.shape[0] - n_slab]] = False
    slab, sp = slab[keep], sp[keep]
    th = math.radians(angle_deg)
    imp = _jitter(imp + np.array([0.1 * Lx, 0.0, radius + dx0]), dx0, jitter, rng)
    pos = np.concatenate([slab, imp])
    spacing = np.r_[sp, np.full(n_imp, dx0)]
    vel = np.zeros_like(pos)
    vel[n_slab:, 0] = speed * math.cos(th)
    vel[n_slab:, 2] = -speed * math.sin(th)
    mat = np.r_[np.zeros(n_slab, np.int32), np.ones(n_imp, np.int32)]
    mats = [granite(strength=True), iron(strength=True)]
    mass = np.where(mat == 1, mats[1]["rho0"], mats[0]["rho0"]) * spacing ** 3
    lo = np.array([-0.05 * Lx - 2 * radius, -0.6 * Ly, -1.2 * Lz])
    hi = np.array([1.05 * Lx, 0.6 * Ly, 4 * radius + 0.2 * Lz])
    return Scenario(f"large_graded_{n_total}", pos, vel, mass, np.zeros(pos.shape[0]), mat,
                    np.zeros(pos.shape[0], np.uint8), lo, hi, np.zeros(3, np.int32),
                    dict(eta=1.3, h_init=1.3 * dx0, alpha=1.0, beta=2.0, eps=0.01, cfl=0.2,
                         eps_as=0.3, damage_on=1, flaw_model=1),
                    mats, dx0, flaws=("multi", 12345), h0=1.3 * spacing)


def batch_sizes(count=256, lo=5000, hi=80000, seed=20261203):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)


def batch_impacts(count=256, lo=5000, hi=80000, seed=20261203):
    """The batched sweep: `count` iron-into-granite impacts with strength and
    damage, particle counts log-uniform in [lo, hi], angle U[1, 45] deg, speed
    U[4, 12] km/s, impactor / target radius ratio U[0.1, 0.3], from one seed."""
    sizes = batch_sizes(count, lo, hi, seed)
    rng = np.random.default_rng(seed + 1)
    out = []
    for i, n in enumerate(sizes):
        out.append(sized_impact(int(n), seed=seed + 7 * i, angle_deg=float(rng.uniform(1.0, 45.0)),
                                speed=float(rng.uniform(4000.0, 12000.0)), ratio=float(rng.uniform(0.1, 0.3))))
    return out


def sized_impact(n_target, seed, angle_deg, speed, ratio, strength=True, flaws="multi", jitter=0.01):
    """One impact of roughly n_target particles: iron sphere of radius ratio x
    the slab half-depth into a granite slab (batched / served workloads)."""
    rng = np.random.default_rng(seed)
    # slab 4:2:1 in units of its depth T with lattice dx; sphere radius ratio * T
    frac_sphere = (4.0 / 3.0) * math.pi * ratio ** 3 / 8.0
    dx_cells = (n_target / (8.0 * (1.0 + frac_sphere))) ** (1.0 / 3.0)  # cells per depth
    nz = max(4, int(round(dx_cells)))
    dx = 1.0
    nx, ny = 4 * nz, 2 * nz
    slab = _jitter(lattice(nx, ny, nz, dx, (0.0, -0.5 * ny * dx, -nz * dx)), dx, jitter, rng)
    R = max(2.0, ratio * nz) * dx
    th = math.radians(angle_deg)
    imp = _jitter(sphere(R, dx, (0.2 * nx * dx, 0.0, R + dx)), dx, jitter, rng)
    pos = np.concatenate([slab, imp])
    vel = np.zeros_like(pos)
    vel[slab.shape[0]:, 0] = speed * math.cos(th)
    vel[slab.shape[0]:, 2] = -speed * math.sin(th)
    mat = np.r_[np.zeros(slab.shape[0], np.int32), np.ones(imp.shape[0], np.int32)]
    mats = [granite(strength), iron(strength)]
    mass = np.where(mat == 1, mats[1]["rho0"], mats[0]["rho0"]) * dx ** 3
    L = np.array([nx, ny, nz]) * dx
    lo = np.array([-0.2 * L[0], -L[1], -1.5 * L[2]])
    hi = np.array([1.2 * L[0], L[1], 1.5 * L[2] + 2 * R])
    prm = dict(eta=1.3, h_init=1.3 * dx, alpha=1.0, beta=2.0, eps=0.01, cfl=0.2,
               eps_as=0.3 if strength else 0.0, damage_on=1 if strength else 0,
               flaw_model=1 if (strength and flaws == "multi") else 0)
    return Scenario(f"impact_{n_target}", pos, vel, mass, np.zeros(pos.shape[0]), mat,
                    np.zeros(pos.shape[0], np.uint8), lo, hi, np.zeros(3, np.int32), prm, mats, dx,
                    flaws=(flaws, int(seed) & 0xffffffff) if strength else None)


# ------------------------------------------------------------ loaders
def _material_struct(cls, d):
    m = cls()
    for k in MAT_FIELDS:
        setattr(m, k, int(d[k]) if k in ("type", "yield_model") else float(d[k]))
    return m


def to_context(ctx, sc: Scenario, prm_overrides=None, material_ids=None):
    """Create one impact of `sc` in a deorbit_gb300.sph.Context; returns its id.
    Material ids of the scenario are offset by the materials already present.
    With a dict `material_ids`, equal materials are added once and shared by
    the impacts created through the same dict (a context holds a few dozen)."""
    from . import sph

    ids = []
    for d in sc.materials:
        key = tuple(sorted(d.items()))
        if material_ids is not None and key in material_ids:
            ids.append(material_ids[key])
            continue
        i = ctx.add_material(_material_struct(sph.Material, d))
        if material_ids is not None:
            material_ids[key] = i
        ids.append(i)
    ids = np.asarray(ids if ids else [0], np.int32)
    p = dict(sc.params)
    if prm_overrides:
        p.update(prm_overrides)
    b = ctx.impact_create(sph.params(**p), sc.lo, sc.hi, sc.periodic)
    ctx.add_particles(b, sc.pos, sc.vel, sc.mass, sc.u, ids[sc.mat], sc.fixed)
    if sc.flaws is not None:
        kind, seed = sc.flaws
        if kind == "multi":
            ctx.seed_flaws_multi(b, sc.dx, seed)
        else:
            ctx.seed_damage(b, sc.dx, seed)
    if sc.h0 is not None:
        ctx.set_h0(b, sc.h0)
    return b


def write_ic(sc: Scenario, path):
    """Reference IC file (run_ic.cpp:4-6): f8 [xlo xhi ylo yhi zlo zhi n] + n x 10 f8."""
    hdr = np.array([sc.lo[0], sc.hi[0], sc.lo[1], sc.hi[1], sc.lo[2], sc.hi[2], sc.n], np.float64)
    rec = np.concatenate([sc.pos, sc.vel, sc.mass[:, None], sc.u[:, None], sc.mat[:, None].astype(float),
                          sc.fixed[:, None].astype(float)], axis=1)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(rec, np.float64).tobytes())


def crop(sc: Scenario, n_keep: int, center=None) -> Scenario:
    """A bounded sample of a workload: all impactor particles plus the target
    particles nearest the impact point, n_keep in total (same dx, materials,
    parameters and domain)."""
    if n_keep >= sc.n:
        return sc
    imp = np.nonzero(sc.mat != 0)[0]
    tgt = np.nonzero(sc.mat == 0)[0]
    if center is None:
        center = sc.pos[imp].mean(0) if imp.size else sc.pos.mean(0)
    d = ((sc.pos[tgt] - center) ** 2).sum(1)
    keep_t = tgt[np.argsort(d, kind="stable")[: max(0, n_keep - imp.size)]]
    keep = np.sort(np.r_[keep_t, imp])[:n_keep]
    return dataclasses.replace(sc, name=sc.name + f"_crop{n_keep}", pos=sc.pos[keep], vel=sc.vel[keep],
                               mass=sc.mass[keep], u=sc.u[keep], mat=sc.mat[keep], fixed=sc.fixed[keep],
                               h0=None if sc.h0 is None else sc.h0[keep])
