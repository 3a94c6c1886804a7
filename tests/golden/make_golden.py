"""Generate the golden vectors under tests/golden/ from the REFERENCE solver.

Runs the reference's own System (hydrocodes/sph/sph.hpp) and EOS
(hydrocodes/common/eos.hpp), compiled unmodified from the reference checkout
(DEORBIT_REFERENCE) by oracle/Makefile into oracle/_ref/libsphref.so, on seeded inputs and stores
inputs and outputs as compressed .npz.  Needs the reference tree; the fixtures
it writes are committed so that the tests never need it.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from deorbit_gb300 import ic  # noqa: E402
from oracle import oracle as O  # noqa: E402

ALL = O.FIELDS


def ref_system(sc):
    S = O.RefSystem()
    for d in sc.materials:
        S.add_material(ic._material_struct(O.Material, d))
    p = dict(sc.params)
    p.pop("flaw_model", None)
    S.set_params(**p)
    S.set_domain(sc.lo, sc.hi, tuple(bool(x) for x in sc.periodic))
    S.add_many(sc.pos, sc.vel, sc.mass, sc.u, sc.mat, sc.fixed)
    if sc.flaws is not None:
        S.seed_damage(sc.dx, sc.flaws[1])
    return S


def scenario_arrays(sc):
    return dict(pos=sc.pos, vel=sc.vel, mass=sc.mass, u=sc.u, mat=sc.mat, fixed=sc.fixed, lo=sc.lo, hi=sc.hi,
                periodic=sc.periodic, dx=np.float64(sc.dx),
                params=np.array([sc.params.get(k, d) for k, d in
                                 (("eta", 1.3), ("h_init", 0.01), ("alpha", 1.0), ("beta", 2.0), ("eps", 0.01),
                                  ("alpha_u", 0.0), ("cfl", 0.2), ("eps_as", 0.0), ("damage_on", 0))]),
                materials=np.array([[d[k] for k in ic.MAT_FIELDS] for d in sc.materials]),
                flaw_seed=np.int64(sc.flaws[1] if sc.flaws else -1))


def state(S, prefix):
    return {f"{prefix}{k}": S.field(k) for k in ALL}


def nbr(S, prefix):
    out = {}
    start, ids = S.cell_csr()
    nc, cw, hm = S.grid()
    out[f"{prefix}cell_start"] = start
    out[f"{prefix}cell_ids"] = ids
    out[f"{prefix}nc"] = nc
    out[f"{prefix}cw"] = cw
    for kind, nm in ((O.NBR_DENSITY, "dens"), (O.NBR_FORCE, "force")):
        c, j = S.neighbors(kind)
        out[f"{prefix}{nm}_counts"] = c
        out[f"{prefix}{nm}_ids"] = j
    return out


def save(name, d):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **d)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    O.build(ref=True)
    R = O.ref_lib()
    # -- EOS known answers over a (rho, u) sweep, eos.hpp:52-113
    mats = {"iron": ic.iron(), "basalt": ic.basalt(),
            "water": ic.tillotson(998, 2.2e9, 9.94e9, 0.7, 0.15, 10, 5, 7.0e6, 4.19e5, 2.69e6),
            "aluminum": ic.tillotson(2700, 7.52e10, 6.5e10, 0.5, 1.63, 5, 5, 5.0e6, 3.0e6, 1.39e7),
            "granite": ic.granite(False)}
    eos = {}
    for nm, d in mats.items():
        m = ic._material_struct(O.Material, d)
        rho = np.repeat(np.r_[0.0, np.linspace(0.3, 2.0, 35)] * d["rho0"], 40)
        u = np.tile(np.r_[0.0, np.geomspace(1e2, 5e7, 39)], 36)
        P = np.zeros_like(rho)
        cs = np.zeros_like(rho)
        R.ref_eos_batch(C.byref(m), rho.size, O._dp(rho), O._dp(u), O._dp(P), O._dp(cs))
        eos[f"{nm}_mat"] = np.array([d[k] for k in ic.MAT_FIELDS])
        eos[f"{nm}_rho"], eos[f"{nm}_u"], eos[f"{nm}_P"], eos[f"{nm}_cs"] = rho, u, P, cs
    gas = O.ideal(1.4)
    rho = np.linspace(0.1, 2.0, 50)
    u = np.linspace(0.0, 3.0, 50)
    P = np.zeros(50)
    cs = np.zeros(50)
    R.ref_eos_batch(C.byref(gas), 50, O._dp(rho), O._dp(u), O._dp(P), O._dp(cs))
    eos.update(ideal_rho=rho, ideal_u=u, ideal_P=P, ideal_cs=cs)
    for which in range(4):
        m = O.Material()
        R.ref_std_material(which, C.byref(m))
        eos[f"std{which}"] = np.array([getattr(m, k) for k in ic.MAT_FIELDS])
    save("eos.npz", eos)

    # -- kernel, derivative and largest eigenvalue, sph.hpp:17-54
    rng = np.random.default_rng(1)
    h = rng.uniform(0.5, 40.0, 4000)
    r = h * rng.uniform(0.0, 2.2, 4000)
    W = np.zeros(4000)
    dW = np.zeros(4000)
    R.ref_kernels(4000, O._dp(r), O._dp(h), O._dp(W), O._dp(dW))
    s6 = rng.normal(0.0, 1e8, (3000, 6))
    s6[:500, 3:] = 0.0  # diagonal branch
    ev = np.zeros(3000)
    R.ref_eig_max(3000, O._dp(np.ascontiguousarray(s6)), O._dp(ev))
    save("kernels.npz", dict(r=r, h=h, W=W, dW=dW, s6=s6, eig=ev))

    # -- the oracle-dump scenario (cpu_dump.cpp:12-64) at L = 10
    sc = ic.sheared_cube(L=10)
    S = ref_system(sc)
    S.init()
    d = scenario_arrays(sc)
    d.update(state(S, "init_"))
    dts = []
    for _ in range(12):
        dts.append(S.timestep())
        S.step(dts[-1])
    S.compute_density_h(2)
    S.compute_forces()
    d.update(state(S, "eval_"))
    d.update(nbr(S, "eval_"))
    dt = S.timestep()
    S.step(dt)
    d.update(state(S, "post_"))
    d["dts"] = np.array(dts + [dt])
    save("sheared_cube_L10.npz", d)

    # -- a small hydro-only impact, 15 steps at CFL 0.3
    sc = ic.impact_halfspace(nx=16, ny=16, nz=8, r_cells=3.0)
    S = ref_system(sc)
    S.init()
    d = scenario_arrays(sc)
    d.update(nbr(S, "init_"))
    dts = []
    for _ in range(15):
        dts.append(S.timestep())
        S.step(dts[-1])
    d.update(state(S, "s15_"))
    d["dts"] = np.array(dts)
    save("impact_small.npz", d)

    # -- periodic bar with frozen ends (periodic y, z; strength on)
    sc = ic.periodic_bar()
    S = ref_system(sc)
    S.init()
    d = scenario_arrays(sc)
    d.update(nbr(S, "init_"))
    dts = []
    for _ in range(10):
        dts.append(S.timestep())
        S.step(dts[-1])
    d.update(state(S, "s10_"))
    d["dts"] = np.array(dts)
    save("periodic_bar.npz", d)

    # -- single-flaw seeding (sph.hpp:117-128)
    mat = (np.arange(5000) % 3 == 1).astype(np.int32)
    S = O.RefSystem()
    S.add_material(ic._material_struct(O.Material, ic.basalt()))
    S.add_material(ic._material_struct(O.Material, ic.iron()))
    S.set_params(h_init=39.0)
    S.add_many(np.zeros((5000, 3)), np.zeros((5000, 3)), 1.0, 0.0, mat)
    S.seed_damage(30.0, 12345)
    save("seed_damage.npz", dict(mat=mat, dx=np.float64(30.0), seed=np.int64(12345), eps_act=S.field("eps_act")))


if __name__ == "__main__":
    main()
