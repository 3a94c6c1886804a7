"""Generate tests/golden/euler_gates.npz from the REFERENCE Euler solver.

Runs the reference's own CPU Euler solver (hydrocodes/euler/hydro_cpu.cpp),
compiled unmodified from the reference checkout (DEORBIT_REFERENCE) by
oracle/Makefile into oracle/_ref/libeulerref.so, on the gate workloads of
deorbit_gb300.grid_ic (small sizes, a bounded number of steps of the drivers'
loop) and on single-operator cases (Lop with every source term, the ROCK
yield with damage and fluidization forms, damage growth, fluidization
activation, the implicit viscosity).  The conjugate-gradient iteration
counts of the implicit viscosity are recorded too.  Inputs, settings and outputs are stored as one compressed .npz;
the tests reproduce them with the C oracle bit for bit, without the
reference tree.

    python tests/golden/make_euler_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from deorbit_gb300 import grid_ic as GI  # noqa: E402
from oracle import euler as EO  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "euler_gates.npz")

# (case, steps of the drivers' loop)
RUNS = [(GI.sod(), 60), (GI.tracer(), 40), (GI.sedov(12), 8), (GI.sedov_axi(16, 32), 10),
        (GI.shear(200), 30), (GI.yield_pulse(100), 40), (GI.vacuum(200), 40), (GI.bshock(100), 20),
        (GI.freefall(), 20), (GI.atmos(50), 10), (GI.tensile(), 20), (GI.alimpact(100), 30),
        (GI.surface(), 20), (GI.impact3d(12), 6), (GI.impact3d(12, af=True), 6),
        (GI.substrate(), 30), (GI.crater(), 20), (GI.crater(tdec=2.0, eta_af=1e8), 20),
        (GI.crater(cppr=3, U=6000.0), 15), (GI.crater(cppr=3, U=6000.0, void_cons=1), 25),
        (GI.crater(cppr=3, U=6000.0, void_amb=0.27), 25),
        (GI.visc_slab(), 20), (GI.visc_slab(eta=5e11, A0=2.0, t_end=5.0), 12), (GI.vib_slab(2), 20),
        (GI.bingham_heap(1, NX=60, NZ=16), 10), (GI.crater(cppr=3, U=6000.0, tdec=2.0, eta_af=1e9, visc_imp=1), 15)]


def perturbed_state(seed, shape, strength=True):
    """A smooth, seeded, non-trivial state for single-operator cases."""
    rng = np.random.default_rng(seed)
    n = shape[0] * shape[1] * shape[2]
    r = 2700.0 * (1.0 + 0.05 * rng.standard_normal(n))
    r[rng.random(n) < 0.05] = 50.0  # a few near-void cells
    f = {"r": r, "mu": r * 300.0 * rng.standard_normal(n), "mv": r * 300.0 * rng.standard_normal(n),
         "mw": r * 300.0 * rng.standard_normal(n)}
    ke = 0.5 * (f["mu"] ** 2 + f["mv"] ** 2 + f["mw"] ** 2) / r
    f["E"] = ke + r * np.abs(2e6 * rng.standard_normal(n))
    if strength:
        for k in ("Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"):
            f[k] = 2e8 * rng.standard_normal(n)
        f["D"] = np.clip(rng.random(n) * 1.2 - 0.1, 0.0, 1.0)
        f["af"] = np.clip(rng.random(n) - 0.5, 0.0, 1.0)
        f["vib"] = np.abs(5.0 * rng.standard_normal(n))
        f["Pmax"] = np.abs(1e8 * rng.standard_normal(n))
    f["rc"] = r * (rng.random(n) < 0.3)
    return f


# single-operator cases: (name, shape, dx, settings, op, arg)
OPS = [
    ("lop_cart", (6, 5, 7), 50.0, {"rock": 1, "gz": 3.71, "rho_cfl": 100.0, "eta_af": 1e7}, "lop", None),
    ("lop_axi", (9, 1, 8), 50.0, {"axisym": 1, "gz": 3.71, "eta_af": 1e7}, "lop", None),
    ("lop_vac", (7, 4, 6), 50.0, {"rho_vac": 100.0}, "lop", None),
    ("vm_rock", (5, 4, 6), 50.0, {"rock": 1, "y_d0": 5e6, "y_bingham": 2e7}, "vonmises", 1),
    ("vm_prel", (5, 4, 6), 50.0, {"rock": 1, "af_prel": 1, "af_reg": 1, "c_reg": 0.2}, "vonmises", 1),
    ("vm_plain", (5, 4, 6), 50.0, {}, "vonmises", 1),
    ("damage", (5, 4, 6), 50.0, {}, "grow_damage", 1e-3),
    ("af", (5, 4, 6), 50.0, {"tdec": 2.0, "c_act": 0.1, "p_act": 1e6}, "update_af", 1e-2),
    ("af_reg", (5, 4, 6), 50.0, {"tdec": 2.0, "c_act": 0.1, "af_reg": 1, "af_seeddp": 1, "rho_cfl": 100.0},
     "update_af", 1e-2),
    ("visc_cart", (6, 5, 7), 50.0, {"visc_imp": 1, "eta_af": 1e9, "rho_cfl": 100.0}, "implicit_visc", 0.05),
    ("visc_cyl", (9, 1, 8), 50.0, {"visc_imp": 1, "eta_af": 1e9, "axisym": 1, "af_reg": 1}, "implicit_visc", 0.05),
]


def main():
    if not EO.ref_available():
        O.build(ref=True)
    out = {}
    for case, steps in RUNS:
        g = EO.from_case(case, EO.RefGrid)
        s, t = EO.run_case(g, case, steps)
        key = case.name + ("_af" if case.params.get("c_act") else "")
        for k, v in case.fields.items():
            out[f"{key}/in/{k}"] = np.asarray(v, dtype=np.float64)
        for k, v in case.post_ref.items():
            out[f"{key}/post/{k}"] = np.asarray(v, dtype=np.float64)
        for k, v in g.fields().items():
            out[f"{key}/out/{k}"] = v
        out[f"{key}/meta"] = np.array(json.dumps({
            "kind": "run", "shape": list(case.shape), "dx": case.dx, "material": case.material,
            "params": case.params, "cfl": case.cfl, "t_end": case.t_end, "max_steps": steps,
            "steps": s, "t": t, "set_ref": case.set_ref, "pin_floor": case.pin_floor,
            "sponge_from": case.sponge_from,
            "visc_iters": g.visc_iters()}))
        g.close()
        print(key, s, t)
    for i, (name, shape, dx, prm, op, arg) in enumerate(OPS):
        f = perturbed_state(100 + i, shape)
        g = EO.RefGrid(*shape, dx, material=O.material_from_dict(GI.ic.basalt()), params=prm)
        for k, v in f.items():
            g.set_field(k, v)
        if op == "lop":
            g.lop()
            res = {f"rhs_{k}": g.rhs(k) for k in EO.RHS}
        else:
            getattr(g, op)(arg)
            res = g.fields()
        res["maxspeed"] = np.array([g.maxspeed()])
        for k, v in f.items():
            out[f"{name}/in/{k}"] = v
        for k, v in res.items():
            out[f"{name}/out/{k}"] = v
        out[f"{name}/meta"] = np.array(json.dumps({
            "kind": "op", "op": op, "arg": arg, "shape": list(shape), "dx": dx, "material": GI.ic.basalt(),
            "params": prm, "visc_iters": g.visc_iters()}))
        g.close()
        print(name, op)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
