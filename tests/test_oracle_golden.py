"""Pins the CPU oracle to the reference: every golden vector in tests/golden/
(made by the reference's own solver, see make_golden.py) is reproduced bit
for bit.  CPU only."""
import ctypes as C
import os

import numpy as np
import pytest

from deorbit_gb300 import ic

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def oracle_from(d, O):
    S = O.OracleSystem()
    for row in d["materials"]:
        S.add_material(ic._material_struct(O.Material, dict(zip(ic.MAT_FIELDS, row))))
    keys = ("eta", "h_init", "alpha", "beta", "eps", "alpha_u", "cfl", "eps_as", "damage_on")
    p = dict(zip(keys, d["params"]))
    p["damage_on"] = int(p["damage_on"])
    S.set_params(**p)
    S.set_domain(d["lo"], d["hi"], tuple(bool(x) for x in d["periodic"]))
    S.add_many(d["pos"], d["vel"], d["mass"], d["u"], d["mat"], d["fixed"])
    if int(d["flaw_seed"]) >= 0:
        S.seed_damage(float(d["dx"]), int(d["flaw_seed"]))
    return S


def test_eos_golden(oracle_lib):
    O = oracle_lib
    d = load("eos.npz")
    for nm in ("iron", "basalt", "water", "aluminum", "granite"):
        m = ic._material_struct(O.Material, dict(zip(ic.MAT_FIELDS, d[f"{nm}_mat"])))
        P, cs = O.eos(m, d[f"{nm}_rho"], d[f"{nm}_u"])
        assert np.array_equal(P, d[f"{nm}_P"]), nm
        assert np.array_equal(cs, d[f"{nm}_cs"]), nm
    P, cs = O.eos(O.ideal(1.4), d["ideal_rho"], d["ideal_u"])
    assert np.array_equal(P, d["ideal_P"]) and np.array_equal(cs, d["ideal_cs"])
    for which, fn in enumerate((O.iron, O.basalt, O.water, O.aluminum)):
        m = fn()
        assert np.array_equal(np.array([getattr(m, k) for k in ic.MAT_FIELDS]), d[f"std{which}"])


def test_kernel_and_eig_golden(oracle_lib):
    L = oracle_lib.lib()
    d = load("kernels.npz")
    W = np.array([L.orc_kW(r, h) for r, h in zip(d["r"], d["h"])])
    dW = np.array([L.orc_kdWdr(r, h) for r, h in zip(d["r"], d["h"])])
    assert np.array_equal(W, d["W"]) and np.array_equal(dW, d["dW"])
    s6 = np.ascontiguousarray(d["s6"])
    ev = np.array([L.orc_eig_max(s6[i].ctypes.data_as(C.POINTER(C.c_double))) for i in range(len(s6))])
    assert np.array_equal(ev, d["eig"])


def test_seed_damage_golden(oracle_lib):
    O = oracle_lib
    d = load("seed_damage.npz")
    S = O.OracleSystem()
    S.add_material(ic._material_struct(O.Material, ic.basalt()))
    S.add_material(ic._material_struct(O.Material, ic.iron()))
    S.set_params(h_init=39.0)
    n = d["mat"].size
    S.add_many(np.zeros((n, 3)), np.zeros((n, 3)), 1.0, 0.0, d["mat"])
    S.seed_damage(float(d["dx"]), int(d["seed"]))
    assert np.array_equal(S.field("eps_act"), d["eps_act"])


def test_sheared_cube_golden(oracle_lib):
    """cpu_dump's scenario: init, 12 steps, one consistent evaluation, one step."""
    O = oracle_lib
    d = load("sheared_cube_L10.npz")
    S = oracle_from(d, O)
    S.init()
    for k in O.FIELDS:
        assert np.array_equal(S.field(k), d["init_" + k]), k
    for dt in d["dts"][:12]:
        assert S.timestep() == dt
        S.step(dt)
    S.compute_density_h(2)
    S.compute_forces()
    for k in O.FIELDS:
        assert np.array_equal(S.field(k), d["eval_" + k]), k
    start, ids = S.cell_csr()
    assert np.array_equal(start, d["eval_cell_start"]) and np.array_equal(ids, d["eval_cell_ids"])
    for kind, nm in ((O.NBR_DENSITY, "dens"), (O.NBR_FORCE, "force")):
        c, j = S.neighbors(kind)
        assert np.array_equal(c, d[f"eval_{nm}_counts"]) and np.array_equal(j, d[f"eval_{nm}_ids"])
    assert S.timestep() == d["dts"][12]
    S.step(d["dts"][12])
    for k in O.FIELDS:
        assert np.array_equal(S.field(k), d["post_" + k]), k


@pytest.mark.parametrize("name,prefix,steps", [("impact_small.npz", "s15_", 15), ("periodic_bar.npz", "s10_", 10)])
def test_trajectory_golden(oracle_lib, name, prefix, steps):
    O = oracle_lib
    d = load(name)
    S = oracle_from(d, O)
    S.init()
    start, ids = S.cell_csr()
    assert np.array_equal(start, d["init_cell_start"]) and np.array_equal(ids, d["init_cell_ids"])
    for kind, nm in ((O.NBR_DENSITY, "dens"), (O.NBR_FORCE, "force")):
        c, j = S.neighbors(kind)
        assert np.array_equal(c, d[f"init_{nm}_counts"]) and np.array_equal(j, d[f"init_{nm}_ids"])
    for dt in d["dts"][:steps]:
        assert S.timestep() == dt
        S.step(dt)
    for k in O.FIELDS:
        assert np.array_equal(S.field(k), d[prefix + k]), k
