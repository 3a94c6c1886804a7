"""ctypes front end for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two back ends with one interface:
  * OracleSystem -- oracle/liborc.so, the C restatement of the reference's FP64
    solver (hydrocodes/sph/sph.hpp + hydrocodes/common/eos.hpp);
  * RefSystem    -- oracle/_ref/libsphref.so, the reference's own System compiled
    from its headers (only where the reference tree is present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libsphref.so")

IDEAL, TILLOTSON = 0, 1
YIELD_VON_MISES, YIELD_COLLINS = 0, 1
FLAWS_SINGLE, FLAWS_MULTI = 0, 1
NBR_DENSITY, NBR_FORCE = 0, 1

FIELDS = ("x y z vx vy vz ax ay az mass rho u dudt P cs csig hh eps_work D eps_act "
          "sigmax Pf Rart dscale Sxx Syy Szz Sxy Sxz Syz dSxx dSyy dSzz dSxy dSxz dSyz").split()


class Material(C.Structure):
    """Layout of orc_material (hydrocodes/common/eos.hpp:15-27 + Collins fields)."""

    _fields_ = [("type", C.c_int32), ("yield_model", C.c_int32), ("gamma", C.c_double)] + [
        (n, C.c_double)
        for n in "rho0 a b A B alpha beta u0 uiv ucv G Y Emod wm wk Y0 mu_i Ylim Yd0 mu_d".split()
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Params(C.Structure):
    """Layout of orc_params (hydrocodes/sph/sph.hpp:86-92 + extension switch)."""

    _fields_ = [(n, C.c_double) for n in "eta h_init alpha beta eps alpha_u cfl eps_as".split()] + [
        ("as_n", C.c_int32), ("damage_on", C.c_int32), ("flaw_model", C.c_int32), ("pad_", C.c_int32)]


def build(ref=False) -> None:
    """Compile liborc.so; ref=True also the reference shim (the reference tree
    must be present), ref="auto" the shim only where the tree is present."""
    targets = ["all"] + (["ref-auto"] if ref == "auto" else ["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def reference_dir() -> str:
    """Root of the reference checkout used by the fixture generators
    (DEORBIT_REFERENCE, default as in oracle/Makefile)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "refdir"], check=True, capture_output=True, text=True)
    return r.stdout.strip()


_lib = None
_ref = None
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


def _declare(lib, prefix):
    p = prefix
    sig = {
        f"{p}create": (C.c_void_p, []),
        f"{p}destroy": (None, [C.c_void_p]),
        f"{p}add_material": (C.c_int, [C.c_void_p, C.POINTER(Material)]),
        f"{p}set_params": (None, [C.c_void_p, C.POINTER(Params)]),
        f"{p}set_domain": (None, [C.c_void_p] + [C.c_double, C.c_double, C.c_int] * 3),
        f"{p}add_many": (None, [C.c_void_p, C.c_int] + [_D] * 8 + [_I32, _U8]),
        f"{p}n": (C.c_int, [C.c_void_p]),
        f"{p}seed_damage": (None, [C.c_void_p, C.c_double, C.c_uint32]),
        f"{p}init": (None, [C.c_void_p]),
        f"{p}timestep": (C.c_double, [C.c_void_p]),
        f"{p}step": (None, [C.c_void_p, C.c_double]),
        f"{p}compute_density_h": (None, [C.c_void_p, C.c_int]),
        f"{p}compute_forces": (None, [C.c_void_p]),
        f"{p}compute_strain_stress": (None, [C.c_void_p]),
        f"{p}grow_damage": (None, [C.c_void_p, C.c_double]),
        f"{p}yield_limit": (None, [C.c_void_p, C.c_int]),
        f"{p}build_cells": (None, [C.c_void_p]),
        f"{p}grid": (None, [C.c_void_p, _I32, _D, _D]),
        f"{p}ncells": (C.c_int64, [C.c_void_p]),
        f"{p}cell_csr": (None, [C.c_void_p, _I32, _I32]),
        f"{p}neighbors": (C.c_int64, [C.c_void_p, C.c_int, _I32, _I32, C.c_int64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        _lib = C.CDLL(ORACLE_SO)
        _declare(_lib, "orc_")
        L = _lib
        L.orc_field.restype = _D
        L.orc_field.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_mat_array.restype = _I32
        L.orc_mat_array.argtypes = [C.c_void_p]
        L.orc_fixed_array.restype = _U8
        L.orc_fixed_array.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_get_threads.argtypes = [C.c_void_p]
        L.orc_get_params.argtypes = [C.c_void_p, C.POINTER(Params)]
        L.orc_set_h0.argtypes = [C.c_void_p, _D]
        L.orc_seed_flaws_multi.restype = C.c_int64
        L.orc_seed_flaws_multi.argtypes = [C.c_void_p, C.c_double, C.c_uint32]
        L.orc_flaw_count.restype = C.c_int64
        L.orc_flaw_count.argtypes = [C.c_void_p]
        L.orc_flaw_arrays.argtypes = [C.c_void_p, _I64, _D]
        L.orc_set_flaws.argtypes = [C.c_void_p, _I64, _D]
        L.orc_cell_of.argtypes = [C.c_void_p, _I32]
        L.orc_eos_batch.argtypes = [C.POINTER(Material), C.c_int, _D, _D, _D, _D]
        for nm in ("orc_kW", "orc_kdWdr"):
            getattr(L, nm).restype = C.c_double
            getattr(L, nm).argtypes = [C.c_double, C.c_double]
        L.orc_eig_max.restype = C.c_double
        L.orc_eig_max.argtypes = [_D]
        for nm in ("iron", "basalt", "water", "aluminum"):
            getattr(L, f"orc_mat_{nm}").restype = Material
        L.orc_mat_tillotson.restype = Material
        L.orc_mat_tillotson.argtypes = [C.c_double] * 14
        L.orc_mat_ideal.restype = Material
        L.orc_mat_ideal.argtypes = [C.c_double]
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("reference shim not built (needs the reference tree): " + REF_SO)
        _ref = C.CDLL(REF_SO)
        _declare(_ref, "ref_")
        R = _ref
        R.ref_get_field.restype = C.c_int
        R.ref_get_field.argtypes = [C.c_void_p, C.c_char_p, _D]
        R.ref_set_field.restype = C.c_int
        R.ref_set_field.argtypes = [C.c_void_p, C.c_char_p, _D]
        R.ref_get_mat.argtypes = [C.c_void_p, _I32]
        R.ref_set_fixed.argtypes = [C.c_void_p, _U8]
        R.ref_eos_batch.argtypes = [C.POINTER(Material), C.c_int, _D, _D, _D, _D]
        R.ref_kernels.argtypes = [C.c_int, _D, _D, _D, _D]
        R.ref_eig_max.argtypes = [C.c_int, _D, _D]
        R.ref_std_material.argtypes = [C.c_int, C.POINTER(Material)]
    return _ref


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I32)


# ---------------------------------------------------------------- materials
def iron() -> Material:
    return lib().orc_mat_iron()


def basalt() -> Material:
    return lib().orc_mat_basalt()


def water() -> Material:
    return lib().orc_mat_water()


def aluminum() -> Material:
    return lib().orc_mat_aluminum()


def tillotson(rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, G=0.0, Y=0.0, wm=0.0, wk=0.0) -> Material:
    return lib().orc_mat_tillotson(rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, G, Y, wm, wk)


def ideal(gamma) -> Material:
    return lib().orc_mat_ideal(gamma)


def collins(m: Material, Y0, mu_i, Ylim, Yd0=0.0, mu_d=0.6) -> Material:
    """Return a copy of m with the (extension) Collins/Lundborg yield switched on."""
    c = Material.from_buffer_copy(m)
    c.yield_model = YIELD_COLLINS
    c.Y0, c.mu_i, c.Ylim, c.Yd0, c.mu_d = Y0, mu_i, Ylim, Yd0, mu_d
    return c


def eos(m: Material, rho, u):
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    P = np.empty_like(rho)
    cs = np.empty_like(rho)
    lib().orc_eos_batch(C.byref(m), rho.size, _dp(rho), _dp(u), _dp(P), _dp(cs))
    return P, cs


# ---------------------------------------------------------------- systems
class _Base:
    prefix = ""

    def _L(self):
        raise NotImplementedError

    def __init__(self):
        self.h = self._f("create")()
        self.materials = []

    def _f(self, name):
        return getattr(self._L(), self.prefix + name)

    def close(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        return self._f("n")(self.h)

    def add_material(self, m: Material) -> int:
        self.materials.append(m)
        return self._f("add_material")(self.h, C.byref(m))

    def set_params(self, **kw):
        p = Params()
        d = dict(eta=1.3, h_init=0.01, alpha=1.0, beta=2.0, eps=0.01, alpha_u=0.0, cfl=0.2,
                 eps_as=0.0, as_n=4, damage_on=0, flaw_model=FLAWS_SINGLE)
        d.update(getattr(self, "_params", {}))
        d.update(kw)
        self._params = d
        for k, v in d.items():
            setattr(p, k, v)
        self._f("set_params")(self.h, C.byref(p))

    def set_domain(self, lo, hi, periodic=(False, False, False)):
        self._f("set_domain")(self.h, lo[0], hi[0], int(periodic[0]), lo[1], hi[1], int(periodic[1]),
                              lo[2], hi[2], int(periodic[2]))

    def add_many(self, pos, vel, mass, u, mat, fixed=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        n = pos.shape[0]
        cols = [np.ascontiguousarray(pos[:, k]) for k in range(3)] + \
               [np.ascontiguousarray(vel[:, k]) for k in range(3)]
        mass = np.ascontiguousarray(np.broadcast_to(mass, (n,)), dtype=np.float64)
        u = np.ascontiguousarray(np.broadcast_to(u, (n,)), dtype=np.float64)
        mat = np.ascontiguousarray(np.broadcast_to(mat, (n,)), dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(np.broadcast_to(fixed, (n,)), dtype=np.uint8)
        self._f("add_many")(self.h, n, *[_dp(c) for c in cols], _dp(mass), _dp(u), _ip(mat),
                            None if fx is None else fx.ctypes.data_as(_U8))

    def seed_damage(self, dx, seed=12345):
        self._f("seed_damage")(self.h, dx, seed)

    def init(self):
        self._f("init")(self.h)

    def timestep(self) -> float:
        return self._f("timestep")(self.h)

    def step(self, dt):
        self._f("step")(self.h, dt)

    def compute_density_h(self, iters=2):
        self._f("compute_density_h")(self.h, iters)

    def compute_forces(self):
        self._f("compute_forces")(self.h)

    def compute_strain_stress(self):
        self._f("compute_strain_stress")(self.h)

    def grow_damage(self, dt):
        self._f("grow_damage")(self.h, dt)

    def yield_limit(self, i):
        self._f("yield_limit")(self.h, i)

    def build_cells(self):
        self._f("build_cells")(self.h)

    def grid(self):
        nc = np.zeros(3, np.int32)
        cw = np.zeros(3)
        hm = np.zeros(1)
        self._f("grid")(self.h, _ip(nc), _dp(cw), _dp(hm))
        return nc, cw, float(hm[0])

    def cell_csr(self):
        nc = int(self._f("ncells")(self.h))
        start = np.zeros(nc + 1, np.int32)
        ids = np.zeros(max(self.n, 1), np.int32)
        self._f("cell_csr")(self.h, _ip(start), _ip(ids))
        return start, ids[: self.n]

    def neighbors(self, kind):
        n = self.n
        counts = np.zeros(n, np.int32)
        cap = 64 * n + 16
        while True:
            ids = np.zeros(cap, np.int32)
            tot = self._f("neighbors")(self.h, kind, _ip(counts), _ip(ids), cap)
            if tot >= 0:
                return counts, ids[:tot]
            cap = -tot + 16

    def fields(self, names=FIELDS):
        return {k: self.field(k) for k in names}


class OracleSystem(_Base):
    """The C restatement (oracle/sph_oracle.c)."""

    prefix = "orc_"

    def _L(self):
        return lib()

    def set_threads(self, nt):
        lib().orc_set_threads(self.h, nt)

    def threads(self):
        return lib().orc_get_threads(self.h)

    def field(self, name):
        p = lib().orc_field(self.h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(self.n,)).copy()

    def set_field(self, name, values):
        p = lib().orc_field(self.h, name.encode())
        if not p:
            raise KeyError(name)
        np.ctypeslib.as_array(p, shape=(self.n,))[:] = values

    def mat(self):
        return np.ctypeslib.as_array(lib().orc_mat_array(self.h), shape=(self.n,)).copy()

    def set_fixed(self, fixed):
        np.ctypeslib.as_array(lib().orc_fixed_array(self.h), shape=(self.n,))[:] = fixed

    def set_h0(self, h0):
        h0 = np.ascontiguousarray(h0, dtype=np.float64)
        lib().orc_set_h0(self.h, _dp(h0))

    def seed_flaws_multi(self, dx, seed=12345):
        return lib().orc_seed_flaws_multi(self.h, dx, seed)

    def flaws(self):
        nf = lib().orc_flaw_count(self.h)
        start = np.zeros(self.n + 1, np.int64)
        eps = np.zeros(max(nf, 1))
        lib().orc_flaw_arrays(self.h, start.ctypes.data_as(_I64), _dp(eps))
        return start, eps[:nf]

    def set_flaws(self, start, eps):
        start = np.ascontiguousarray(start, dtype=np.int64)
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        lib().orc_set_flaws(self.h, start.ctypes.data_as(_I64), _dp(eps))

    def cell_of(self):
        c = np.zeros(self.n, np.int32)
        lib().orc_cell_of(self.h, _ip(c))
        return c


class RefSystem(_Base):
    """The reference's own System (oracle/_ref/libsphref.so)."""

    prefix = "ref_"

    def _L(self):
        return ref_lib()

    def field(self, name):
        out = np.zeros(self.n)
        if ref_lib().ref_get_field(self.h, name.encode(), _dp(out)) != 0:
            raise KeyError(name)
        return out

    def set_field(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if ref_lib().ref_set_field(self.h, name.encode(), _dp(v)) != 0:
            raise KeyError(name)

    def mat(self):
        out = np.zeros(self.n, np.int32)
        ref_lib().ref_get_mat(self.h, _ip(out))
        return out

    def set_fixed(self, fixed):
        f = np.ascontiguousarray(fixed, dtype=np.uint8)
        ref_lib().ref_set_fixed(self.h, f.ctypes.data_as(_U8))


def material_from_dict(d) -> Material:
    """orc_material from a material dict with the fields of Material."""
    m = Material()
    for name, _ in Material._fields_:
        setattr(m, name, int(d[name]) if name in ("type", "yield_model") else float(d[name]))
    return m


def from_scenario(sc, threads=0, cls=None):
    """The oracle system of a workload scenario (deorbit_gb300.ic.Scenario):
    same materials, parameters, domain, particles, flaws and per-particle h0 as
    the CUDA solver is given."""
    S = (cls or OracleSystem)()
    if threads:
        S.set_threads(threads)
    for d in sc.materials:
        S.add_material(material_from_dict(d))
    S.set_params(**dict(sc.params))
    S.set_domain(sc.lo, sc.hi, tuple(bool(x) for x in sc.periodic))
    S.add_many(sc.pos, sc.vel, sc.mass, sc.u, sc.mat, sc.fixed)
    if sc.flaws is not None:
        kind, seed = sc.flaws
        if kind == "multi":
            S.seed_flaws_multi(sc.dx, seed)
        else:
            S.seed_damage(sc.dx, seed)
    if sc.h0 is not None:
        S.set_h0(sc.h0)
    return S
