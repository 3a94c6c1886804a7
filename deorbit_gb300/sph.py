"""Python front end of libdeorbit_sph.so (ctypes over include/deorbit_sph.h).

`System` mirrors the reference's in-process solver (hydrocodes/sph/sph.hpp:72-380):
same parameter names, `add` / `set_domain` / `seed_damage` / `init` /
`timestep` / `step`, and field access in the original particle order.  It is a
single impact of a `Context`; `Context` exposes the batched API (many impacts
per GPU).  There is no CPU fallback: without the CUDA library or a GPU every
call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libdeorbit_sph.so")

FP64, MIXED = 0, 1
EOS_IDEAL, EOS_TILLOTSON = 0, 1
YIELD_VON_MISES, YIELD_COLLINS = 0, 1
FLAWS_SINGLE, FLAWS_MULTI = 0, 1
NBR_DENSITY, NBR_FORCE = 0, 1

FIELDS = ("x y z vx vy vz ax ay az mass rho u dudt P cs csig hh eps_work D eps_act "
          "sigmax Pf Rart dscale Sxx Syy Szz Sxy Sxz Syz dSxx dSyy dSzz dSxy dSxz dSyz").split()


class SphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Material(C.Structure):
    """sph_material: Tillotson / ideal EOS + strength (eos.hpp:15-27) + Collins fields."""

    _fields_ = [("type", C.c_int32), ("yield_model", C.c_int32), ("gamma", C.c_double)] + [
        (n, C.c_double)
        for n in "rho0 a b A B alpha beta u0 uiv ucv G Y Emod wm wk Y0 mu_i Ylim Yd0 mu_d".split()]


class Params(C.Structure):
    """sph_params: System's parameter members (sph.hpp:86-92)."""

    _fields_ = [(n, C.c_double) for n in "eta h_init alpha beta eps alpha_u cfl eps_as".split()] + [
        ("as_n", C.c_int32), ("damage_on", C.c_int32), ("flaw_model", C.c_int32), ("reserved", C.c_int32)]


class ImpactInfo(C.Structure):
    _fields_ = [("n", C.c_int64), ("steps", C.c_int64), ("t", C.c_double), ("dt", C.c_double),
                ("h_max", C.c_double), ("nc", C.c_int32 * 3), ("cw", C.c_double * 3),
                ("density_rounds", C.c_int32), ("initialized", C.c_int32)]


class Conservation(C.Structure):
    _fields_ = [("mass", C.c_double), ("kinetic", C.c_double), ("internal", C.c_double),
                ("energy", C.c_double), ("momentum", C.c_double * 3)]


class GrazingSpec(C.Structure):
    _fields_ = [("theta_deg", C.c_double), ("v", C.c_double), ("D", C.c_double), ("rho_imp", C.c_double),
                ("rho_target", C.c_double), ("x_impact_frac", C.c_double), ("start_h", C.c_double),
                ("cppr", C.c_int32), ("tgt_mat", C.c_int32), ("imp_mat", C.c_int32), ("reserved", C.c_int32)]


class Diagnostics(C.Structure):
    _fields_ = [("count", C.c_int64), ("melted", C.c_int64), ("mean_pos", C.c_double * 3),
                ("mean_vel", C.c_double * 3), ("mean_speed", C.c_double), ("dispersion", C.c_double),
                ("u_max", C.c_double)]


class Request(C.Structure):
    """sph_request: one impact run submitted to a server."""
    _fields_ = [("params", C.POINTER(Params)), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("periodic", C.c_int32 * 3), ("flaws", C.c_int32), ("n", C.c_int64)] + [
        (k, C.POINTER(C.c_double)) for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "u")] + [
        ("mat", C.POINTER(C.c_int32)), ("fixed", C.POINTER(C.c_uint8)), ("h0", C.POINTER(C.c_double)),
        ("flaw_dx", C.c_double), ("flaw_seed", C.c_uint32), ("reserved", C.c_int32), ("steps", C.c_int64),
        ("arrival", C.c_double)]


class ServeRecord(C.Structure):
    _fields_ = [("n", C.c_int64), ("steps", C.c_int64), ("state", C.c_int32), ("impact", C.c_int32),
                ("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double)]


class ServeSummary(C.Structure):
    _fields_ = [("done", C.c_int64), ("queued", C.c_int64), ("resident", C.c_int64)] + [
        (k, C.c_double) for k in ("p50_latency_s", "p99_latency_s", "mean_latency_s", "particle_steps",
                                  "throughput", "busy_throughput", "busy_s", "peak_device_bytes",
                                  "admit_wait_s", "host_s")]


SERVE_FLAWS = {None: 0, "single": 1, "multi": 2}
SERVE_QUEUED, SERVE_RESIDENT, SERVE_DONE, SERVE_FAILED = 0, 1, 2, 3

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)
_P = C.c_void_p

_SIGS = {
    "sph_abi_version": (C.c_int, []),
    "sph_last_error": (C.c_char_p, []),
    "sph_material_tillotson": (None, [C.POINTER(Material)] + [C.c_double] * 14),
    "sph_material_ideal": (None, [C.POINTER(Material), C.c_double]),
    "sph_material_standard": (C.c_int, [C.c_int, C.POINTER(Material)]),
    "sph_params_default": (None, [C.POINTER(Params)]),
    "sph_seed_flaws_single": (C.c_int, [C.c_int64, _I32, C.POINTER(Material), C.c_int, C.c_double, C.c_uint32, _D]),
    "sph_seed_flaws_multi_host": (C.c_int, [C.c_int64, _I32, C.POINTER(Material), C.c_int, C.c_double,
                                            C.c_uint32, _I64, _D, C.c_int64, _I64, _D]),
    "sph_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int]),
    "sph_destroy": (C.c_int, [_P]),
    "sph_add_material": (C.c_int, [_P, C.POINTER(Material), _I32]),
    "sph_impact_create": (C.c_int, [_P, C.POINTER(Params), _D, _D, _I32, _I32]),
    "sph_impact_set_domain": (C.c_int, [_P, C.c_int32, _D, _D, _I32]),
    "sph_impact_set_params": (C.c_int, [_P, C.c_int32, C.POINTER(Params)]),
    "sph_impact_get_params": (C.c_int, [_P, C.c_int32, C.POINTER(Params)]),
    "sph_impact_add_particles": (C.c_int, [_P, C.c_int32, C.c_int64] + [_D] * 8 + [_I32, _U8]),
    "sph_impact_seed_damage": (C.c_int, [_P, C.c_int32, C.c_double, C.c_uint32]),
    "sph_impact_seed_flaws_multi": (C.c_int, [_P, C.c_int32, C.c_double, C.c_uint32, _I64]),
    "sph_impact_set_h0": (C.c_int, [_P, C.c_int32, _D]),
    "sph_impact_remove": (C.c_int, [_P, C.c_int32]),
    "sph_impact_set_step_limit": (C.c_int, [_P, C.c_int32, C.c_int64]),
    "sph_impact_count": (C.c_int, [_P, _I32]),
    "sph_impact_info_get": (C.c_int, [_P, C.c_int32, C.POINTER(ImpactInfo)]),
    "sph_init": (C.c_int, [_P]),
    "sph_timestep": (C.c_int, [_P, C.c_int32, _D]),
    "sph_step": (C.c_int, [_P, C.c_double]),
    "sph_run": (C.c_int, [_P, C.c_int32, C.c_double]),
    "sph_compute_density_h": (C.c_int, [_P, C.c_int32]),
    "sph_compute_forces": (C.c_int, [_P]),
    "sph_synchronize": (C.c_int, [_P]),
    "sph_read_field": (C.c_int, [_P, C.c_int32, C.c_char_p, _D]),
    "sph_write_field": (C.c_int, [_P, C.c_int32, C.c_char_p, _D]),
    "sph_read_fields": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D)]),
    "sph_write_fields": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D)]),
    "sph_step_fields": (C.c_int, [_P, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D),
                                  C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D), _D]),
    "sph_read_mat": (C.c_int, [_P, C.c_int32, _I32]),
    "sph_read_fixed": (C.c_int, [_P, C.c_int32, _U8]),
    "sph_write_fixed": (C.c_int, [_P, C.c_int32, _U8]),
    "sph_conservation_get": (C.c_int, [_P, C.c_int32, C.POINTER(Conservation)]),
    "sph_grazing_spec_default": (None, [C.c_void_p]),
    "sph_impact_create_grazing": (C.c_int, [_P, C.POINTER(Params), C.c_void_p, _I32, _D, _I64]),
    "sph_impact_diagnostics": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                         C.POINTER(Diagnostics)]),
    "sph_eos_eval": (C.c_int, [_P, C.c_int32, C.c_int64, _D, _D, _D, _D]),
    "sph_debug_ref_cells": (C.c_int, [_P, C.c_int32, _I32, _D, _I32, C.c_int64, _I32]),
    "sph_debug_neighbors": (C.c_int, [_P, C.c_int32, C.c_int32, _I32, _I32, C.c_int64, _I64]),
    "sph_debug_flaws": (C.c_int, [_P, C.c_int32, _I64, _D, C.c_int64, _I64]),
    "sph_load_ic": (C.c_int, [_P, C.c_char_p, C.POINTER(Params), _I32]),
    "sph_write_snapshot": (C.c_int, [_P, C.c_int32, C.c_char_p]),
    "sph_write_checkpoint": (C.c_int, [_P, C.c_int32, C.c_char_p, C.c_double]),
    "sph_load_checkpoint": (C.c_int, [_P, C.c_char_p, C.POINTER(Params), _I32, _D]),
    "sph_set_tuning": (C.c_int, [_P, C.c_int32, C.c_double]),
    "sph_launch_count": (C.c_int, [_P, _I64]),
    "sph_set_option": (C.c_int, [_P, C.c_char_p, C.c_double]),
    "sph_cell_sort": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sph_cell_sort_static": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sph_get_option": (C.c_int, [_P, C.c_char_p, _D]),
    "sph_phase_times": (C.c_int, [_P, _D]),
    "sph_set_profiling": (C.c_int, [_P, C.c_int32]),
    "sph_kernel_stats": (C.c_int, [_P, C.c_int32, _D, _I64]),
    "sph_kernel_stats_reset": (C.c_int, [_P]),
    "sph_event_record": (C.c_int, [_P, C.c_int32]),
    "sph_event_elapsed": (C.c_int, [_P, C.c_int32, C.c_int32, _D]),
    "sph_serve_create": (C.c_int, [_P, C.c_double, C.c_int32, C.c_char_p, C.POINTER(_P)]),
    "sph_serve_destroy": (C.c_int, [_P]),
    "sph_serve_now": (C.c_int, [_P, _D]),
    "sph_serve_submit": (C.c_int, [_P, C.POINTER(Request), _I64]),
    "sph_serve_poll": (C.c_int, [_P, C.c_double, _I64, C.c_int32, _I32]),
    "sph_serve_request_info": (C.c_int, [_P, C.c_int64, C.POINTER(ServeRecord)]),
    "sph_serve_result": (C.c_int, [_P, C.c_int64, C.c_char_p, _D]),
    "sph_serve_release": (C.c_int, [_P, C.c_int64]),
    "sph_serve_stats": (C.c_int, [_P, C.POINTER(ServeSummary)]),
}

KERNEL_CLASSES = ["kick", "sort", "grid", "list_density", "density", "eos", "list_force", "force",
                  "damage", "finish", "dt", "other"]

_lib = None


def lib():
    """Load the CUDA library; raise if it is missing (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() or "
                              "python deorbit_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        raise SphError(rc, lib().sph_last_error().decode(errors="replace"))


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I32)


def _out64(a, n):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous and a.size == n):
        raise ValueError(f"output buffer must be a contiguous float64 array of {n}")
    return a


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None:
        a = np.ascontiguousarray(np.broadcast_to(a, (n,)))
    return a


# ------------------------------------------------------------------ materials
def tillotson(rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, G=0.0, Y=0.0, wm=0.0, wk=0.0) -> Material:
    """Material::tillotson (eos.hpp:30-39)."""
    m = Material()
    lib().sph_material_tillotson(C.byref(m), rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, G, Y, wm, wk)
    return m


def ideal(gamma) -> Material:
    m = Material()
    lib().sph_material_ideal(C.byref(m), gamma)
    return m


def standard(which: int) -> Material:
    m = Material()
    check(lib().sph_material_standard(which, C.byref(m)))
    return m


def iron() -> Material:
    return standard(0)


def basalt() -> Material:
    return standard(1)


def water() -> Material:
    return standard(2)


def aluminum() -> Material:
    return standard(3)


def collins(m: Material, Y0, mu_i, Ylim, Yd0=0.0, mu_d=0.6) -> Material:
    """Copy of m with the Collins / Lundborg pressure-dependent yield switched on."""
    c = Material.from_buffer_copy(m)
    c.yield_model = YIELD_COLLINS
    c.Y0, c.mu_i, c.Ylim, c.Yd0, c.mu_d = Y0, mu_i, Ylim, Yd0, mu_d
    return c


def params(**kw) -> Params:
    p = Params()
    lib().sph_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def seed_flaws_single(mat, materials, dx, seed=12345):
    """Host-side System::seed_damage (sph.hpp:117-128) over material ids."""
    mat = np.ascontiguousarray(mat, dtype=np.int32)
    arr = (Material * max(len(materials), 1))(*materials)
    out = np.zeros(mat.size)
    check(lib().sph_seed_flaws_single(mat.size, _ip(mat), arr, len(materials), dx, seed, _dp(out)))
    return out


def seed_flaws_multi(mat, materials, dx, seed=12345):
    """Host-side Benz-Asphaug multi-flaw seeding -> (ptr, eps, eps_act)."""
    mat = np.ascontiguousarray(mat, dtype=np.int32)
    arr = (Material * max(len(materials), 1))(*materials)
    n = mat.size
    ptr = np.zeros(n + 1, np.int64)
    eps_act = np.zeros(n)
    total = np.zeros(1, np.int64)
    cap = int(n * (np.log(max(n, 2)) + 2) + 16)
    eps = np.zeros(cap)
    check(lib().sph_seed_flaws_multi_host(n, _ip(mat), arr, len(materials), dx, seed,
                                          ptr.ctypes.data_as(_I64), _dp(eps), cap,
                                          total.ctypes.data_as(_I64), _dp(eps_act)))
    return ptr, eps[: int(total[0])], eps_act


# ------------------------------------------------------------------ context
class Context:
    """One engine on one GPU holding any number of impacts."""

    def __init__(self, precision=FP64, device=0):
        self.h = _P()
        check(lib().sph_create(C.byref(self.h), precision, device))
        self.precision = precision

    def close(self):
        if getattr(self, "h", None):
            lib().sph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_material(self, m: Material) -> int:
        i = C.c_int32()
        check(lib().sph_add_material(self.h, C.byref(m), C.byref(i)))
        return i.value

    def impact_create(self, prm: Params, lo=(0, 0, 0), hi=(0, 0, 0), periodic=(0, 0, 0)) -> int:
        lo = _f64(lo)
        hi = _f64(hi)
        per = np.ascontiguousarray(periodic, dtype=np.int32)
        b = C.c_int32()
        check(lib().sph_impact_create(self.h, C.byref(prm), _dp(lo), _dp(hi), _ip(per), C.byref(b)))
        return b.value

    def add_particles(self, b, pos, vel, mass, u, mat=None, fixed=None):
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        cols = [np.ascontiguousarray(pos[:, k]) for k in range(3)] + [np.ascontiguousarray(vel[:, k]) for k in range(3)]
        mass = _f64(mass, n)
        u = _f64(u, n)
        mt = None if mat is None else np.ascontiguousarray(np.broadcast_to(mat, (n,)), dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(np.broadcast_to(fixed, (n,)), dtype=np.uint8)
        check(lib().sph_impact_add_particles(self.h, b, n, *[_dp(c) for c in cols], _dp(mass), _dp(u),
                                             None if mt is None else _ip(mt),
                                             None if fx is None else fx.ctypes.data_as(_U8)))

    def seed_damage(self, b, dx, seed=12345):
        check(lib().sph_impact_seed_damage(self.h, b, dx, seed))

    def seed_flaws_multi(self, b, dx, seed=12345):
        nf = C.c_int64()
        check(lib().sph_impact_seed_flaws_multi(self.h, b, dx, seed, C.byref(nf)))
        return nf.value

    def set_h0(self, b, h0):
        h0 = _f64(h0)
        check(lib().sph_impact_set_h0(self.h, b, _dp(h0)))

    def set_params(self, b, prm: Params):
        check(lib().sph_impact_set_params(self.h, b, C.byref(prm)))

    def get_params(self, b) -> Params:
        p = Params()
        check(lib().sph_impact_get_params(self.h, b, C.byref(p)))
        return p

    def set_step_limit(self, b, steps):
        check(lib().sph_impact_set_step_limit(self.h, b, int(steps)))

    def remove(self, b):
        check(lib().sph_impact_remove(self.h, b))

    def info(self, b) -> ImpactInfo:
        inf = ImpactInfo()
        check(lib().sph_impact_info_get(self.h, b, C.byref(inf)))
        return inf

    def n(self, b) -> int:
        return int(self.info(b).n)

    def init(self):
        check(lib().sph_init(self.h))

    def timestep(self, b=0) -> float:
        d = C.c_double()
        check(lib().sph_timestep(self.h, b, C.byref(d)))
        return d.value

    def step(self, dt):
        check(lib().sph_step(self.h, dt))

    def run(self, nsteps, t_end=0.0):
        check(lib().sph_run(self.h, nsteps, t_end))

    def compute_density_h(self, iters=2):
        check(lib().sph_compute_density_h(self.h, iters))

    def compute_forces(self):
        check(lib().sph_compute_forces(self.h))

    def synchronize(self):
        check(lib().sph_synchronize(self.h))

    def read(self, b, name, out=None) -> np.ndarray:
        """One field in original particle order (into `out`, a contiguous
        float64 array of n, when given: page-locked buffers copy fastest)."""
        out = np.zeros(self.n(b)) if out is None else _out64(out, self.n(b))
        check(lib().sph_read_field(self.h, b, name.encode(), _dp(out)))
        return out

    def write(self, b, name, values):
        v = _f64(values, self.n(b))
        check(lib().sph_write_field(self.h, b, name.encode(), _dp(v)))

    def read_many(self, b, names, outs=None):
        """Several fields with one synchronisation: {name: array}."""
        n = self.n(b)
        outs = [np.zeros(n) for _ in names] if outs is None else [_out64(o, n) for o in outs]
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        ptrs = (_D * len(names))(*[_dp(o) for o in outs])
        check(lib().sph_read_fields(self.h, b, len(names), cn, ptrs))
        return dict(zip(names, outs))

    def write_many(self, b, fields):
        """Several fields ({name: values}) with one synchronisation."""
        n = self.n(b)
        names = list(fields)
        vals = [_f64(fields[k], n) for k in names]
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        ptrs = (_D * len(names))(*[_dp(v) for v in vals])
        check(lib().sph_write_fields(self.h, b, len(names), cn, ptrs))

    def step_fields(self, b, fields, out_names, outs=None, dt=-1.0):
        """write_many(b, fields); dt = timestep(b) when dt < 0; step(dt);
        read_many(b, out_names) -- one call whose host copies overlap the
        step (page-locked buffers copy fastest).  Returns (dt, {name: array})."""
        n = self.n(b)
        names = list(fields)
        vals = [_f64(fields[k], n) for k in names]
        outs = [np.zeros(n) for _ in out_names] if outs is None else [_out64(o, n) for o in outs]
        cin = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        pin = (_D * max(1, len(names)))(*[_dp(v) for v in vals])
        cout = (C.c_char_p * max(1, len(out_names)))(*[k.encode() for k in out_names])
        pout = (_D * max(1, len(out_names)))(*[_dp(o) for o in outs])
        used = C.c_double()
        check(lib().sph_step_fields(self.h, b, float(dt), len(names), cin, pin, len(out_names), cout, pout,
                                    C.byref(used)))
        return used.value, dict(zip(out_names, outs))

    def mat(self, b) -> np.ndarray:
        out = np.zeros(self.n(b), np.int32)
        check(lib().sph_read_mat(self.h, b, _ip(out)))
        return out

    def fixed(self, b) -> np.ndarray:
        out = np.zeros(self.n(b), np.uint8)
        check(lib().sph_read_fixed(self.h, b, out.ctypes.data_as(_U8)))
        return out

    def set_fixed(self, b, fixed):
        f = np.ascontiguousarray(np.broadcast_to(fixed, (self.n(b),)), dtype=np.uint8)
        check(lib().sph_write_fixed(self.h, b, f.ctypes.data_as(_U8)))

    def conservation(self, b) -> Conservation:
        c = Conservation()
        check(lib().sph_conservation_get(self.h, b, C.byref(c)))
        return c

    def create_grazing(self, prm: Params, theta_deg, v, cppr=8, D=1000.0, tgt_mat=0, imp_mat=1,
                       x_impact_frac=None, start_h=None, rho_imp=7800.0, rho_target=2700.0):
        """The campaign's grazing IC (boundary_daemon.build_grazing_ic) generated in
        place: returns (impact, dx, n)."""
        s = GrazingSpec()
        lib().sph_grazing_spec_default(C.byref(s))
        s.theta_deg, s.v, s.D, s.cppr = theta_deg, v, D, cppr
        s.tgt_mat, s.imp_mat, s.rho_imp, s.rho_target = tgt_mat, imp_mat, rho_imp, rho_target
        s.x_impact_frac = float("nan") if x_impact_frac is None else x_impact_frac
        s.start_h = float("nan") if start_h is None else start_h
        b, dx, n = C.c_int32(), C.c_double(), C.c_int64()
        check(lib().sph_impact_create_grazing(self.h, C.byref(prm), C.byref(s), C.byref(b), C.byref(dx),
                                              C.byref(n)))
        return b.value, dx.value, n.value

    def diagnostics(self, b, mat_lo, mat_hi, u_melt=1.0e6) -> Diagnostics:
        """Projectile centroid, bulk velocity, speed, dispersion and melt count
        over materials mat_lo..mat_hi, reduced on the device."""
        d = Diagnostics()
        check(lib().sph_impact_diagnostics(self.h, b, mat_lo, mat_hi, u_melt, C.byref(d)))
        return d

    def eos(self, mat, rho, u):
        rho = _f64(rho)
        u = _f64(u)
        P = np.zeros_like(rho)
        cs = np.zeros_like(rho)
        check(lib().sph_eos_eval(self.h, mat, rho.size, _dp(rho), _dp(u), _dp(P), _dp(cs)))
        return P, cs

    def ref_cells(self, b):
        nc = np.zeros(3, np.int32)
        cw = np.zeros(3)
        # first call with a minimal start buffer reports nothing; size from the grid
        inf = self.info(b)
        n = int(inf.n)
        # the grid of the last build is reported by info only after a build; allocate generously
        ncell_guess = int(np.prod(np.maximum(np.array(inf.nc[:]), 1)))
        start = np.zeros(max(ncell_guess, 1) + 1, np.int32)
        ids = np.zeros(max(n, 1), np.int32)
        rc = lib().sph_debug_ref_cells(self.h, b, _ip(nc), _dp(cw), _ip(start), start.size, _ip(ids))
        if rc == -6:  # capacity: the grid changed, retry at its size
            start = np.zeros(int(np.prod(nc)) + 1, np.int32)
            rc = lib().sph_debug_ref_cells(self.h, b, _ip(nc), _dp(cw), _ip(start), start.size, _ip(ids))
        check(rc)
        ncell = int(np.prod(nc))
        return nc, cw, start[: ncell + 1], ids[:n]

    def neighbors(self, b, kind):
        n = self.n(b)
        counts = np.zeros(n, np.int32)
        total = np.zeros(1, np.int64)
        check(lib().sph_debug_neighbors(self.h, b, kind, _ip(counts), None, 0, total.ctypes.data_as(_I64)))
        ids = np.zeros(max(int(total[0]), 1), np.int32)
        check(lib().sph_debug_neighbors(self.h, b, kind, _ip(counts), _ip(ids), ids.size,
                                        total.ctypes.data_as(_I64)))
        return counts, ids[: int(total[0])]

    def flaws(self, b):
        """Device multi-flaw CSR of impact b: (ptr[n+1], eps[total])."""
        n = self.n(b)
        ptr = np.zeros(n + 1, np.int64)
        total = np.zeros(1, np.int64)
        check(lib().sph_debug_flaws(self.h, b, ptr.ctypes.data_as(_I64), None, 0, total.ctypes.data_as(_I64)))
        eps = np.zeros(max(int(total[0]), 1))
        check(lib().sph_debug_flaws(self.h, b, ptr.ctypes.data_as(_I64), _dp(eps), eps.size,
                                    total.ctypes.data_as(_I64)))
        return ptr, eps[: int(total[0])]

    def load_ic(self, path, prm: Params) -> int:
        b = C.c_int32()
        check(lib().sph_load_ic(self.h, str(path).encode(), C.byref(prm), C.byref(b)))
        return b.value

    def write_snapshot(self, b, path):
        check(lib().sph_write_snapshot(self.h, b, str(path).encode()))

    def write_checkpoint(self, b, path, dx):
        check(lib().sph_write_checkpoint(self.h, b, str(path).encode(), dx))

    def load_checkpoint(self, path, prm: Params):
        b = C.c_int32()
        dx = C.c_double()
        check(lib().sph_load_checkpoint(self.h, str(path).encode(), C.byref(prm), C.byref(b), C.byref(dx)))
        return b.value, dx.value

    def set_tuning(self, block=0, cell_factor=0.0):
        check(lib().sph_set_tuning(self.h, block, cell_factor))

    def set_option(self, key, value):
        check(lib().sph_set_option(self.h, key.encode(), float(value)))

    def get_option(self, key) -> float:
        v = C.c_double()
        check(lib().sph_get_option(self.h, key.encode(), C.byref(v)))
        return v.value

    def launches(self) -> int:
        v = C.c_int64()
        check(lib().sph_launch_count(self.h, C.byref(v)))
        return v.value

    def set_profiling(self, on=True):
        check(lib().sph_set_profiling(self.h, int(on)))

    def phase_times(self):
        ms = np.zeros(5)
        check(lib().sph_phase_times(self.h, _dp(ms)))
        return ms

    def kernel_stats(self):
        """{class name: (total device ms, launches)} accumulated while profiling."""
        out = {}
        for i, nm in enumerate(KERNEL_CLASSES):
            ms = C.c_double()
            n = C.c_int64()
            check(lib().sph_kernel_stats(self.h, i, C.byref(ms), C.byref(n)))
            out[nm] = (ms.value, n.value)
        return out

    def kernel_stats_reset(self):
        check(lib().sph_kernel_stats_reset(self.h))

    def event_record(self, slot):
        check(lib().sph_event_record(self.h, slot))

    def event_elapsed(self, a, b) -> float:
        ms = C.c_double()
        check(lib().sph_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value


# ------------------------------------------------------------------ System
class System:
    """Mirror of the reference `struct System` (hydrocodes/sph/sph.hpp:72-380).

    Parameters are plain attributes (eta, h_init, alpha, beta, eps, alpha_u, cfl,
    eps_as, as_n, damage_on); `materials` is a list; particles are added with
    `add` (or `add_many`) before `init`.  After the first device call the state
    lives on the GPU; fields are read with `field(name)` or the properties.
    """

    _PARAMS = ("eta", "h_init", "alpha", "beta", "eps", "alpha_u", "cfl", "eps_as", "as_n", "damage_on")

    def __init__(self, precision=FP64, device=0):
        self.precision = precision
        self.device = device
        # sph.hpp:86-92 defaults
        self.eta, self.h_init, self.alpha, self.beta, self.eps = 1.3, 0.01, 1.0, 2.0, 0.01
        self.alpha_u, self.cfl, self.eps_as, self.as_n, self.damage_on = 0.0, 0.2, 0.0, 4, False
        self.materials = []
        self.cur_mat = 0
        self._dom = (np.zeros(3), np.zeros(3), np.zeros(3, np.int32))
        self._pending = []
        self._seed = None
        self._h0 = None
        self.ctx = None
        self.b = None

    # -- construction (before the device) --
    def set_domain(self, xl, xh, px, yl, yh, py, zl, zh, pz):
        self._dom = (np.array([xl, yl, zl], float), np.array([xh, yh, zh], float),
                     np.array([px, py, pz], np.int32))

    def add(self, p, v, m, u, fixed=False):
        """System::add (sph.hpp:103-111)."""
        self._pending.append((np.asarray(p, float).reshape(1, 3), np.asarray(v, float).reshape(1, 3),
                              np.array([m], float), np.array([u], float),
                              np.array([self.cur_mat], np.int32), np.array([int(bool(fixed))], np.uint8),
                              self.h_init))

    def add_many(self, pos, vel, mass, u, mat=None, fixed=None):
        pos = np.asarray(pos, float).reshape(-1, 3)
        n = pos.shape[0]
        mat = np.full(n, self.cur_mat, np.int32) if mat is None else np.broadcast_to(mat, (n,)).astype(np.int32)
        fixed = np.zeros(n, np.uint8) if fixed is None else np.broadcast_to(fixed, (n,)).astype(np.uint8)
        self._pending.append((pos, np.asarray(vel, float).reshape(-1, 3), np.broadcast_to(mass, (n,)).astype(float),
                              np.broadcast_to(u, (n,)).astype(float), mat, fixed, self.h_init))

    def seed_damage(self, dx, seed=12345):
        """System::seed_damage (sph.hpp:117-128)."""
        if self.ctx is None:
            self._seed = ("single", dx, seed)
        else:
            self.ctx.seed_damage(self.b, dx, seed)

    def seed_flaws_multi(self, dx, seed=12345):
        if self.ctx is None:
            self._seed = ("multi", dx, seed)
        else:
            self.ctx.seed_flaws_multi(self.b, dx, seed)

    def set_h0(self, h0):
        self._h0 = np.asarray(h0, float)
        if self.ctx is not None:
            self.ctx.set_h0(self.b, self._h0)

    def _params(self) -> Params:
        return params(**{k: (int(getattr(self, k)) if k in ("as_n", "damage_on") else float(getattr(self, k)))
                         for k in self._PARAMS})

    def _materialize(self):
        if self.ctx is not None:
            self.ctx.set_params(self.b, self._params())
            return
        self.ctx = Context(self.precision, self.device)
        for m in self.materials:
            self.ctx.add_material(m)
        lo, hi, per = self._dom
        self.b = self.ctx.impact_create(self._params(), lo, hi, per)
        if self._pending:
            pos = np.concatenate([p[0] for p in self._pending])
            vel = np.concatenate([p[1] for p in self._pending])
            mass = np.concatenate([p[2] for p in self._pending])
            u = np.concatenate([p[3] for p in self._pending])
            mat = np.concatenate([p[4] for p in self._pending])
            fixed = np.concatenate([p[5] for p in self._pending])
            self.ctx.add_particles(self.b, pos, vel, mass, u, mat, fixed)
            hs = np.concatenate([np.full(len(p[0]), p[6]) for p in self._pending])
            if np.any(hs != self.h_init) and self._h0 is None:
                self.ctx.write(self.b, "hh", hs)
        self._pending = []
        if self._seed is not None:
            kind, dx, seed = self._seed
            if kind == "single":
                self.ctx.seed_damage(self.b, dx, seed)
            else:
                self.ctx.seed_flaws_multi(self.b, dx, seed)
        if self._h0 is not None:
            self.ctx.set_h0(self.b, self._h0)

    # -- stepping --
    def init(self):
        """System::init (sph.hpp:379)."""
        self._materialize()
        self.ctx.init()

    def timestep(self) -> float:
        """System::timestep (sph.hpp:350-355)."""
        self._materialize()
        return self.ctx.timestep(self.b)

    def step(self, dt):
        """System::step (sph.hpp:357-377)."""
        self._materialize()
        self.ctx.step(dt)

    def compute_density_h(self, iters=2):
        self._materialize()
        self.ctx.compute_density_h(iters)

    def compute_forces(self):
        self._materialize()
        self.ctx.compute_forces()

    # -- fields --
    @property
    def n(self):
        if self.ctx is None:
            return sum(len(p[0]) for p in self._pending)
        return self.ctx.n(self.b)

    def field(self, name):
        self._materialize()
        return self.ctx.read(self.b, name)

    def set_field(self, name, values):
        self._materialize()
        self.ctx.write(self.b, name, values)

    def fields(self, names=FIELDS):
        return {k: self.field(k) for k in names}

    def _vec(self, a, b, c):
        return np.stack([self.field(a), self.field(b), self.field(c)], axis=1)

    pos = property(lambda s: s._vec("x", "y", "z"))
    vel = property(lambda s: s._vec("vx", "vy", "vz"))
    acc = property(lambda s: s._vec("ax", "ay", "az"))
    rho = property(lambda s: s.field("rho"))
    u = property(lambda s: s.field("u"))
    hh = property(lambda s: s.field("hh"))
    P = property(lambda s: s.field("P"))
    D = property(lambda s: s.field("D"))

    @property
    def mat(self):
        self._materialize()
        return self.ctx.mat(self.b)

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None
