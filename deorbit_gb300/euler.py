"""Python front end of the GB300 Eulerian grid hydrocode (include/deorbit_euler.h).

`Grid` mirrors the reference's CPU Euler solver (hydrocodes/euler/hydro_cpu.cpp):
the grid of conserved and material fields (hydro_cpu.cpp:90-93) with the
operators Lop (98-214), vonmises (229-252), grow_damage (253-258), update_af
(390-410), maxspeed (378-380) and step_rk2 (411-425), plus the drivers' time
loop (`run`, hydro_cpu.cpp:452) with dt and the stop test on the device.  The
reference's file-scope settings (GZ, TDEC, ROCK, RHO_CFL, ...) are per-grid
parameters with the same names in lower case; its global MAT is the grid's
material.  Every call runs CUDA kernels of libdeorbit_sph.so; there is no
CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import sph

FIELDS = "r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D af rc vib Pmax".split()
FP64, MIXED = 0, 1  # eu_form: the Lop in FP64 (reference order) or in FP32 (state FP64)
# eu_set_driver flags
DRIVER_PIN_STRESS, DRIVER_VOID_AMBIENT, DRIVER_TRACK_PMAX = 1, 2, 4
RHS = "r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D rc vib".split()


class Params(C.Structure):
    """eu_params: the settings of hydro_cpu.cpp:17-36 and 222-223."""

    _fields_ = [(n, C.c_double) for n in ("gz tdec eta_af c_act p_coh p_act rho_cfl damp rho_vac "
                                          "y_i0 mu_i mu_d y_d0 y_m y_bingham c_reg af_sat").split()] + [
        (n, C.c_int32) for n in "axisym rock af_reg af_prel af_seeddp reserved".split()] + [("void_amb", C.c_double), ("void_cons", C.c_int32), ("visc_imp", C.c_int32)]


_D = C.POINTER(C.c_double)
_P = C.c_void_p
_SIGS = {
    "eu_params_default": (None, [C.POINTER(Params)]),
    "eu_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(_P)]),
    "eu_create_form": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                 C.POINTER(_P)]),
    "eu_destroy": (C.c_int, [_P]),
    "eu_set_material": (C.c_int, [_P, C.POINTER(sph.Material)]),
    "eu_set_params": (C.c_int, [_P, C.POINTER(Params)]),
    "eu_get_shape": (C.c_int, [_P, C.POINTER(C.c_int32), _D]),
    "eu_write_field": (C.c_int, [_P, C.c_char_p, _D, C.c_int64]),
    "eu_read_field": (C.c_int, [_P, C.c_char_p, _D, C.c_int64]),
    "eu_write_fields": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D), C.c_int64]),
    "eu_read_fields": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(_D), C.c_int64]),
    "eu_lop": (C.c_int, [_P]),
    "eu_read_rhs": (C.c_int, [_P, C.c_char_p, _D, C.c_int64]),
    "eu_vonmises": (C.c_int, [_P, C.c_int32]),
    "eu_grow_damage": (C.c_int, [_P, C.c_double]),
    "eu_update_af": (C.c_int, [_P, C.c_double]),
    "eu_maxspeed": (C.c_int, [_P, _D]),
    "eu_read_pressure": (C.c_int, [_P, _D, C.c_int64]),
    "eu_step": (C.c_int, [_P, C.c_double]),
    "eu_run": (C.c_int, [_P, C.c_double, C.c_double, C.c_int64, C.POINTER(C.c_int64), _D]),
    "eu_set_time": (C.c_int, [_P, C.c_double]),
    "eu_get_time": (C.c_int, [_P, _D]),
    "eu_synchronize": (C.c_int, [_P]),
    "eu_event_record": (C.c_int, [_P, C.c_int32]),
    "eu_event_elapsed": (C.c_int, [_P, C.c_int32, C.c_int32, _D]),
    "eu_device_bytes": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "eu_launches": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "eu_set_ref": (C.c_int, [_P]),
    "eu_clear_ref": (C.c_int, [_P]),
    "eu_read_ref": (C.c_int, [_P, _D, _D, C.c_int64]),
    "eu_implicit_visc": (C.c_int, [_P, C.c_double]),
    "eu_set_driver": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "eu_visc_iterations": (C.c_int, [_P, C.POINTER(C.c_int64)]),
}
_declared = False


def lib():
    """The CUDA library with the grid solver's entry points declared (raises
    if it is not built)."""
    global _declared
    L = sph.lib()
    if not _declared:
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _declared = True
    return L


def default_params() -> Params:
    p = Params()
    lib().eu_params_default(C.byref(p))
    return p


def _material(m) -> sph.Material:
    if isinstance(m, sph.Material):
        return m
    out = sph.Material()
    for name, _ in sph.Material._fields_:
        setattr(out, name, int(m[name]) if name in ("type", "yield_model") else float(m[name]))
    return out


class Grid:
    """One Eulerian grid on one GPU (the reference's `Grid`, hydro_cpu.cpp:90-93)."""

    def __init__(self, nx, ny, nz, dx, material=None, params=None, device=0, form=FP64):
        L = lib()
        h = _P()
        sph.check(L.eu_create_form(int(nx), int(ny), int(nz), float(dx), int(device), int(form), C.byref(h)))
        self.form = int(form)
        self.h = h
        self.shape = (int(nx), int(ny), int(nz))
        self.n = int(nx) * int(ny) * int(nz)
        self.dx = float(dx)
        self.params = default_params()
        if material is not None:
            self.set_material(material)
        if params:
            self.set_params(params)

    # -- settings
    def set_material(self, m):
        self._mat = _material(m)
        sph.check(lib().eu_set_material(self.h, C.byref(self._mat)))

    def set_params(self, values: dict):
        for k, v in values.items():
            if not hasattr(self.params, k):
                raise KeyError(k)
            setattr(self.params, k, v)
        sph.check(lib().eu_set_params(self.h, C.byref(self.params)))

    # -- fields
    def write(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if a.size != self.n:
            raise ValueError(f"{name}: {a.size} values for {self.n} cells")
        sph.check(lib().eu_write_field(self.h, name.encode(), a.ctypes.data_as(_D), self.n))

    def read(self, name, out=None):
        out = np.empty(self.n) if out is None else out
        sph.check(lib().eu_read_field(self.h, name.encode(), out.ctypes.data_as(_D), self.n))
        return out

    def write_many(self, fields: dict):
        names = list(fields)
        arrs = [np.ascontiguousarray(fields[k], dtype=np.float64).reshape(-1) for k in names]
        for k, a in zip(names, arrs):
            if a.size != self.n:
                raise ValueError(f"{k}: {a.size} values for {self.n} cells")
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        cp = (_D * len(names))(*[a.ctypes.data_as(_D) for a in arrs])
        sph.check(lib().eu_write_fields(self.h, len(names), cn, cp, self.n))

    def read_many(self, names, outs=None):
        names = list(names)
        outs = [np.empty(self.n) for _ in names] if outs is None else list(outs)
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        cp = (_D * len(names))(*[o.ctypes.data_as(_D) for o in outs])
        sph.check(lib().eu_read_fields(self.h, len(names), cn, cp, self.n))
        return dict(zip(names, outs))

    def fields(self, names=FIELDS):
        return self.read_many(names)

    def set_ref(self):
        """set_ref (hydro_cpu.cpp:259-261): the current density and pressure
        become the hydrostatic reference (well-balanced sweep, void reset)."""
        sph.check(lib().eu_set_ref(self.h))

    def clear_ref(self):
        sph.check(lib().eu_clear_ref(self.h))

    def set_driver(self, pin_floor=0, sponge_from=-1, flags=0):
        """Per-step driver adjustments applied on the device after every step
        (eu_set_driver): floor pin, radial sponge, DRIVER_* flags."""
        sph.check(lib().eu_set_driver(self.h, int(pin_floor), int(sponge_from), int(flags)))

    def reference(self):
        r0, p0 = np.empty(self.n), np.empty(self.n)
        sph.check(lib().eu_read_ref(self.h, r0.ctypes.data_as(_D), p0.ctypes.data_as(_D), self.n))
        return r0, p0

    def pressure(self):
        out = np.empty(self.n)
        sph.check(lib().eu_read_pressure(self.h, out.ctypes.data_as(_D), self.n))
        return out

    # -- operators of the reference
    def lop(self):
        sph.check(lib().eu_lop(self.h))

    def rhs(self, name):
        out = np.empty(self.n)
        sph.check(lib().eu_read_rhs(self.h, name.encode(), out.ctypes.data_as(_D), self.n))
        return out

    def vonmises(self, reg=True):
        sph.check(lib().eu_vonmises(self.h, int(reg)))

    def grow_damage(self, dt):
        sph.check(lib().eu_grow_damage(self.h, float(dt)))

    def update_af(self, dt):
        sph.check(lib().eu_update_af(self.h, float(dt)))

    def implicit_visc(self, dt):
        """implicit_visc(g, dt): the backward-Euler fluidization viscosity."""
        sph.check(lib().eu_implicit_visc(self.h, float(dt)))

    def visc_iters(self) -> int:
        """Conjugate-gradient iterations of the implicit viscosity so far."""
        v = C.c_int64()
        sph.check(lib().eu_visc_iterations(self.h, C.byref(v)))
        return v.value

    def maxspeed(self) -> float:
        v = C.c_double()
        sph.check(lib().eu_maxspeed(self.h, C.byref(v)))
        return v.value

    def step(self, dt):
        """step_rk2 at a host dt."""
        sph.check(lib().eu_step(self.h, float(dt)))

    def run(self, cfl, t_end, max_steps=-1):
        """The drivers' loop from the grid's current time: returns (steps, t)."""
        s = C.c_int64()
        t = C.c_double()
        sph.check(lib().eu_run(self.h, float(cfl), float(t_end), int(max_steps), C.byref(s), C.byref(t)))
        return s.value, t.value

    def set_time(self, t):
        sph.check(lib().eu_set_time(self.h, float(t)))

    def time(self) -> float:
        t = C.c_double()
        sph.check(lib().eu_get_time(self.h, C.byref(t)))
        return t.value

    # -- measurement
    def synchronize(self):
        sph.check(lib().eu_synchronize(self.h))

    def event_record(self, slot):
        sph.check(lib().eu_event_record(self.h, int(slot)))

    def event_elapsed(self, a, b) -> float:
        ms = C.c_double()
        sph.check(lib().eu_event_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value

    def device_bytes(self) -> int:
        v = C.c_int64()
        sph.check(lib().eu_device_bytes(self.h, C.byref(v)))
        return v.value

    def launches(self) -> int:
        v = C.c_int64()
        sph.check(lib().eu_launches(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            lib().eu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def from_case(case, device=0, form=FP64) -> Grid:
    """A grid loaded with a workload case (grid_ic.Case)."""
    g = Grid(*case.shape, case.dx, material=case.material, params=case.params, device=device, form=form)
    g.write_many(case.fields)
    if getattr(case, "set_ref", False):
        g.set_ref()
        if case.post_ref:
            g.write_many(case.post_ref)
    return g


def run_case(g, case, steps):
    """The drivers' loop on a grid built from `case`, with the case's floor pin
    and radial sponge applied on the device after every step
    (hydro_cpu.cpp:634-637, 855)."""
    if case.pin_floor or case.sponge_from >= 0 or case.driver_flags:
        g.set_driver(case.pin_floor, case.sponge_from, case.driver_flags)
    return g.run(case.cfl, case.t_end, steps)
