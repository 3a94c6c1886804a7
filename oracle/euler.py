"""ctypes front end for the CPU oracle of the Eulerian grid hydrocode
(TEST INFRASTRUCTURE ONLY).

Two back ends with one interface:
  * OracleGrid -- oracle/liborc.so (eorc_*), the C restatement of the
    reference's CPU Euler solver (hydrocodes/euler/hydro_cpu.cpp);
  * RefGrid    -- oracle/_ref/libeulerref.so (eref_*), the reference's own
    hydro_cpu.cpp compiled unmodified (only where the reference tree is
    present).

Only tests/ and bench.py's CPU legs import this.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import oracle as O

REF_SO = os.path.join(O.HERE, "_ref", "libeulerref.so")

FIELDS = "r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D af rc vib Pmax".split()
RHS = "r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D rc vib".split()


class Params(C.Structure):
    """Layout of eorc_params: the file-scope settings of hydro_cpu.cpp:15-36."""

    _fields_ = [(n, C.c_double) for n in ("gz tdec eta_af c_act p_coh p_act rho_cfl damp rho_vac "
                                          "y_i0 mu_i mu_d y_d0 y_m y_bingham c_reg af_sat").split()] + [
        (n, C.c_int32) for n in "axisym rock af_reg af_prel af_seeddp pad_".split()] + [("void_amb", C.c_double), ("void_cons", C.c_int32), ("visc_imp", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if not n.startswith("pad")}


_D = C.POINTER(C.c_double)


def _declare(lib, p):
    sig = {
        f"{p}params_default": (None, [C.POINTER(Params)]),
        f"{p}create": (C.c_void_p, [C.c_int, C.c_int, C.c_int, C.c_double]),
        f"{p}destroy": (None, [C.c_void_p]),
        f"{p}set_material": (None, [C.c_void_p, C.POINTER(O.Material)]),
        f"{p}set_params": (None, [C.c_void_p, C.POINTER(Params)]),
        f"{p}field": (_D, [C.c_void_p, C.c_char_p]),
        f"{p}rhs": (_D, [C.c_void_p, C.c_char_p]),
        f"{p}lop": (None, [C.c_void_p]),
        f"{p}vonmises": (None, [C.c_void_p, C.c_int]),
        f"{p}grow_damage": (None, [C.c_void_p, C.c_double]),
        f"{p}update_af": (None, [C.c_void_p, C.c_double]),
        f"{p}maxspeed": (C.c_double, [C.c_void_p]),
        f"{p}step_rk2": (None, [C.c_void_p, C.c_double]),
        f"{p}run": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _D]),
        f"{p}pcell": (C.c_double, [C.c_void_p, C.c_int]),
        f"{p}set_ref": (None, [C.c_void_p]),
        f"{p}clear_ref": (None, [C.c_void_p]),
        f"{p}implicit_visc": (None, [C.c_void_p, C.c_double]),
        f"{p}visc_iters": (C.c_long, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


_ref = None
_declared = False


def _orc():
    global _declared
    lib = O.lib()
    if not _declared:
        _declare(lib, "eorc_")
        _declared = True
    return lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _eref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference Euler shim not built (make -C oracle ref)")
        _ref = C.CDLL(REF_SO)
        _declare(_ref, "eref_")
    return _ref


def default_params(ref=False) -> Params:
    p = Params()
    (_eref().eref_params_default if ref else _orc().eorc_params_default)(C.byref(p))
    return p


class _Grid:
    _prefix = ""

    def __init__(self, nx, ny, nz, dx, material=None, params=None):
        self._lib = self._load()
        self.shape = (int(nx), int(ny), int(nz))
        self.n = int(nx) * int(ny) * int(nz)
        self.dx = float(dx)
        self.h = self._f("create")(int(nx), int(ny), int(nz), float(dx))
        if material is not None:
            self.set_material(material)
        self.params = default_params(ref=self._prefix == "eref_")
        if params:
            self.set_params(params)

    def _f(self, name):
        return getattr(self._lib, self._prefix + name)

    def set_material(self, m: O.Material):
        self.material = m
        self._f("set_material")(self.h, C.byref(m))

    def set_params(self, values: dict):
        for k, v in values.items():
            setattr(self.params, k, v)
        self._f("set_params")(self.h, C.byref(self.params))

    def _view(self, getter, name):
        p = self._f(getter)(self.h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(self.n,))

    def field(self, name):
        return self._view("field", name).copy()

    def set_field(self, name, values):
        self._view("field", name)[:] = np.asarray(values, dtype=np.float64).reshape(-1)

    def rhs(self, name):
        return self._view("rhs", name).copy()

    def fields(self, names=FIELDS):
        return {k: self.field(k) for k in names}

    def lop(self):
        self._f("lop")(self.h)

    def vonmises(self, reg=True):
        self._f("vonmises")(self.h, int(reg))

    def grow_damage(self, dt):
        self._f("grow_damage")(self.h, float(dt))

    def update_af(self, dt):
        self._f("update_af")(self.h, float(dt))

    def maxspeed(self) -> float:
        return self._f("maxspeed")(self.h)

    def step(self, dt):
        self._f("step_rk2")(self.h, float(dt))

    def run(self, cfl, t_end, max_steps=-1):
        t = np.zeros(1)
        s = self._f("run")(self.h, float(cfl), float(t_end), int(max_steps), t.ctypes.data_as(_D))
        return int(s), float(t[0])

    def pcell(self, c) -> float:
        return self._f("pcell")(self.h, int(c))

    def set_ref(self):
        """set_ref: the current density and pressure become the hydrostatic reference."""
        self._f("set_ref")(self.h)

    def clear_ref(self):
        self._f("clear_ref")(self.h)

    def implicit_visc(self, dt):
        """implicit_visc(g, dt): the backward-Euler fluidization viscosity."""
        self._f("implicit_visc")(self.h, float(dt))

    def visc_iters(self) -> int:
        """Conjugate-gradient iterations of the implicit viscosity so far."""
        return int(self._f("visc_iters")(self.h))

    def close(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleGrid(_Grid):
    _prefix = "eorc_"

    @staticmethod
    def _load():
        return _orc()


class RefGrid(_Grid):
    _prefix = "eref_"

    @staticmethod
    def _load():
        return _eref()


def from_case(case, cls=OracleGrid):
    """A grid loaded with a workload case (deorbit_gb300.grid_ic.Case)."""
    g = cls(*case.shape, case.dx, material=O.material_from_dict(case.material), params=case.params)
    for k, v in case.fields.items():
        g.set_field(k, v)
    if getattr(case, "set_ref", False):
        g.set_ref()
        for k, v in case.post_ref.items():
            g.set_field(k, v)
    return g


PIN_STRESS, VOID_AMBIENT, TRACK_PMAX = 1, 2, 4  # the C ABI's EU_DRIVER_* flags


def drive(g, case, pin=None, isp=None, flags=None):
    """The reference drivers' own adjustments after a step, in the order the
    CUDA solver's eu_set_driver applies them: the lowest `pin` (default
    case.pin_floor) z-layers back to the reference density at rest with no
    energy (PIN_STRESS: no deviatoric stress either; hydro_cpu.cpp:634, 855,
    893-894); columns i >= isp (default case.sponge_from) relaxed toward the
    reference with weight ((i - isp) / max(1, nx - 1 - isp))^2 (635-637);
    VOID_AMBIENT: cells below RHO_CFL to ambient gas at rest, no energy and
    stress (823-824); TRACK_PMAX: Pmax = max(Pmax, Pcell) (769).  The
    reference density is the case's pre-impact field (what set_ref froze)."""
    nx, ny, nz = case.shape
    pin = case.pin_floor if pin is None else pin
    isp = getattr(case, "sponge_from", -1) if isp is None else isp
    flags = getattr(case, "driver_flags", 0) if flags is None else flags
    if not pin and isp < 0 and not flags:
        return
    names = ("r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz")
    f = {k: g.field(k).reshape(nx, ny, nz) for k in names}
    if pin or isp >= 0:
        ref = np.asarray(case.fields["r"], dtype=np.float64).reshape(nx, ny, nz)
    if pin:
        f["r"][:, :, :pin] = ref[:, :, :pin]
        for k in ("mu", "mv", "mw", "E") + (names[5:] if flags & PIN_STRESS else ()):
            f[k][:, :, :pin] = 0.0
    if isp >= 0:
        for i in range(isp, nx):
            xi = float(i - isp) / max(1, nx - 1 - isp)
            sp = xi * xi
            f["r"][i] = (1 - sp) * f["r"][i] + sp * ref[i]
            for k in ("mu", "mv", "mw", "E"):
                f[k][i] *= (1 - sp)
    if flags & VOID_AMBIENT:
        v = f["r"] < g.params.rho_cfl
        f["r"][v] = 0.27
        for k in names[1:]:
            f[k][v] = 0.0
    for k, a in f.items():
        g.set_field(k, a)
    if flags & TRACK_PMAX:
        pm = g.field("Pmax")
        P = np.array([g.pcell(c) for c in range(g.n)])
        g.set_field("Pmax", np.where(P > pm, P, pm))


def run_case(g, case, steps):
    """The drivers' loop on a grid built from `case` (steps of step_rk2 at
    dt = cfl dx / maxspeed clipped at t_end), with the case's floor pin and
    sponge after every step (hydro_cpu.cpp:634-637, 855): returns (steps, t)."""
    if not case.pin_floor and getattr(case, "sponge_from", -1) < 0 and not getattr(case, "driver_flags", 0):
        return g.run(case.cfl, case.t_end, steps)
    t, s = 0.0, 0
    while t < case.t_end and s < steps:
        dt = case.cfl * case.dx / g.maxspeed()
        if t + dt > case.t_end:
            dt = case.t_end - t
        g.step(dt)
        drive(g, case)
        t += dt
        s += 1
    return s, t


class DrivenGrid:
    """An oracle (or reference) grid behind the interface the crater driver
    (deorbit_gb300.crater.run) uses: the drivers' loop from the grid's own
    time with the floor pin and sponge after every step."""

    def __init__(self, case, cls=OracleGrid):
        self.case = case
        self.g = from_case(case, cls)
        self.t = 0.0
        self.pin, self.isp, self.flags = 0, -1, 0

    def set_driver(self, pin_floor=0, sponge_from=-1, flags=0):
        self.pin, self.isp, self.flags = int(pin_floor), int(sponge_from), int(flags)

    def reference(self):
        return np.asarray(self.case.fields["r"], dtype=np.float64).copy(), None

    def run(self, cfl, t_end, max_steps=-1):
        s = 0
        while self.t < t_end and (max_steps < 0 or s < max_steps):
            dt = cfl * self.g.dx / self.g.maxspeed()
            if self.t + dt > t_end:
                dt = t_end - self.t
            self.g.step(dt)
            drive(self.g, self.case, self.pin, self.isp, self.flags)
            self.t += dt
            s += 1
        return s, self.t

    def read(self, name):
        return self.g.field(name)

    def pressure(self):
        return np.array([self.g.pcell(c) for c in range(self.g.n)])

    def close(self):
        self.g.close()
