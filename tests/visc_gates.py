"""The reference driver's implicit-viscosity gates (hydrocodes/euler/
hydro_cpu.cpp modes visc_diff, visc_agree, visc_energy, vib_regen,
bingham_slope), at its sizes and with its pass criteria, for any grid with
the deorbit_gb300.euler Grid interface (read, write, set_params, set_driver,
implicit_visc, update_af, run from the grid's own time, visc_iters, close).
The GPU tests run them all on the CUDA solver; the oracle tests run the first
four on the oracle through `OracleGrid` below (bingham_slope takes ~10^5
steps).

Each gate returns (passed, the measured quantities).
"""
import math

import numpy as np

from deorbit_gb300 import grid_ic as GI


class OracleGrid:
    """The Grid interface over an oracle grid (oracle.euler), with the
    drivers' loop continuing from the grid's own time as eu_run does."""

    def __init__(self, case):
        from oracle import euler as EO
        self.EO, self.case = EO, case
        self.g = EO.from_case(case)
        self.t = 0.0
        self.pin, self.isp, self.flags = 0, -1, 0

    def set_driver(self, pin_floor=0, sponge_from=-1, flags=0):
        self.pin, self.isp, self.flags = pin_floor, sponge_from, flags

    def read(self, name):
        return self.g.field(name)

    def write(self, name, values):
        self.g.set_field(name, values)

    def set_params(self, prm):
        self.g.set_params(prm)

    def implicit_visc(self, dt):
        self.g.implicit_visc(dt)

    def update_af(self, dt):
        self.g.update_af(dt)

    def visc_iters(self):
        return self.g.visc_iters()

    def lop(self):
        self.g.lop()

    def rhs(self, name):
        return self.g.rhs(name)

    def pressure(self):
        return np.array([self.g.pcell(c) for c in range(self.g.n)])

    def run(self, cfl, t_end, max_steps=-1):
        s = 0
        while self.t < t_end and (max_steps < 0 or s < max_steps):
            dt = cfl * self.g.dx / self.g.maxspeed()
            if self.t + dt > t_end:
                dt = t_end - self.t
            self.g.step(dt)
            self.EO.drive(self.g, self.case, self.pin, self.isp, self.flags)
            self.t += dt
            s += 1
        return s, self.t

    def close(self):
        self.g.close()


def visc_diff(make):
    """hydro_cpu.cpp:907-946: (A) each backward-Euler application scales the
    cosine mode by exactly 1 / (1 + nu lam dt) (implied nu within 1e-6), the
    decay tracks exp(-nu k^2 t) within 10 %, the v_z mode decays by the same
    factor to 1e-6; (B) the cylindrical v_r = A r is untouched near the axis
    (1e-5) and v_z = const stays constant (1e-10)."""
    N, m, nu, NS, A0 = 256, 4, 1.0, 12, 1.0
    case = GI.visc_mode(N, m, nu)
    dx = case.dx
    kk = m * math.pi / (N * dx)
    lam = (2.0 - 2.0 * math.cos(kk * dx)) / (dx * dx)
    dtv = 20.0 * dx * dx / (2.0 * nu)
    ph = np.cos(kk * (np.arange(N) + 0.5) * dx)
    den = float(np.sum(ph * ph))
    g = make(case)
    amp, worst = A0, 0.0
    for _ in range(NS):
        g.implicit_visc(dtv)
        a1 = float(np.sum(g.read("mv") / g.read("r") * ph)) / den
        f = a1 / amp
        amp = a1
        worst = max(worst, abs((1.0 / f - 1.0) / (lam * dtv) - nu) / nu)
    fex = 1.0 / (1.0 + nu * lam * dtv)
    ampz = float(np.sum(g.read("mw") / g.read("r") * ph)) / den
    expz = 0.5 * A0 * fex ** NS
    zerr = abs(ampz - expz) / expz
    exact = A0 * math.exp(-nu * kk * kk * NS * dtv)
    g.close()
    ok_a = worst < 1e-6 and abs(amp - exact) / exact < 0.10 and zerr < 1e-6

    Nr, Nz, A0r, W0 = 64, 8, 1e-2, 3.0
    case = GI.visc_axi(Nr, Nz, A0r, W0, nu)
    g = make(case)
    g.implicit_visc(10.0 * case.dx * case.dx / nu)
    v_r = (g.read("mu") / g.read("r")).reshape(Nr, Nz)
    v_z = (g.read("mw") / g.read("r")).reshape(Nr, Nz)
    g.close()
    r = (np.arange(Nr) + 0.5)[:, None] * case.dx
    eru = float(np.max(np.abs(v_r[:20] - A0r * r[:20]) / (A0r * Nr * case.dx)))
    erw = float(np.max(np.abs(v_z[:20] - W0) / W0))
    ok_b = eru < 1e-5 and erw < 1e-10
    return ok_a and ok_b, {"nu_err": worst, "amp": amp, "exact": exact, "vz_err": zerr, "vr_null": eru,
                           "vz_const": erw}


def _mode(g, case, m=24):
    N = case.shape[0]
    kk = m * math.pi / (N * case.dx)
    ph = np.cos(kk * (np.arange(N) + 0.5) * case.dx)
    vy = g.read("mv") / g.read("r")
    return vy, float(np.sum(vy * ph) / np.sum(ph * ph))


def visc_agree(make):
    """hydro_cpu.cpp:947-967: at eta = 1e8 (both schemes stable) the explicit
    (Lop) and implicit viscous runs of the full step agree to 1e-3 A0 after
    25 s, and the mode has decayed by more than 1 %."""
    out = []
    for vi in (0, 1):
        case = GI.visc_slab(eta=1e8, A0=1.0, t_end=25.0, visc_imp=vi)
        g = make(case)
        g.run(case.cfl, case.t_end)
        out.append(_mode(g, case))
        g.close()
    (vy1, amp1), (vy2, amp2) = out
    dmax = float(np.max(np.abs(vy1 - vy2)))
    dec = 1.0 - amp1 / 1.0
    return dmax < 1e-3 and dec > 0.01, {"dmax": dmax, "amp_explicit": amp1, "amp_implicit": amp2}


def visc_energy(make):
    """hydro_cpu.cpp:968-987: at eta = 5e11 (nu dt / dx^2 ~ 30) more than half
    of the mode's kinetic energy is dissipated in 5 s, all of it reappears as
    internal energy (to 1e-4 of KE0) and the total is conserved to 1e-4."""
    case = GI.visc_slab(eta=5e11, A0=2.0, t_end=5.0)

    def energies(g):
        r, e = g.read("r"), g.read("E")
        ke = 0.5 * (g.read("mu") ** 2 + g.read("mv") ** 2 + g.read("mw") ** 2) / r
        return float(e.sum()), float(ke.sum()), float((e - ke).sum())

    g = make(case)
    E0, KE0, _ = energies(g)
    g.run(case.cfl, case.t_end)
    E1, KE1, IE1 = energies(g)
    iters = g.visc_iters()
    g.close()
    drift, keloss, heat = abs(E1 - E0) / KE0, (KE0 - KE1) / KE0, IE1 / KE0
    ok = drift < 1e-4 and abs(heat - keloss) < 1e-4 and keloss > 0.5 and iters > 0
    return ok, {"drift": drift, "ke_lost": keloss, "heat": heat, "cg_iters": iters}


def vib_regen(make):
    """hydro_cpu.cpp:988-1027: with regeneration (C_REG = 1) the shear flow
    sustains the vibrations (> 3x the control at 10 s) and they re-lock once
    the shear has died (at 40 s below 0.3x their 10 s level); the bookkeeping
    conserves KE + IE + rho vib^2 / 2 to 2e-2 with and without regeneration;
    a huge vibration saturates at AF_SAT x the overburden."""
    T1, T2 = 10.0, 40.0
    v1, v2, drift = [], [], []
    for cs in range(3):
        case = GI.vib_slab(cs, t_end=T2)
        N = case.shape[0]
        rho0, A0, vib0 = case.material["rho0"], 10.0, 10.0
        g = make(case)

        def etot():
            return float(np.sum(g.read("E") + 0.5 * g.read("r") * g.read("vib") ** 2))

        E0 = etot()
        t = 0.0
        while t < T1:  # the driver records vib at the first step end past T1
            _, t = g.run(case.cfl, T2, 1)
        v1.append(float(g.read("vib").mean()))
        g.run(case.cfl, T2)
        v2.append(float(g.read("vib").mean()))
        KE0, EV0 = 0.5 * rho0 * A0 * A0 * 0.5, 0.5 * rho0 * vib0 * vib0
        drift.append((etot() - E0) / (N * (KE0 + EV0)))
        g.close()
    case = GI.vib_slab(2, N=4)  # saturation: huge vibrations, one fluidization update
    rho0 = case.material["rho0"]
    g = make(case)
    g.set_params({"af_sat": 1.0})
    g.write("vib", np.full(4, 1e3))
    g.write("E", np.zeros(4))
    g.write("mv", np.zeros(4))
    g.update_af(1e-9)
    vib, af = g.read("vib"), g.read("af")
    g.close()
    pvib = rho0 * sound_speed(case.material, rho0, 0.0) * float(vib[1])
    sat = pvib <= 1.01 * 1.0 * 1e6 and af[1] <= 0.51
    ok = abs(drift[1]) < 2e-2 and abs(drift[2]) < 2e-2 and v1[2] > 3.0 * v1[1] and v2[2] < 0.3 * v1[2] and sat
    return ok, {"vib_T1": v1, "vib_T2": v2, "drift": drift, "pvib": pvib, "af": float(af[1])}


def sound_speed(mat, rho, u):
    """MAT.sound_speed(rho, u) through the oracle's EOS (eos.hpp:95-113)."""
    import ctypes as C

    from oracle import oracle as O
    f = O.lib().orc_sound_speed
    f.restype = C.c_double
    f.argtypes = [C.POINTER(O.Material), C.c_double, C.c_double]
    m = O.material_from_dict(mat)
    return float(f(C.byref(m), float(rho), float(u)))


def bingham_slope(make):
    """hydro_cpu.cpp:1028-1077: a fluidized heap on an intact substrate with
    the implicit viscosity: (A) with the Bingham floor at 2.5x the peak flank
    stress the peak holds (> 92 % of H after 400 s); (B) at 0.2x it flows
    (peak < 75 % of H) and then arrests (peak decay over the last 400 s of
    1200 s below 15 % of the first 400 s, steepest flank stress within 8x the
    yield envelope); (C) with no floor (Newtonian control) it keeps
    collapsing (late decay > 3x case B's, lower peak).  The heap height is the
    column mass above the substrate plane, sampled at the first step end past
    every 100 s."""
    res = []
    for cs in range(3):
        case = GI.bingham_heap(cs)
        nx, _, nz = case.shape
        dx, rho0, z0, H = case.dx, case.material["rho0"], 1500.0, 2000.0
        gz = case.params["gz"]
        yb = case.params["y_bingham"]
        tauy = yb / math.sqrt(3.0) if yb > 0 else 1e30
        g = make(case)
        g.set_driver(case.pin_floor, -1)

        def surf(r):
            r = r.reshape(nx, nz)
            m = np.cumsum(np.where(r > 100.0, r, 0.0), axis=1)[:, -1]
            return m * dx / rho0

        def peak(r):
            hm = 0.0
            for v in surf(r)[2:nx - 2] - z0:
                hm = max(hm, float(v))
            return hm

        hsamp, t, nlog, tc = [H], 0.0, 100.0, case.t_end
        dt_last = None
        while t < tc:
            k = 1 if dt_last is None else max(1, int(0.9 * (nlog - t) / dt_last))
            t0 = t
            n, t = g.run(case.cfl, tc, k)
            if n == 0:
                break
            dt_last = (t - t0) / n
            if t >= nlog:
                hsamp.append(peak(g.read("r")))
                nlog += 100.0
        r = g.read("r")
        g.close()
        h = surf(r) - z0
        hmax, ratio = 0.0, 0.0
        for i in range(2, nx - 2):
            hmax = max(hmax, float(h[i]))
            if h[i] > 500.0:
                ratio = max(ratio, rho0 * gz * h[i] * abs(h[i + 1] - h[i - 1]) / (2 * dx) / tauy)
        ns = len(hsamp)
        early = hsamp[0] - hsamp[min(4, ns - 1)]
        late = hsamp[max(0, ns - 5)] - hsamp[ns - 1]
        res.append((hmax / H, early, late, ratio))
    ok_a = res[0][0] > 0.92
    ok_b = res[1][0] < 0.75 and res[1][2] < 0.15 * res[1][1] and res[1][3] < 8.0
    ok_c = res[2][2] > 3.0 * res[1][2] and res[2][0] < res[1][0]
    return ok_a and ok_b and ok_c, {"static": res[0], "arrest": res[1], "control": res[2]}


GATES = {"visc_diff": visc_diff, "visc_agree": visc_agree, "visc_energy": visc_energy, "vib_regen": vib_regen,
         "bingham_slope": bingham_slope}
