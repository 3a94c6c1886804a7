"""The reference driver's crater mode on the GPU grid solver.

`hydrocodes/euler/hydro_cpu.cpp:557-680` (mode `crater`): a basalt sphere of
radius a on the axis of a cylindrical (r, z) domain, tangent to the free
surface of a lithostatic basalt half-space under gravity, moving down at U;
the pre-impact column frozen as the well-balanced reference; ROCK yield,
near-void and vacuum-aware faces, optionally shock-activated acoustic
fluidization (TDEC > 0) with the crater defaults (acoustic seeding,
overburden relief), and every later option of the mode's command line
(argument order of the reference, below).  The loop takes CFL 0.4 steps with
the far-field floor pinned and the outer 15 % of the radius relaxed toward the
reference after every step, both on the device; it runs to a fixed time or,
by default, until two consecutive window means of the bowl-floor depth agree
to 2 % (at most 6 gravity timescales), and measures the crater from the
column-mass deficit against the reference: apparent diameter and depth, the
transient depth (deepest floor sampled every 20 steps), rim uplift, d/D.

    from deorbit_gb300 import crater
    res = crater.run(crater.setup(a=500.0, U=12000.0))
    print(res["result_line"])        # "RESULT a D_app depth transient d/D"

The loop and the measurements are the reference's, and so are the lines it
prints at the end (`lines`; the RESULT line last).  Its progress line goes to
an optional callback; its field snapshots, Lagrangian tracers and void-reset
instrumentation counters are not reproduced.  `run` takes any grid factory
with the deorbit_gb300.euler.Grid interface (the mixed form, or a CPU grid for
comparison).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import grid_ic as GI


@dataclass
class Setup:
    case: GI.Case
    a: float
    U: float
    tdec: float
    eta_af: float
    gz: float
    tend: float
    t_auto: float
    fixed: bool
    rho0: float


def setup(a=500.0, U=12000.0, tdec=0.0, eta_af=0.0, gz=3.71, cppr=5.0, tend=-1.0, Rfac=30.0, Zfac=22.0,
          rock=1, y_d0=None, void_amb=None, y_bingham=None, visc_imp=None, void_cons=None, c_reg=None,
          af_sat=None, c_act=None, legacy_seed=False, legacy_afcut=False) -> Setup:
    """The mode's arguments in its order (hydro_cpu.cpp:560-580): impactor
    radius a (m), speed U (m/s), TDEC, ETA_AF, gravity, cells per radius,
    end time (<= 0: run to settling), domain radius and height in impactor
    radii, ROCK, Y_D0, VOID_AMB, Y_BINGHAM, VISC_IMP, VOID_CONS, C_REG (>= 0
    also enables the regeneration bookkeeping), AF_SAT; c_act, legacy_seed and
    legacy_afcut stand for the AF_CACT, AF_LEGACY_SEED and AF_LEGACY_AFCUT
    environment overrides."""
    case = GI.crater(cppr=cppr, Rfac=Rfac, Zfac=Zfac, a=a, U=U, gz=gz)
    p = case.params
    p.update(rock=int(rock), af_seeddp=0 if legacy_seed else 1, af_prel=0 if legacy_afcut else 1, p_coh=1.0e6)
    if tdec > 0:
        p.update(tdec=float(tdec), eta_af=float(eta_af), c_act=0.5 if c_act is None else float(c_act), p_act=1.0e8)
    else:
        p.update(tdec=0.0, eta_af=float(eta_af), c_act=0.0, p_act=0.0)
    if c_reg is not None:
        p.update(c_reg=max(float(c_reg), 0.0), af_reg=int(c_reg >= 0))
    if af_sat is not None:
        p["af_sat"] = float(af_sat)
    for k, v in (("y_d0", y_d0), ("void_amb", void_amb), ("y_bingham", y_bingham)):
        if v is not None:
            p[k] = float(v)
    for k, v in (("visc_imp", visc_imp), ("void_cons", void_cons)):
        if v is not None:
            p[k] = int(bool(v))
    nr = case.shape[0]
    case.pin_floor = 2
    case.sponge_from = int(0.85 * nr)
    t_auto = 2.0 * math.sqrt((Rfac * a) / gz)
    fixed = tend > 0
    case.t_end = tend if fixed else 6.0 * t_auto
    case.name = f"crater_a{a:.0f}_U{U:.0f}"
    return Setup(case, a, U, tdec, eta_af, gz, case.t_end, t_auto, fixed, case.material["rho0"])


class _Metrics:
    """The mode's column-mass measurements (hydro_cpu.cpp:598-603, 654-660)."""

    def __init__(self, st: Setup, ref_r0):
        nx, _, nz = st.case.shape
        self.nr, self.nz, self.dx, self.rho0 = nx, nz, st.case.dx, st.rho0
        self.ref = np.asarray(ref_r0, dtype=np.float64).reshape(nx, nz)

    def dcol(self, r):
        """Per column: the mass deficit against the reference over rho0 (m),
        summed over z in cell order."""
        m = np.cumsum(self.ref - np.asarray(r).reshape(self.nr, self.nz), axis=1)[:, -1]
        return m * self.dx / self.rho0

    def dfloor(self, r):
        d = self.dcol(r)
        return max(0.0, float(d.max()))

    def vexc(self, r):
        d = self.dcol(r)
        w = np.where(d > 0, d * (np.arange(self.nr) + 0.5), 0.0)
        return float(np.cumsum(w)[-1])


class Settling:
    """The run-to-settling test (hydro_cpu.cpp:659-664): bowl-floor depths
    sampled every 5 steps after t_auto are averaged over windows of 2 t_auto
    (a window closes at the first sample at least that long after its first);
    the run has settled when a window's mean agrees with the previous
    window's to tol (relative to the newer mean)."""

    def __init__(self, window, tol=0.02):
        self.window, self.tol = window, tol
        self.sum, self.count, self.start, self.prev = 0.0, 0, -1.0, -1.0

    def sample(self, t, depth) -> bool:
        if self.start < 0:
            self.start = t
        self.sum += depth
        self.count += 1
        if t - self.start >= self.window:
            mean = self.sum / self.count
            if self.prev > 0 and abs(mean - self.prev) < self.tol * mean:
                return True
            self.prev, self.sum, self.count, self.start = mean, 0.0, 0, t
        return False


def _next_event(n, settling):
    """The step count after step n at which the loop next samples the floor
    (steps 1, 21, 41, ...: the reference samples before counting the step) or,
    while the settling test is on, may test settling (multiples of 5).  The
    log is checked there too, so a progress line can come a few steps after
    its 20 s mark."""
    a = n + 1
    while not (a % 20 == 1 or (settling and a % 5 == 0)):
        a += 1
    return a


def run(st: Setup, make_grid=None, form=0, device=0, log=None) -> dict:
    """Run the crater mode; `make_grid(case)` builds the grid (default: the
    CUDA solver in `form` on `device`).  `log(line)` receives a progress line
    every 20 s of simulated time after the first gravity timescale.  Returns
    the crater measures, the run's state and the mode's printed lines."""
    from . import euler as E

    case = st.case
    if make_grid is None:
        def make_grid(c):
            return E.from_case(c, device=device, form=form)
    g = make_grid(case)
    g.set_driver(case.pin_floor, case.sponge_from)
    ref_r0, _ = g.reference()
    M = _Metrics(st, ref_r0)
    settle = Settling(2.0 * st.t_auto)
    dmax_t, t, s = 0.0, 0.0, 0
    t_settled, next_log = -1.0, st.t_auto
    dt_last = 0.0
    while t < st.tend:
        # stop every 5 steps once t may pass t_auto within the next 20 steps
        settling = not st.fixed and (t > st.t_auto or dt_last <= 0 or t + 25 * dt_last > st.t_auto)
        want = _next_event(s, settling) - s
        t_prev = t
        k, t = g.run(case.cfl, st.tend, want)
        s += k
        if k:
            dt_last = (t - t_prev) / k
        if k < want:  # t reached the end before the next sampling step
            break
        r = None
        if (s - 1) % 20 == 0:  # the floor sample after the step taken at s % 20 == 0 (hydro_cpu.cpp:638)
            r = g.read("r")
            dmax_t = max(dmax_t, M.dfloor(r))
        if log is not None and t >= next_log:
            r = g.read("r") if r is None else r
            log(_progress(st, g, M, r, t, s))
            next_log += 20.0
        if not st.fixed and t > st.t_auto and s % 5 == 0:  # run-to-settling test (hydro_cpu.cpp:659-664)
            r = g.read("r") if r is None else r
            if settle.sample(t, M.dfloor(r)):
                t_settled = t
                break
    f = {k: g.read(k) for k in ("r", "mu", "mv", "mw")}
    P = g.pressure()
    out = _measure(st, M, f, P)
    out.update(steps=int(s), t=float(t), settled=t_settled > 0, t_settled=float(t_settled),
               transient_depth=dmax_t)
    out["lines"] = _lines(st, out)
    out["result_line"] = out["lines"][-1]
    out["profile"] = np.stack([(np.arange(M.nr) + 0.5) * M.dx, -M.dcol(f["r"])], axis=1)
    if hasattr(g, "close"):
        g.close()
    return out


def run_many(setups, form=0, device=0, workers=None, make_grid=None):
    """Several crater runs at once (a parameter sweep, as the reference's
    campaign scripts run the mode over impactor sizes and speeds): one grid,
    CUDA stream and host thread per run, so the small grids' kernels overlap
    on the device.  Returns the results in the order of `setups`; each equals
    the same run made alone (the runs share nothing)."""
    import concurrent.futures as cf

    setups = list(setups)
    n = workers or min(len(setups), 16)
    with cf.ThreadPoolExecutor(max_workers=max(1, n)) as ex:
        futs = [ex.submit(run, st, make_grid, form, device) for st in setups]
        return [f.result() for f in futs]


def _measure(st, M, f, P):
    """Final geometry (hydro_cpu.cpp:666-674)."""
    r = f["r"]
    dense = r > 1350.0
    v = np.sqrt(f["mu"] * f["mu"] + f["mv"] * f["mv"] + f["mw"] * f["mw"]) / r
    vmx = float(v[dense].max()) if dense.any() else 0.0
    pmx = float(P[dense].max()) if dense.any() else 0.0
    d = M.dcol(r)
    dapp, ifloor = 0.0, 0
    for i in range(M.nr):
        if d[i] > dapp:
            dapp, ifloor = float(d[i]), i
    i_d = M.nr - 1
    for i in range(ifloor, M.nr):
        if d[i] <= 0.25 * M.dx:
            i_d = i
            break
    r_d = (i_d + 0.5) * M.dx
    d_app = 2.0 * r_d
    zrim, rrim = 0.0, 0.0
    for i in range(M.nr):
        u = -float(d[i])
        if u > zrim:
            zrim, rrim = u, (i + 0.5) * M.dx
    return {"D_app": d_app, "depth": dapp, "d_over_D": dapp / d_app if d_app > 0 else 0.0, "rim_uplift": zrim,
            "rim_r": rrim, "max_v": vmx, "max_p": pmx,
            "finite": bool(np.isfinite(vmx) and np.isfinite(pmx) and np.isfinite(dapp))}


def _progress(st, g, M, r, t, s):
    dense = r > 1350.0
    mu, mv, mw = g.read("mu"), g.read("mv"), g.read("mw")
    v = np.sqrt(mu * mu + mv * mv + mw * mw) / r
    af, D = g.read("af"), g.read("D")
    n = int(dense.sum())
    amean = float(af[dense].sum() / n) if n else 0.0
    amax = float(af[dense].max()) if n else 0.0
    dmean = float(D[dense].sum() / n) if n else 0.0
    dfrac = float((D[dense] > 0.95).sum() / n) if n else 0.0
    return (f"  [crater a={st.a:.0f}] t={t:.1f}/{st.tend:.0f}s steps={s} max|v|={float(v[dense].max()) if n else 0.0:.2f} "
            f"Vexc={M.vexc(r):.4e} depth={M.dfloor(r) / 1e3:.2f}km af={amean:.3f}/{amax:.3f} "
            f"D(mean,frac>.95)={dmean:.3f},{dfrac:.2f}")


def _lines(st, o):
    c = st.case
    nr, _, nz = c.shape
    zsurf = nz * c.dx - 5.0 * st.a
    vi = " IMPLICIT" if c.params.get("visc_imp") else ""
    state = "SETTLED" if o["settled"] else ("FIXED-RUN" if st.fixed else "NOT-SETTLED@cap")
    return [
        f"CRATER a={st.a:.0f}m U={st.U:.0f} g={st.gz:.2f} TDEC={st.tdec:.3g} ETA={st.eta_af:.3g}{vi} | grid {nr}x{nz} "
        f"dx={c.dx:.0f} zsurf={zsurf / 1e3:.1f}km tend={st.tend:.1f}s steps={o['steps']}",
        f"  settling: {state} at t={o['t_settled'] if o['settled'] else o['t']:.1f}s (t_auto={st.t_auto:.1f}s "
        f"cap={st.tend:.1f}s tolM=2.0% Wwin={2.0 * st.t_auto:.1f}s final max|v|={o['max_v']:.1f} m/s)",
        f"  D_app={o['D_app'] / 1e3:.2f} km  depth(below datum)={o['depth'] / 1e3:.2f} km  transient depth="
        f"{o['transient_depth'] / 1e3:.2f} km  rim uplift={o['rim_uplift'] / 1e3:.2f} km @ r={o['rim_r'] / 1e3:.2f} km  "
        f"d/D={o['d_over_D']:.3f}  (column-mass metric)",
        f"  stability: max|v|={o['max_v']:.1f} m/s  maxP={o['max_p']:.2e} Pa  "
        f"{'FINITE' if o['finite'] else 'NONFINITE-BLOWUP'}",
        f"RESULT {st.a:.1f} {o['D_app']:.4f} {o['depth']:.4f} {o['transient_depth']:.4f} {o['d_over_D']:.4f}",
    ]


def setup_from_args(args, env=None):
    """setup() from the mode's command line after the mode name, read as the
    reference reads it (hydro_cpu.cpp:560-580): a U TDEC ETA_AF g cppr tend
    Rfac Zfac profile ROCK Y_D0 VOID_AMB Y_BINGHAM VISC_IMP VOID_CONS C_REG
    AF_SAT, each optional from the right; the environment's AF_CACT,
    AF_LEGACY_SEED and AF_LEGACY_AFCUT as there.  Returns (setup, profile
    path)."""
    import os

    env = os.environ if env is None else env

    def arg(i, default, conv=float):
        return conv(args[i]) if len(args) > i else default

    tdec = arg(2, 0.0)
    kw = dict(a=arg(0, 500.0), U=arg(1, 12000.0), tdec=tdec, eta_af=arg(3, 0.0), gz=arg(4, 3.71), cppr=arg(5, 5.0),
              tend=arg(6, -1.0), Rfac=arg(7, 30.0), Zfac=arg(8, 22.0), rock=arg(10, 1, int))
    for i, name, conv in ((11, "y_d0", float), (12, "void_amb", float), (13, "y_bingham", float),
                          (14, "visc_imp", int), (15, "void_cons", int), (16, "c_reg", float), (17, "af_sat", float)):
        if len(args) > i:
            kw[name] = conv(args[i])
    if env.get("AF_CACT") and tdec > 0:
        kw["c_act"] = float(env["AF_CACT"])
    kw["legacy_seed"] = bool(env.get("AF_LEGACY_SEED"))
    kw["legacy_afcut"] = bool(env.get("AF_LEGACY_AFCUT"))
    return setup(**kw), (args[9] if len(args) > 9 else "crater_profile.txt")


def write_profile(path, st: Setup, res):
    """The final surface profile in the reference's file format
    (hydro_cpu.cpp:676-678)."""
    c = st.case
    zsurf = c.shape[2] * c.dx - 5.0 * st.a
    vi = " IMP" if c.params.get("visc_imp") else ""
    with open(path, "w") as f:
        f.write(f"# r_m  -dcol_m (column-mass surface vs datum)   (a={st.a:.0f} U={st.U:.0f} g={st.gz:.2f} "
                f"TDEC={st.tdec:.3g} ETA={st.eta_af:.3g}{vi} dx={c.dx:.0f} zsurf={zsurf:.1f})\n")
        for r, d in res["profile"]:
            f.write(f"{r:.1f} {d:.3f}\n")


def main(argv=None):
    """`python -m deorbit_gb300.crater [a U TDEC ETA_AF g cppr tend Rfac Zfac
    profile ROCK ...]`: the reference's `crater` mode on the GPU; prints its
    lines, writes its profile file.  --mixed runs the mixed form, --log the
    progress lines (stderr)."""
    import sys

    argv = sys.argv[1:] if argv is None else list(argv)
    if "-h" in argv or "--help" in argv:
        print("usage: python -m deorbit_gb300.crater [--mixed] [--log] [a U TDEC ETA_AF g cppr tend Rfac Zfac "
              "profile ROCK Y_D0 VOID_AMB Y_BINGHAM VISC_IMP VOID_CONS C_REG AF_SAT]\n"
              "The reference driver's crater mode (hydro_cpu.cpp crater) on the GPU; defaults as there.")
        return 0
    form = 1 if "--mixed" in argv else 0
    log = (lambda line: print(line, file=sys.stderr, flush=True)) if "--log" in argv else None
    args = [a for a in argv if a not in ("--mixed", "--log")]
    st, prof = setup_from_args(args)
    res = run(st, form=form, log=log)
    for line in res["lines"]:
        print(line, flush=True)
    write_profile(prof, st, res)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
