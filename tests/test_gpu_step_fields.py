"""sph_step_fields: one call that writes host fields, steps and reads fields
back, with the host copies overlapping the step's kernels.  Checked bit for
bit against the separate calls it stands for (sph_write_fields, sph_timestep,
sph_step, sph_read_fields) on two contexts built from the same initial state.
The host state is edited between steps, so every written field matters: u, D
and S reach the device only just before the EOS pass and x, y, z and hh are
read back while the force pass runs, so a late write that went missing or a
read taken before its field was final would show as a difference."""
import numpy as np
import pytest

from deorbit_gb300 import ic

pytestmark = pytest.mark.gpu

CARRIED = ["x", "y", "z", "vx", "vy", "vz", "u", "hh", "D", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"]
OUTS = CARRIED + ["rho", "P", "mass", "csig"]


@pytest.fixture(scope="module")
def sph_mod(cuda_lib):
    from deorbit_gb300 import sph
    return sph


def _contexts(sph, precision, scenarios):
    out = []
    for _ in range(2):
        ctx = sph.Context(precision, device=0)
        bs = [ic.to_context(ctx, sc) for sc in scenarios]
        ctx.init()
        out.append((ctx, bs))
    return out


def _edit(state, k):
    """Deterministic host-side changes between steps."""
    s = dict(state)
    s["u"] = state["u"] * (1.0 + 1e-3 * (k + 1))
    s["D"] = np.minimum(state["D"] + 0.01, 1.0)
    s["Sxx"] = state["Sxx"] + 1.0e5
    s["Syz"] = state["Syz"] * 0.99
    s["vx"] = state["vx"] + 0.5
    s["hh"] = state["hh"] * (1.0 + 1e-4)
    return s


def _pinned(n):
    import torch
    return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("precision,graphs", [(0, 1), (1, 1), (1, 0)], ids=["fp64", "mixed", "mixed_uncaptured"])
def test_step_fields_equals_separate_calls(sph_mod, precision, graphs):
    """graphs = 1: the fused step replays its two captured halves; 0: the
    same kernels launched one by one."""
    sph = sph_mod
    prec = sph.FP64 if precision == 0 else sph.MIXED
    (A, (a,)), (B, (b,)) = _contexts(sph, prec, [ic.grazing(n_total=16384, gap=0.25)])
    B.set_option("graphs", graphs)
    n = A.n(a)
    state = A.read_many(a, CARRIED)
    ins = {k: _pinned(n) for k in CARRIED}
    outs = [_pinned(n) for _ in OUTS]
    for k in range(4):
        edited = _edit(state, k)
        A.write_many(a, edited)
        dt_a = A.timestep(a)
        A.step(dt_a)
        got_a = A.read_many(a, OUTS)
        for name in CARRIED:
            ins[name][:] = edited[name]
        dt_b, got_b = B.step_fields(b, ins, OUTS, outs)
        assert dt_b == dt_a
        for name in OUTS:
            assert np.array_equal(got_a[name], got_b[name]), (k, name)
        state = {name: got_a[name].copy() for name in CARRIED}
    assert A.info(a).steps == B.info(b).steps and A.info(a).t == B.info(b).t
    A.close()
    B.close()


def test_step_fields_partial_sets_two_impacts(sph_mod):
    """Only late inputs, only early outputs, an explicit dt, and a second
    impact that steps along: both impacts' whole state stays equal."""
    sph = sph_mod
    scen = [ic.grazing(n_total=12000, gap=0.25), ic.impact_halfspace(nx=14, ny=14, nz=7, r_cells=2.0)]
    (A, (a0, a1)), (B, (b0, b1)) = _contexts(sph, sph.MIXED, scen)
    n = A.n(a0)
    for k in range(3):
        u = A.read(a0, "u") * (1.0 + 2e-3)
        sxy = A.read(a0, "Sxy") + 3.0e4
        dt = 0.5 * A.timestep(a0)
        A.write_many(a0, {"u": u, "Sxy": sxy})
        A.step(dt)
        got_a = A.read_many(a0, ["x", "hh", "z"])
        dt_b, got_b = B.step_fields(b0, {"u": u, "Sxy": sxy}, ["x", "hh", "z"], dt=dt)
        assert dt_b == dt
        for name in ("x", "hh", "z"):
            assert np.array_equal(got_a[name], got_b[name]), (k, name)
    for (ca, ia), (cb, ib) in (((A, a0), (B, b0)), ((A, a1), (B, b1))):
        fa = ca.read_many(ia, OUTS)
        fb = cb.read_many(ib, OUTS)
        for name in OUTS:
            assert np.array_equal(fa[name], fb[name]), name
    assert n == B.n(b0)
    A.close()
    B.close()


def test_step_fields_rejects_bad_arguments(sph_mod):
    sph = sph_mod
    ctx = sph.Context(sph.FP64, device=0)
    b = ic.to_context(ctx, ic.impact_halfspace(nx=10, ny=10, nz=5, r_cells=2.0))
    ctx.init()
    x = ctx.read(b, "x")
    with pytest.raises(sph.SphError):
        ctx.step_fields(b, {"nope": x}, ["x"])
    with pytest.raises(sph.SphError):
        ctx.step_fields(b, {"x": x}, ["nope"])
    with pytest.raises(sph.SphError):
        ctx.step_fields(b, {"x": x}, ["x"], dt=float("inf"))
    steps0 = ctx.info(b).steps
    ctx.step_fields(b, {"x": x}, ["x"])  # the context still steps after the refusals
    assert ctx.info(b).steps == steps0 + 1
    ctx.close()
