"""The gpu_ic command-line driver (deorbit_gb300/csrc/gpu_ic.cpp): the
reference's command line, progress line and snapshot files (gpu_ic.cpp:38-139),
with the CPU solver's physics.  CPU: usage and option handling.  GPU: the
snapshots of a --frac run equal the oracle's state at the same steps."""
import os
import re
import subprocess

import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O

from parity import rel_l2


def cli():
    from deorbit_gb300 import build as B
    B.build()
    return B.CLI


def test_usage_and_rejected_options():
    exe = cli()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage: gpu_ic" in r.stdout
    # the Metal driver's gravity / damping terms are not part of the solver
    r = subprocess.run([exe, "ic.bin", "10", "1", "--g", "3.7"], capture_output=True, text=True)
    assert r.returncode == 1 and "--g" in r.stdout
    r = subprocess.run([exe, "ic.bin", "10", "1", "--precision", "fp16"], capture_output=True, text=True)
    assert r.returncode == 1


def read_snapshot(path):
    raw = np.fromfile(path, dtype=np.float64)
    n = int(raw[:1].view(np.int64)[0])
    return raw[1:].reshape(n, 10)


@pytest.mark.gpu
def test_frac_run_matches_oracle(cuda_lib, oracle_lib, tmp_path):
    exe = cli()
    sc = ic.sheared_cube(L=10)   # basalt + iron, the --frac parameters and flaw seed
    icf = tmp_path / "ic.bin"
    ic.write_ic(sc, str(icf))
    t_end, snap = 0.05, 0.02
    r = subprocess.run([exe, str(icf), f"{sc.dx}", f"{t_end}", "--frac", "--precision", "fp64",
                        "--snap", f"{snap}"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout
    assert re.search(r"loaded .*: n=1000 \((\d+) iron\)", out)
    assert "init done, E0=" in out and "DONE: " in out
    melts = re.findall(r"melt=(\d+)%", out)
    assert melts, out
    nsteps = int(re.search(r"DONE: (\d+) steps", out).group(1))
    snaps = sorted(f for f in os.listdir(tmp_path) if f.startswith("gpu_snap_"))
    assert len(snaps) >= 2

    # the oracle with the driver's stepping: CFL dt, last step clipped at
    # t_end, a snapshot at the first step reaching each snapshot time
    orc = O.from_scenario(sc)
    orc.init()
    t, next_snap, want, steps = 0.0, snap, [], 0
    names = ["x", "y", "z", "vx", "vy", "vz", "u", "rho", "hh"]
    while t < t_end:
        dt = orc.timestep()
        if t + dt > t_end:
            dt = t_end - t
        orc.step(dt)
        t += dt
        steps += 1
        if t >= next_snap:
            want.append(np.stack([orc.field(k) for k in names], axis=1))
            next_snap += snap
    assert steps == nsteps
    assert len(want) == len(snaps)
    for s, w in zip(snaps, want):
        got = read_snapshot(tmp_path / s)
        assert np.array_equal(got[:, 9], sc.mat.astype(float))
        for c, k in enumerate(names):
            assert rel_l2(got[:, c], w[:, c]) < 1e-9, (s, k)


@pytest.mark.gpu
def test_mixed_run_and_restart(cuda_lib, tmp_path):
    """Default (mixed) form, a checkpoint, and a restart from it."""
    exe = cli()
    sc = ic.sheared_cube(L=8)
    icf = tmp_path / "ic.bin"
    ic.write_ic(sc, str(icf))
    r = subprocess.run([exe, str(icf), f"{sc.dx}", "0.03", "--frac", "--snap", "1", "--checkpoint", "0.01"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "gpu_chk.bin").exists()
    r2 = subprocess.run([exe, str(icf), f"{sc.dx}", "0.04", "--frac", "--restart", str(tmp_path / "gpu_chk.bin"),
                         "--snap", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r2.returncode == 0, r2.stdout + r2.stderr
    m = re.search(r"DONE: (\d+) steps to t=([0-9.]+)", r2.stdout)
    assert m and abs(float(m.group(2)) - 0.04) < 1e-9


@pytest.mark.gpu
def test_generated_grazing_ic_run(cuda_lib, tmp_path):
    """--grazing generates the campaign IC in place (no IC file) and runs it."""
    exe = cli()
    r = subprocess.run([exe, "-", "0", "1.0", "--grazing", "5,15000,1,4000", "--snap", "0.4"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "loaded grazing IC (generated): n=11527 (7 iron)" in r.stdout, r.stdout
    assert re.findall(r"melt=(\d+)%", r.stdout)
    snaps = sorted(f for f in os.listdir(tmp_path) if f.startswith("gpu_snap_"))
    assert snaps
    s = read_snapshot(tmp_path / snaps[-1])
    assert s.shape == (11527, 10) and set(np.unique(s[:, 9])) == {0.0, 1.0}
