"""The reference's own drivers compile UNMODIFIED against the GPU library.

hydrocodes/sph/cpu_dump.cpp (cpu_dump.cpp:7-64) and cpu_bench.cpp
(cpu_bench.cpp:4-32) include "sph.hpp" and drive `System` directly.  With the
tests-only shim tests/refshim/sph.hpp (which includes the System facade,
include/deorbit_sph_system.hpp) first on the include path, each source file is
compiled byte for byte as it lies in the reference tree and linked against
libdeorbit_sph.so, so the drop-in claim (a reference driver rebuilds against
the GPU backend with no source change) is checked on the drivers themselves,
not on a look-alike.  The source is fed to the compiler on standard input from
an empty directory, so that `#include "sph.hpp"` cannot find the reference's
own header beside the driver.  Needs the reference checkout (DEORBIT_REFERENCE,
located through oracle/Makefile); skipped where it is absent."""
import os
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "deorbit_gb300", "_lib")


def compile_reference_driver(name, out_path, cwd):
    src = os.path.join(O.reference_dir(), "hydrocodes", "sph", name + ".cpp")
    if not os.path.exists(src):
        pytest.skip("reference checkout not present")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "tests", "refshim"),
           "-I", os.path.join(ROOT, "include"), "-x", "c++", "-", "-x", "none", "-o", out_path,
           "-L", LIBDIR, "-ldeorbit_sph", f"-Wl,-rpath,{LIBDIR}"]
    with open(src, "rb") as f:
        r = subprocess.run(cmd, stdin=f, capture_output=True, cwd=cwd)
    assert r.returncode == 0, (r.stdout + r.stderr).decode()
    return out_path


@pytest.mark.parametrize("name", ["cpu_dump", "cpu_bench"])
def test_reference_driver_builds_against_the_facade(cuda_lib, tmp_path, name):
    exe = compile_reference_driver(name, str(tmp_path / name), str(tmp_path))
    # the binary drives the GPU library, not the reference's header-only solver
    r = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True)
    syms = set(line.split()[-1] for line in r.stdout.splitlines() if line.strip())
    assert {"sph_create", "sph_init", "sph_step", "sph_impact_add_particles"} <= syms, sorted(syms)[:20]
