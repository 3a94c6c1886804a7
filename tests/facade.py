"""Build helper for the C++ System-facade driver (tests/facade_driver.cpp)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "deorbit_gb300", "_lib")


def compile_driver(out_path, link=True):
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "facade_driver.cpp")]
    if link:
        cmd += ["-o", out_path, "-L", LIBDIR, "-ldeorbit_sph", f"-Wl,-rpath,{LIBDIR}"]
    else:
        cmd += ["-fsyntax-only"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out_path
