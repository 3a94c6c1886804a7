"""Generate tests/golden/euler_modes.json from the REFERENCE's driver modes.

Runs the reference driver itself -- `main` of hydrocodes/euler/hydro_cpu.cpp,
compiled unmodified from the reference checkout by oracle/Makefile into
oracle/_ref/libeulerref.so and called as `eref_main` -- once per mode below,
each in its own child process (in parallel), and stores what each prints.
The modes are the reference's validation runs with no counterpart among the
other fixtures: cylindrical strength (lame), cylindrical fluidization
viscosity (af_visc), vibration advection (vib_advect), shock activation of
fluidization (af_activate), the fluidized step collapse (collapse), Pierazzo
et al. 2008's Al-on-Al benchmark (pierazzo2d) and Prater 1970's crater growth
(prater), all at their default arguments.  tests/euler_gates.py re-runs each
mode and formats its lines the same way: over the oracle the lines match
character for character, on the GPU number by number.

    python tests/golden/make_mode_golden.py
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import euler as EO  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "euler_modes.json")
MODES = ["lame", "af_visc", "vib_advect", "af_activate", "collapse", "pierazzo2d", "prater"]

CHILD = """
import ctypes as C, sys
lib = C.CDLL(sys.argv[1])
args = [b"hydro_cpu"] + [a.encode() for a in sys.argv[2:]]
argv = (C.c_char_p * len(args))(*args)
rc = lib.eref_main(len(args), argv)
C.CDLL(None).fflush(None)
sys.exit(rc)
"""


def run(mode):
    with tempfile.TemporaryDirectory() as tmp:  # the modes write their own data files into the working directory
        t0 = time.time()
        r = subprocess.run([sys.executable, "-c", CHILD, EO.REF_SO, mode], capture_output=True, text=True, cwd=tmp,
                           check=True)
        return mode, r.stdout.splitlines(), time.time() - t0


def main():
    if not EO.ref_available():
        O.build(ref=True)
    out = {}
    with cf.ThreadPoolExecutor(max_workers=len(MODES)) as ex:
        for mode, lines, el in ex.map(run, MODES):
            out[mode] = {"lines": lines, "reference_seconds": round(el, 1)}
            print(mode, f"{el:.1f} s", lines[-1])
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
