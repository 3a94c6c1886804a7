"""Generate tests/golden/crater_modes.json from the REFERENCE's crater mode.

Runs the reference driver itself -- `main` of hydrocodes/euler/hydro_cpu.cpp,
compiled unmodified from the reference checkout by oracle/Makefile into
oracle/_ref/libeulerref.so and called as `eref_main` -- in a child process
for each command line below (small grids, fixed end times: a few hundred to a
thousand steps), and stores what it prints (its final lines; the void-reset
instrumentation line is left out) and the profile file it writes.  The tests
reproduce both with the crater driver (deorbit_gb300.crater) over the oracle
exactly, and with the CUDA solver to the solver's tolerance.

    python tests/golden/make_crater_golden.py
    python tests/golden/make_crater_golden.py --default   # also crater_default.json (~3 h)

--default also runs the mode with no arguments (its default crater: a = 500 m,
12 km/s, 150 x 110 cells, to the 763 s cap, 3 x 10^5 steps) into
tests/golden/crater_default.json.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import euler as EO  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "crater_modes.json")
OUT_DEFAULT = os.path.join(HERE, "crater_default.json")

# the mode's arguments after "crater" (profile path inserted at position 10)
MODES = [
    ["500", "6000", "0", "0", "3.71", "3", "3.0", "8", "8"],
    ["500", "6000", "2.0", "1e8", "3.71", "3", "3.0", "8", "8"],
    ["500", "6000", "2.0", "1e9", "3.71", "3", "2.0", "8", "8", "P", "1", "5e6", "0.27", "1e7", "1", "0", "0.5", "1.0"],
    ["500", "6000", "0", "0", "3.71", "3", "2.0", "8", "8", "P", "1", "0", "0", "0", "0", "1"],
    ["300", "9000", "0", "0", "9.81", "4", "1.5", "6", "6", "P", "0"],
]

CHILD = """
import ctypes as C, sys
lib = C.CDLL(sys.argv[1])
args = [b"hydro_cpu", b"crater"] + [a.encode() for a in sys.argv[2:]]
argv = (C.c_char_p * len(args))(*args)
rc = lib.eref_main(len(args), argv)
C.CDLL(None).fflush(None)
sys.exit(rc)
"""


def main():
    if not EO.ref_available():
        O.build(ref=True)
    out = []
    modes = list(MODES) + ([None] if "--default" in sys.argv else [])
    with tempfile.TemporaryDirectory() as tmp:
        for args in modes:
            if args is None:  # the default crater: profile path only (argument 11 needs 2-10 given)
                import time
                prof = os.path.join(tmp, "profile.txt")
                full = ["500", "12000", "0", "0", "3.71", "5", "-1", "30", "22", prof]
                t0 = time.time()
                r = subprocess.run([sys.executable, "-c", CHILD, EO.REF_SO] + full, capture_output=True, text=True,
                                   cwd=tmp, check=True)
                lines = [ln for ln in r.stdout.splitlines() if not ln.lstrip().startswith("voidzero:")]
                with open(prof) as f:
                    d = {"args": [], "lines": lines, "profile": f.read(), "reference_seconds": round(time.time() - t0)}
                with open(OUT_DEFAULT, "w") as f:
                    json.dump(d, f, indent=1)
                print(lines[-1])
                continue
            prof = os.path.join(tmp, "profile.txt")
            full = list(args[:9]) + [prof] + list(args[10:])
            r = subprocess.run([sys.executable, "-c", CHILD, EO.REF_SO] + full, capture_output=True, text=True,
                               cwd=tmp, check=True)
            lines = [ln for ln in r.stdout.splitlines() if not ln.lstrip().startswith("voidzero:")]
            with open(prof) as f:
                profile = f.read()
            out.append({"args": args, "lines": lines, "profile": profile})
            print(lines[-1])
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
