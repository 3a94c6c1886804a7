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
    with tempfile.TemporaryDirectory() as tmp:
        for args in MODES:
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
