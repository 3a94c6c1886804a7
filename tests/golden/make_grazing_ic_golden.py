"""Golden ICs of the campaign's grazing-impact builder, from the REFERENCE.

Calls the reference's own `build_grazing_ic` (src/deorbit/impact/boundary_daemon.py,
imported from the reference checkout, DEORBIT_REFERENCE) on small configurations and stores, per case, the
arguments, the returned (dx, N), the 7-double header and the SHA-256 of the particle
records (N x 10 float64, the file's body), plus every 97th record.  Needs the reference
tree; the fixture it writes (grazing_ic.json) is committed so the tests never need it.

    python tests/golden/make_grazing_ic_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (theta_deg, v, cppr, D, x_impact_frac, start_h): small lattices (the slab is at least
# 20 x 4 x 6 km, so resolution comes from a coarse dx = D / (2 cppr))
CASES = [
    (5.0, 15000.0, 1, 4000.0, None, None),
    (30.0, 20000.0, 2, 8000.0, None, None),
    (45.0, 12000.0, 1, 6000.0, 0.5, 3000.0),
]


def main():
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), ""))
    from oracle import oracle as O

    sys.path.insert(0, os.path.join(O.reference_dir(), "src"))
    from deorbit.impact import boundary_daemon as bd  # the reference builder

    out = {"source": "boundary_daemon.build_grazing_ic (reference)", "sph": {k: bd.SPH[k] for k in
           ("rho_imp", "imp_mat", "tgt_mat")}, "cases": []}
    with tempfile.TemporaryDirectory() as tmp:
        for theta, v, cppr, D, xf, sh in CASES:
            path = os.path.join(tmp, "ic.bin")
            dx, n = bd.build_grazing_ic(theta, v, path, cppr=cppr, D=D, x_impact_frac=xf, start_h=sh)
            raw = np.fromfile(path, dtype=np.float64)
            hdr, rec = raw[:7], raw[7:].reshape(-1, 10)
            assert rec.shape[0] == n
            out["cases"].append({
                "theta_deg": theta, "v": v, "cppr": cppr, "D": D, "x_impact_frac": xf, "start_h": sh,
                "dx": dx, "n": int(n), "header": hdr.tolist(),
                "records_sha256": hashlib.sha256(rec.tobytes()).hexdigest(),
                "sample_every": 97, "sample": rec[::97].tolist(),
                "n_fixed": int(rec[:, 9].sum()), "n_impactor": int((rec[:, 8] == bd.SPH["imp_mat"]).sum()),
            })
    with open(os.path.join(HERE, "grazing_ic.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", os.path.join(HERE, "grazing_ic.json"), [c["n"] for c in out["cases"]])


if __name__ == "__main__":
    main()
