"""The campaign's grazing-impact IC generated in place (sph_impact_create_grazing)
equals the reference builder's file (boundary_daemon.build_grazing_ic) bit for
bit: same particle count, spacing, domain, and the SHA-256 of the N x 10 records
[x y z vx vy vz mass u mat fixed] -- fixtures made from the reference by
tests/golden/make_grazing_ic_golden.py.  The records are read back through a
lossless checkpoint, whose first ten columns are the IC layout."""
import hashlib
import json
import os

import numpy as np
import pytest

from deorbit_gb300 import ic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grazing_ic.json")


def cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


def test_fixture_is_consistent():
    for c in cases():
        assert c["n"] == c["n_impactor"] + (c["n"] - c["n_impactor"]) and c["n_impactor"] > 0
        assert len(c["header"]) == 7 and int(c["header"][6]) == c["n"]
        assert len(c["sample"]) == (c["n"] + c["sample_every"] - 1) // c["sample_every"]


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(3))
def test_generated_ic_equals_reference_file(cuda_lib, tmp_path, k):
    from deorbit_gb300 import sph
    c = cases()[k]
    ctx = sph.Context(sph.FP64)
    ctx.add_material(ic._material_struct(sph.Material, ic.basalt()))
    ctx.add_material(ic._material_struct(sph.Material, ic.iron()))
    prm = sph.params(eta=1.3, h_init=1.3 * c["dx"])
    b, dx, n = ctx.create_grazing(prm, c["theta_deg"], c["v"], cppr=c["cppr"], D=c["D"], tgt_mat=0, imp_mat=1,
                                  x_impact_frac=c["x_impact_frac"], start_h=c["start_h"])
    assert dx == c["dx"] and n == c["n"]
    path = str(tmp_path / "chk.bin")
    ctx.write_checkpoint(b, path, dx)
    ctx.close()
    raw = np.fromfile(path, dtype=np.float64)
    hdr, rec = raw[:9], raw[9:].reshape(n, 18)[:, :10]
    assert hdr[:6].tolist() == c["header"][:6] and int(hdr[6]) == n
    ref_sample = np.array(c["sample"])
    got_sample = rec[:: c["sample_every"]]
    assert np.array_equal(got_sample, ref_sample)
    assert hashlib.sha256(np.ascontiguousarray(rec).tobytes()).hexdigest() == c["records_sha256"]
