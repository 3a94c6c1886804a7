"""The reference driver's validation modes lame, af_visc, vib_advect,
af_activate and collapse (hydrocodes/euler/hydro_cpu.cpp:490-539, 860-900)
over the oracle: every line the mode prints matches what the reference's
compiled driver printed (tests/golden/euler_modes.json) character for
character, pass / fail verdict included.  pierazzo2d and prater (10^3-10^4
steps of 10^4 cells) run on the GPU only (tests/test_gpu_euler_modes.py)."""
import json
import os

import pytest

import euler_gates as EG
import visc_gates as VG

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "euler_modes.json")))


@pytest.mark.parametrize("mode", EG.ORACLE_MODES)
def test_oracle_mode_prints_what_the_reference_prints(mode):
    ok, lines = EG.MODES[mode](VG.OracleGrid)
    assert lines == GOLD[mode]["lines"]
    assert ok == lines[-1].endswith("PASS")
