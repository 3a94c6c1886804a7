"""The crater driver (deorbit_gb300.crater: the reference's `crater` mode,
hydrocodes/euler/hydro_cpu.cpp:557-680) over the oracle against the
reference's own crater mode (tests/golden/crater_modes.json, made by running
the reference's compiled driver): every printed line and the profile file are
reproduced character for character."""
import json
import os

import pytest

from deorbit_gb300 import crater
from oracle import euler as EO

GOLD = os.path.join(os.path.dirname(__file__), "golden", "crater_modes.json")
MODES = json.load(open(GOLD))


@pytest.mark.parametrize("mode", MODES, ids=lambda m: "_".join(m["args"][:7]))
def test_oracle_driver_reproduces_reference_mode(mode, tmp_path):
    st, _ = crater.setup_from_args(mode["args"], env={})
    res = crater.run(st, make_grid=lambda c: EO.DrivenGrid(c))
    assert res["lines"] == mode["lines"]
    prof = tmp_path / "profile.txt"
    crater.write_profile(str(prof), st, res)
    assert prof.read_text() == mode["profile"]


def test_arguments_read_as_the_reference_reads_them():
    st, prof = crater.setup_from_args(["400", "9000", "2.0", "1e9", "1.62", "4", "-1", "20", "15", "out.txt", "0",
                                       "3e6", "0.27", "2e7", "1", "1", "0.3", "2.0"], env={"AF_CACT": "0.1"})
    p = st.case.params
    assert prof == "out.txt" and st.a == 400.0 and st.U == 9000.0 and st.gz == 1.62 and not st.fixed
    assert st.case.dx == 100.0 and st.case.shape == (80, 1, 60)
    assert p["rock"] == 0 and p["y_d0"] == 3e6 and p["void_amb"] == 0.27 and p["y_bingham"] == 2e7
    assert p["visc_imp"] == 1 and p["void_cons"] == 1 and p["c_reg"] == 0.3 and p["af_reg"] == 1
    assert p["af_sat"] == 2.0 and p["c_act"] == 0.1 and p["p_act"] == 1e8 and p["tdec"] == 2.0
    assert st.case.pin_floor == 2 and st.case.sponge_from == int(0.85 * 80)
    # defaults: the reference's crater with no arguments
    st, prof = crater.setup_from_args([], env={})
    assert (st.a, st.U, st.tdec, st.gz) == (500.0, 12000.0, 0.0, 3.71) and prof == "crater_profile.txt"
    assert st.case.shape == (150, 1, 110) and st.case.params["c_act"] == 0.0
    # a negative C_REG keeps the regeneration bookkeeping off
    st, _ = crater.setup_from_args(["500", "12000", "0", "0", "3.71", "2", "-1", "8", "8", "p", "1", "0", "0", "0",
                                    "0", "0", "-1"], env={})
    assert st.case.params["af_reg"] == 0 and st.case.params["c_reg"] == 0.0


def test_settling_windows():
    """hydro_cpu.cpp:659-664: window means of the floor depth over 2 t_auto;
    settled when two consecutive means agree to 2 % of the newer one.  The
    first window only opens the comparison; a window closes at its first
    sample at least a window after its start, and the next window starts at
    that sample's time."""
    st = crater.Settling(window=10.0)
    # first window: samples at t = 0..10 of depth 100 -> mean 100, no verdict
    assert not any(st.sample(t, 100.0) for t in range(0, 11))
    assert st.prev == 100.0 and st.count == 0 and st.start == 10
    # second window: t = 11..20 (closes at 20 - 10 >= 10), mean 103 -- 3 % apart, not settled
    assert not any(st.sample(t, 103.0) for t in range(11, 21))
    assert st.prev == 103.0 and st.start == 20
    # third window: mean 104 -- |104 - 103| < 0.02 * 104, settled when it closes at t = 30
    assert not any(st.sample(t, 104.0) for t in range(21, 30))
    assert st.sample(30, 104.0)
