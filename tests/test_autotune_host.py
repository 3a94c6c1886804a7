"""Host logic of the autotuner (deorbit_gb300/autotune.py) on the CPU: workload
classes, the shipped GB300 table, and how a configuration reaches a context's
options -- with a stand-in context that records the calls."""
import json
import types

import pytest

from deorbit_gb300 import autotune, sph

OPTIONS = {"list_mode", "slack", "cell_factor", "cell_factor_z", "block"}


class RecordingContext:
    def __init__(self):
        self.tuning = None
        self.options = {}

    def set_tuning(self, block, cell_factor):
        self.tuning = (block, cell_factor)

    def set_option(self, key, value):
        self.options[key] = value


def scenario(n, strength=True):
    return types.SimpleNamespace(n=n, params={"damage_on": int(strength)},
                                 materials=[{"G": 2.4e10 if strength else 0.0}])


def test_workload_classes():
    assert autotune.workload_class(scenario(1 << 20)) == "s1_n2^20"
    assert autotune.workload_class(scenario(1 << 24, strength=False)) == "s0_n2^24"
    assert autotune.workload_class(scenario(3000), per_impact_n=30000) == "s1_n2^15"


def test_shipped_table_is_complete():
    with open(autotune.SHIPPED) as f:
        table = json.load(f)
    want = {"NVIDIA GB300|p1|s1_n2^20", "NVIDIA GB300|p0|s1_n2^20", "NVIDIA GB300|p1|s1_n2^15",
            "NVIDIA GB300|p1|s1_n2^24"}
    assert want <= set(table)
    for k in want:
        best = table[k]["best"]
        assert set(best) <= OPTIONS and {"list_mode", "cell_factor", "block"} <= set(best), k
        # the best entry is the fastest row of its own measured table
        rows = [r for r in table[k]["table"] if isinstance(r.get("ms_per_step"), float)]
        fastest = min(rows, key=lambda r: r["ms_per_step"])
        assert all(fastest.get(o) == best.get(o) for o in best), k


@pytest.mark.parametrize("precision,cls,n", [(sph.MIXED, "s1_n2^20", 1 << 20), (sph.MIXED, "s1_n2^24", 1 << 24)])
def test_apply_sets_every_option(monkeypatch, precision, cls, n):
    monkeypatch.setattr(autotune, "gpu_name", lambda device=0: "NVIDIA GB300")
    monkeypatch.setattr(autotune, "CACHE", "/nonexistent/tuned.json")
    ctx = RecordingContext()
    cfg = autotune.apply(ctx, scenario(n), precision)
    with open(autotune.SHIPPED) as f:
        best = json.load(f)[f"NVIDIA GB300|p{precision}|{cls}"]["best"]
    assert cfg == best
    assert ctx.tuning == (best["block"], best["cell_factor"])
    assert ctx.options["cell_factor_z"] == best.get("cell_factor_z", 1.0)
    assert ctx.options["list_mode"] == best["list_mode"] and ctx.options["slack"] == best["slack"]


def test_unknown_gpu_keeps_the_defaults(monkeypatch):
    monkeypatch.setattr(autotune, "gpu_name", lambda device=0: "some other GPU")
    monkeypatch.setattr(autotune, "CACHE", "/nonexistent/tuned.json")
    ctx = RecordingContext()
    assert autotune.apply(ctx, scenario(1 << 20), sph.MIXED) is None
    assert ctx.tuning is None and not ctx.options
