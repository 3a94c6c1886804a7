"""bench.py's frozen traffic constants agree with the engine's state layout."""
import bench


def test_step_bytes_follow_the_layout():
    for real, frozen in bench.STEP_BYTES.items():
        assert bench.step_bytes(real) == frozen
    plain, mixed = bench.state_layout(8), bench.state_layout(4)
    assert plain.keys() == mixed.keys()
    for k in ("pos", "vel", "u", "mat", "fixed"):   # the same storage in both forms
        assert plain[k] == mixed[k]


def test_roofline_tables_are_consistent():
    assert set(bench.ALG_BYTES) <= set(bench.KERNEL_OF_CLASS)
    for fixed, per_entry in bench.ALG_BYTES.values():
        assert fixed > 0 and per_entry >= 0
    assert set(bench.FLOPS_PER_ENTRY) <= set(bench.ALG_BYTES)
    assert bench.FP32_LANES_PER_SM == 128  # FP32 lanes per SM of compute capability 10.x
