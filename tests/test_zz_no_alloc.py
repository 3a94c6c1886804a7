"""The allocation-free cell sort, sph_cell_sort_static, for callers that must
not allocate device memory while running (fixed device-memory budgets, their
own pool allocators, latency-critical loops).  Called through the C ABI and
checked against the allocating sph_cell_sort and a host stable sort on the same
inputs, on calls in a row (the shared static scratch keeps the previous call's
contents, so later calls also check that everything that must start at zero is
cleared): a large case, the documented maximum of 262,144 keys over 16,777,216
cells, a small case, an empty key array, a key out of range and a call on a
stream under graph capture.  Collected last on purpose: it passes alone in a
fresh process and after the other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPH_ERR_ARG, SPH_ERR_STATE, SPH_ERR_CAPACITY = -1, -3, -6


def _sort(fn, keys, ncells):
    import torch
    n = keys.size
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    perm = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    start = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(dk.data_ptr() if n else None, n, ncells, perm.data_ptr(), start.data_ptr(), None)
    return rc, perm.cpu().numpy()[:n], start.cpu().numpy()


def _host_start(keys, ncells):
    return np.r_[0, np.cumsum(np.bincount(keys, minlength=ncells))].astype(np.int32)


def test_static_cell_sort_matches_allocating_one(cuda_lib):
    from deorbit_gb300 import sph
    L = sph.lib()
    rng = np.random.default_rng(2024)
    # calls in a row: large, the documented maximum, small, empty
    cases = [(200_000, 3000), (1 << 18, 1 << 24), (1234, 77), (0, 5)]
    for n, ncells in cases:
        keys = rng.integers(0, ncells, size=n).astype(np.uint32)
        rc0, p0, s0 = _sort(L.sph_cell_sort, keys, ncells)
        rc1, p1, s1 = _sort(L.sph_cell_sort_static, keys, ncells)
        assert rc0 == 0 and rc1 == 0, (n, ncells, L.sph_last_error())
        assert np.array_equal(p0, p1) and np.array_equal(s0, s1), (n, ncells)
        assert np.array_equal(p1, np.argsort(keys, kind="stable")), (n, ncells)
        assert np.array_equal(s1, _host_start(keys, ncells)), (n, ncells)


def test_static_cell_sort_rejects_bad_input(cuda_lib):
    from deorbit_gb300 import sph
    L = sph.lib()
    rc = L.sph_cell_sort_static(None, (1 << 18) + 1, 10, None, None, None)
    assert rc == SPH_ERR_CAPACITY and b"262144" in L.sph_last_error()
    rc = L.sph_cell_sort_static(None, 10, (1 << 24) + 1, None, None, None)
    assert rc == SPH_ERR_CAPACITY
    # a key outside [0, ncells) is reported, and the next call is clean again
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 100, size=5000).astype(np.uint32)
    keys[1234] = 100
    rc, _, _ = _sort(L.sph_cell_sort_static, keys, 100)
    assert rc == SPH_ERR_ARG and b"outside" in L.sph_last_error()
    keys[1234] = 99
    rc, p, s = _sort(L.sph_cell_sort_static, keys, 100)
    assert rc == 0
    assert np.array_equal(p, np.argsort(keys, kind="stable"))
    assert np.array_equal(s, _host_start(keys, 100))


def test_static_cell_sort_refuses_capture(cuda_lib):
    """The call synchronizes, so on a stream being captured it must refuse
    before touching the stream (the capture itself stays valid)."""
    import torch
    from deorbit_gb300 import sph
    L = sph.lib()
    keys = torch.zeros(64, dtype=torch.int32, device="cuda")
    perm = torch.zeros(64, dtype=torch.int32, device="cuda")
    start = torch.zeros(9, dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=side):
        rc = L.sph_cell_sort_static(keys.data_ptr(), 64, 8, perm.data_ptr(), start.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream)
        keys.add_(0)  # the capture holds some work of its own
    assert rc == SPH_ERR_STATE and b"captur" in L.sph_last_error()
    g.replay()
    torch.cuda.synchronize()
