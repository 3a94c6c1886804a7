"""The allocation-free cell sort, sph_cell_sort_static, for callers that must
not allocate device memory while running (fixed device-memory budgets, their
own pool allocators, latency-critical loops).  Called through the C ABI and
checked against the allocating sph_cell_sort on the same inputs, on two calls
in a row (the shared static scratch keeps the previous call's contents, so the
second call also checks that everything that must start at zero is cleared).
Collected last on purpose: it passes alone in a fresh process and after the
other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(fn, keys, ncells):
    import torch
    n = keys.size
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    perm = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    start = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(dk.data_ptr() if n else None, n, ncells, perm.data_ptr(), start.data_ptr(), None)
    return rc, perm.cpu().numpy()[:n], start.cpu().numpy()


def test_static_cell_sort_matches_allocating_one(cuda_lib):
    from deorbit_gb300 import sph
    L = sph.lib()
    rng = np.random.default_rng(2024)
    cases = [(200_000, 3000), (1234, 77)]  # two calls in a row, the second smaller
    for n, ncells in cases:
        keys = rng.integers(0, ncells, size=n).astype(np.uint32)
        rc0, p0, s0 = _sort(L.sph_cell_sort, keys, ncells)
        rc1, p1, s1 = _sort(L.sph_cell_sort_static, keys, ncells)
        assert rc0 == 0 and rc1 == 0, L.sph_last_error()
        assert np.array_equal(p0, p1) and np.array_equal(s0, s1)
        assert np.array_equal(p1, np.argsort(keys, kind="stable"))


def test_static_cell_sort_rejects_oversize(cuda_lib):
    from deorbit_gb300 import sph
    L = sph.lib()
    rc = L.sph_cell_sort_static(None, (1 << 18) + 1, 10, None, None, None)
    assert rc == -6 and b"262144" in L.sph_last_error()
