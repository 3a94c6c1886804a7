"""sph_cell_sort (the radix cell sort as a device primitive) against a host
stable sort: permutation and cell starts bit-exact, bad keys rejected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,ncells", [(0, 5), (1, 1), (1000, 37), (300000, 1 << 12), (70000, 3_000_000)])
def test_cell_sort_matches_host(cuda_lib, n, ncells):
    import torch
    from deorbit_gb300 import sph
    rng = np.random.default_rng(n + ncells)
    keys = rng.integers(0, ncells, size=n).astype(np.uint32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    start = torch.empty(ncells + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    sph.check(sph.lib().sph_cell_sort(dk.data_ptr() if n else None, n, ncells, perm.data_ptr(),
                                      start.data_ptr(), None))
    ref_perm = np.argsort(keys, kind="stable")
    ref_start = np.r_[0, np.cumsum(np.bincount(keys, minlength=ncells))]
    assert np.array_equal(perm.cpu().numpy()[:n], ref_perm)
    assert np.array_equal(start.cpu().numpy(), ref_start)


def test_cell_sort_rejects_bad_keys(cuda_lib):
    import torch
    from deorbit_gb300 import sph
    dk = torch.tensor([0, 1, 7], dtype=torch.int32, device="cuda")
    perm = torch.empty(3, dtype=torch.int32, device="cuda")
    start = torch.empty(5, dtype=torch.int32, device="cuda")
    rc = sph.lib().sph_cell_sort(dk.data_ptr(), 3, 4, perm.data_ptr(), start.data_ptr(), None)
    assert rc == -1 and b"outside" in sph.lib().sph_last_error()
