"""The allocation-free scan, for callers that cannot allocate device memory.

Collected last on purpose: a failure here leaves every other test already run.
It compares letkf_exclusive_scan_static with the allocating
letkf_exclusive_scan on two calls in a row (the second with a smaller input,
so stale contents of the shared scratch array would show).  Offsets are
integers: the bar is equality."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_scan_matches_allocating_scan(cuda):
    import torch

    from letkf_gb300.core import exclusive_scan, exclusive_scan_static
    from letkf_gb300.lib import LETKF_OK

    rng = np.random.default_rng(42)
    for n in (3_000_001, 5_000):
        counts = torch.as_tensor(rng.integers(0, 2100, n).astype(np.int32), device=cuda)
        ref = exclusive_scan(counts)
        out = torch.full((n + 1,), -7, dtype=torch.int64, device=cuda)
        assert exclusive_scan_static(counts, out) == LETKF_OK
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
        assert int(out[-1]) == int(counts.to(torch.int64).sum())


def test_static_scan_rejects_sizes_beyond_its_array(cuda):
    import ctypes

    from letkf_gb300.lib import LETKF_ERR_CAPACITY, lib

    n = 16 * 1024 * 1024 + 1
    st = lib().letkf_exclusive_scan_static(n, ctypes.c_void_p(1), ctypes.c_void_p(1), None)
    assert st == LETKF_ERR_CAPACITY
