"""The allocation-free entry point, gbp_npairs_3d_static, against gbp_npairs_3d.

gbp_npairs_3d_static serves callers that cannot allocate device memory while
they count (their device memory belongs to another allocator, or a
cudaMalloc/cudaFree would stall a latency-critical loop): all its scratch is
one static device array inside the library.  This test calls it through the
C ABI twice in a row, on two different samples, and requires the same
integer counts as the ordinary entry point each time, so a call must not see
the previous call's leftovers.  It is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_counts(lib, x_dev, rbins, period, stream):
    import torch
    out = torch.zeros(len(rbins), dtype=torch.int64, device=x_dev.device)
    rb = np.ascontiguousarray(rbins, dtype=np.float64)
    per = np.ascontiguousarray(period, dtype=np.float64)
    rc = lib.gbp_npairs_3d_static(
        ctypes.c_void_p(x_dev.data_ptr()), x_dev.shape[0],
        rb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(rb),
        per.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    stream.synchronize()
    return out.cpu().numpy()


def test_static_entry_matches_plan_entry_twice(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(123)
    cases = [
        (rng.uniform(0, 150.0, (60000, 3)), np.logspace(-1, np.log10(20), 15), 150.0),
        (rng.uniform(0, 80.0, (25000, 3)), np.array([0.0, 0.5, 2.0, 5.0, 9.0]), 80.0),
    ]
    for x, rb, L in cases:
        want = gpu.npairs_3d(x, x, rb, period=L)
        got = _static_counts(lib, torch.from_numpy(x).cuda(), rb, [L] * 3, stream)
        assert np.array_equal(got, want), (got, want)


def test_static_entry_rejects_oversize(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    n = 131072 + 1
    x = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.int64, device="cuda")
    rb = np.array([0.1, 0.2, 0.3, 0.4])
    per = np.array([10.0, 10.0, 10.0])
    rc = lib.gbp_npairs_3d_static(
        ctypes.c_void_p(x.data_ptr()), n, rb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4,
        per.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1, ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(0))
    assert rc == _native.GBP_ERR_INVALID
