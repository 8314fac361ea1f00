"""The allocation-free entry point, gbp_npairs_3d_static, against the oracle.

gbp_npairs_3d_static serves callers that cannot allocate device memory while
they count (their device memory belongs to another framework's caching
allocator, or a cudaMalloc/cudaFree would stall a latency-critical loop): all
its scratch is one static device array inside the library.  These tests call
it through the C ABI: three times in a row on different samples (periodic and
not), each against the oracle's integer counts and the allocating entry
point's, so a call must not see the previous call's leftovers; with a point
outside the box (every count -1, and the next call clean again); checking
that free device memory does not move across a call; and on a stream being
captured (refused).  The file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _call(lib, x_dev, out, rbins, period, pbc, stream):
    rb = np.ascontiguousarray(rbins, dtype=np.float64)
    per = np.ascontiguousarray(period, dtype=np.float64)
    return lib.gbp_npairs_3d_static(
        ctypes.c_void_p(x_dev.data_ptr()), x_dev.shape[0],
        rb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(rb),
        per.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(pbc),
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))


def _static_counts(lib, x_dev, rbins, period, pbc, stream):
    import torch
    out = torch.zeros(len(rbins), dtype=torch.int64, device=x_dev.device)
    rc = _call(lib, x_dev, out, rbins, period, pbc, stream)
    assert rc == 0, rc
    stream.synchronize()
    return out.cpu().numpy()


def test_static_entry_matches_oracle_twice(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(123)
    cases = [
        (rng.uniform(0, 150.0, (60000, 3)), np.logspace(-1, np.log10(20), 15), 150.0, 1),
        (rng.uniform(0, 80.0, (25000, 3)), np.array([0.0, 0.5, 2.0, 5.0, 9.0]), 80.0, 0),
        (rng.uniform(0, 100.0, (131072, 3)), np.logspace(-1, np.log10(12), 20), 100.0, 1),
    ]
    for x, rb, L, pbc in cases:
        # pbc = 0: no wrap inside the box [0, L] (the oracle's period=None
        # encloses the same points; the separations and counts are the same)
        want = oracle.npairs_3d(x, x, rb, period=L if pbc else None, num_threads=8)
        got = _static_counts(lib, torch.from_numpy(x).cuda(), rb, [L] * 3, pbc, stream)
        assert np.array_equal(got, want), (pbc, got, want)
        # and the allocating entry point (gbp_npairs_3d behind npairs_3d) agrees
        assert np.array_equal(got, gpu.npairs_3d(x, x, rb, period=L if pbc else None))


def test_static_entry_out_of_box_gives_minus_one_then_recovers(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(7)
    x = rng.uniform(0, 50.0, (5000, 3))
    rb = np.logspace(-1, np.log10(10), 8)
    bad = x.copy()
    bad[17, 0] = 75.0  # outside [0, 50]
    got = _static_counts(lib, torch.from_numpy(bad).cuda(), rb, [50.0] * 3, 1, stream)
    assert np.all(got == -1), got
    got = _static_counts(lib, torch.from_numpy(x).cuda(), rb, [50.0] * 3, 1, stream)
    assert np.array_equal(got, oracle.npairs_3d(x, x, rb, period=50.0))


def test_static_entry_allocates_no_device_memory(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream()
    x = torch.from_numpy(np.random.default_rng(9).uniform(0, 60.0, (40000, 3))).cuda()
    out = torch.zeros(10, dtype=torch.int64, device="cuda")
    rb = np.logspace(-1, np.log10(12), 10)
    assert _call(lib, x, out, rb, [60.0] * 3, 1, stream) == 0  # first call: set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, x, out, rb, [60.0] * 3, 1, stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_static_entry_refuses_a_capturing_stream(gpu):
    import torch
    from halotools_gb300 import _native
    lib = _native.load()
    x = torch.from_numpy(np.random.default_rng(3).uniform(0, 30.0, (1000, 3))).cuda()
    out = torch.zeros(5, dtype=torch.int64, device="cuda")
    rb = np.array([0.5, 1.0, 2.0, 4.0, 8.0])
    assert _call(lib, x, out, rb, [30.0] * 3, 1, torch.cuda.current_stream()) == 0
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    y = torch.zeros(1, device="cuda")
    with torch.cuda.graph(g, stream=s):
        y.add_(1.0)
        rc = _call(lib, x, out, rb, [30.0] * 3, 1, s)
    assert rc == _native.GBP_ERR_INVALID


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
