"""Parity at the benchmark configurations' full sizes, through the C ABI,
against the oracle (oracle/oracle.py, pinned to the reference's compiled
engines by tests/test_oracle.py):

* config 2: npairs_xy_z on 2M clustered points, bit-exact;
* config 3: 64 GPU-drawn Zheng07 mocks in one batched, graph-captured,
  autotuned launch, bit-exact per mock (float32 positions upcast exactly);
* config 4: the Zheng07-weighted count of 2M halos, forward within 1e-6 of
  FP64 per bin, dC_k/dtheta per bin against the FP64 Jacobian, and against
  central finite differences (h = 1e-4) of the FP64 forward on a box of 1/8
  the volume at the same density;
* config 5: 10M clustered points: npairs_3d and npairs_s_mu bit-exact, the two
  mark components of marked_npairs_3d (id 1) within 1e-6 of FP64 per bin;
* the rare paths those sizes could reach: the early flush of the 32-bit
  histogram words and the work-item overflow-and-retry, forced on small
  inputs through gbp_plan_set_limits.

These cost a few minutes of host time (the oracle on all host cores).
"""
import os

import numpy as np
import pytest

from oracle import oracle, parity

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8
THETA = np.array([12.0, 0.3, 12.0, 13.3, 1.0])


@pytest.fixture(scope="module")
def points_10m():
    from halotools_gb300 import mocks
    return mocks.clustered_points(10_000_000, 2000.0, 1_000_000, logm_range=(11.0, 15.5), seed=2)


def test_config2_npairs_xy_z_2m_exact(gpu):
    from halotools_gb300 import mocks
    x = mocks.clustered_points(2_000_000, 1000.0, 200_000, logm_range=(11.0, 15.0), seed=2)
    rp, pi = np.logspace(-1, np.log10(30), 20), np.linspace(0, 40, 40)
    got = gpu.npairs_xy_z(x, x, rp, pi, period=1000.0)
    want = oracle.npairs_xy_z(x, x, rp, pi, period=1000.0, num_threads=THREADS)
    assert parity.exact(got, want)["exact"]
    assert want[-1, -1] > 9e8


def test_config3_batched_64_mocks_exact(gpu):
    from halotools_gb300 import BatchedCounter, mocks
    L = 1000.0
    pos, mass, conc = mocks.halo_table(1_000_000, L, seed=11)
    rng = np.random.default_rng(12)
    lmin = rng.uniform(11.8, 12.4, 64)
    thetas = np.stack([lmin, rng.uniform(0.2, 0.5, 64), lmin, lmin + 1.3,
                       rng.uniform(0.9, 1.1, 64)], axis=1)
    xyz, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, thetas, seed=13)
    rb = np.logspace(-1, np.log10(20), 15)
    bc = BatchedCounter(0, graph=True, autotune=True)
    out = bc.count_device(xyz, offs, rb, L)
    again = bc.count_device(xyz, offs, rb, L)  # the graph replay
    assert np.array_equal(out, again)
    xs = xyz.cpu().numpy().astype(np.float64)
    assert len(offs) == 65
    for m in range(64):
        s = xs[offs[m]:offs[m + 1]]
        want = oracle.npairs_3d(s, s, rb, period=L, num_threads=THREADS)
        assert np.array_equal(out[m], want), m


def _jacobian_gpu(D, th_np, xd, md, rb, L):
    import torch
    th = torch.tensor(th_np, dtype=torch.float64, device="cuda", requires_grad=True)
    C = D.hod_pair_counts(th, xd, md, rb, L)
    J = np.stack([torch.autograd.grad(C[k], th, retain_graph=True)[0].cpu().numpy()
                  for k in range(len(rb))])
    return C.detach().cpu().numpy(), J


def test_config4_weighted_2m_forward_and_jacobian(gpu):
    import torch
    from halotools_gb300 import differentiable as D, mocks
    L = 1000.0
    pos, mass, _ = mocks.halo_table(2_000_000, L, seed=21)
    rb = np.logspace(-1, np.log10(30), 20)
    C, J = _jacobian_gpu(D, THETA, torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda(),
                         rb, L)
    w = parity.zheng07_fp64(THETA, mass)
    S = oracle.weighted_per_object_3d(pos, w, rb, L, THREADS)
    C64, J64 = parity.weighted_counts_and_jacobian(S, w, parity.zheng07_jacobian_fp64(THETA, mass))
    rel = np.array(parity.rel_per_bin(C, C64))
    assert rel.max() < 1e-6, rel
    # per bin, the largest error over the 5 parameters against the bin's largest entry
    jr = np.abs(J - J64).max(axis=1) / np.abs(J64).max(axis=1)
    assert jr.max() < 1e-5, jr


def test_config4_jacobian_against_central_differences(gpu):
    """dC_k/dtheta per bin against central differences (h = 1e-4) of the FP64
    forward, on 250k halos in L = 500 (config 4's density, 1/8 of its volume)."""
    import torch
    from halotools_gb300 import differentiable as D, mocks
    L = 500.0
    pos, mass, _ = mocks.halo_table(250_000, L, seed=22)
    rb = np.logspace(-1, np.log10(30), 20)
    _, J = _jacobian_gpu(D, THETA, torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda(),
                         rb, L)
    h = 1e-4
    fd = np.zeros_like(J)
    for p in range(5):
        e = np.zeros(5)
        e[p] = h
        cp = oracle.marked_npairs_3d(pos, pos, rb, 1, period=L,
                                     weights1=parity.zheng07_fp64(THETA + e, mass),
                                     weights2=parity.zheng07_fp64(THETA + e, mass),
                                     num_threads=THREADS)
        cm = oracle.marked_npairs_3d(pos, pos, rb, 1, period=L,
                                     weights1=parity.zheng07_fp64(THETA - e, mass),
                                     weights2=parity.zheng07_fp64(THETA - e, mass),
                                     num_threads=THREADS)
        fd[:, p] = (cp - cm) / (2 * h)
    scale = np.abs(fd).max(axis=1)
    assert np.all(np.abs(J - fd).max(axis=1) <= 2e-4 * scale), np.abs(J - fd).max(axis=1) / scale


def test_config5_npairs_3d_10m_exact(gpu, points_10m):
    x = points_10m
    rb = np.logspace(np.log10(0.5), np.log10(50), 30)
    got = gpu.npairs_3d(x, x, rb, period=2000.0)
    want = oracle.npairs_3d(x, x, rb, period=2000.0, num_threads=THREADS)
    assert np.array_equal(got, want)
    assert want[-1] > 6e9


def test_config5_npairs_s_mu_10m_exact(gpu, points_10m):
    x = points_10m
    sb = np.logspace(np.log10(0.5), np.log10(50), 30)
    mu = np.linspace(0.0, 1.0, 21)
    got = gpu.npairs_s_mu(x, x, sb, mu, period=2000.0)
    want = oracle.npairs_s_mu(x, x, sb, mu, period=2000.0, num_threads=THREADS)
    assert np.array_equal(got, want)


def test_config5_marked_two_components_10m(gpu, points_10m):
    import torch
    from halotools_gb300 import _native as N
    x = points_10m
    n = len(x)
    rb = np.logspace(np.log10(0.5), np.log10(50), 30)
    rng = np.random.default_rng(51)
    comp = np.stack([rng.lognormal(0.0, 0.5, n), rng.uniform(0.0, 1.0, n)], axis=1)
    xd = torch.from_numpy(x).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(comp)).cuda()
    plan = N.Plan(0)
    out = np.zeros((2, len(rb)))
    box = np.array([2000.0] * 3)
    plan.check(plan.lib.gbp_marked_npairs_3d_channels(
        plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, cd.data_ptr(), cd.data_ptr(), 2,
        N.pd(rb), len(rb), N.pd(box), 1, N.GBP_MEM_DEVICE, N.pd(out)))
    for c in range(2):
        want = oracle.marked_npairs_3d(x, x, rb, 1, period=2000.0, weights1=comp[:, c],
                                       weights2=comp[:, c], num_threads=THREADS)
        rel = np.array(parity.rel_per_bin(out[c], want))
        assert rel.max() < 1e-6, (c, rel)


def test_early_histogram_flush_and_item_retry(gpu):
    """The 32-bit histogram words moved to the 64-bit totals after every work
    item (flush_after = 1, or 64: after each item of more than one j-batch),
    and a first item capacity of 64 that the call overflows and repeats:
    counts unchanged, for the 1-D, (rp, pi) and (s, mu') kernels."""
    from halotools_gb300 import _native as N
    from halotools_gb300 import mocks
    x = mocks.clustered_points(200_000, 300.0, 20_000, seed=5)
    rb = np.logspace(-1, np.log10(25), 15)
    pi = np.linspace(0, 30, 16)
    mu = np.linspace(0, 1, 11)
    want3 = oracle.npairs_3d(x, x, rb, period=300.0, num_threads=THREADS)
    wantx = oracle.npairs_xy_z(x, x, rb, pi, period=300.0, num_threads=THREADS)
    wants = oracle.npairs_s_mu(x, x, rb, mu, period=300.0, num_threads=THREADS)
    plan = N.default_plan()
    try:
        for cap, flush in ((64, 1), (64, 0), (0, 64)):
            plan.set_limits(first_item_cap=cap, flush_after=flush)
            assert np.array_equal(gpu.npairs_3d(x, x, rb, period=300.0), want3)
            plan.set_limits(first_item_cap=cap, flush_after=flush)
            assert np.array_equal(gpu.npairs_xy_z(x, x, rb, pi, period=300.0), wantx)
            plan.set_limits(first_item_cap=cap, flush_after=flush)
            assert np.array_equal(gpu.npairs_s_mu(x, x, rb, mu, period=300.0), wants)
    finally:
        plan.set_limits(0, 0)
