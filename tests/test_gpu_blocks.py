"""Two-level grid: fine cells grouped into blocks of bf^3 cells (the i-side of
a work item) with a run-length stencil of fine cells around the block.  Every
engine must give the reference's counts whatever the block factor.
"""
import contextlib

import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import clustered

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def forced(gpu, block=0, reach=0):
    plan = gpu.default_plan()
    plan.set_block(block)
    plan.set_reach(reach)
    try:
        yield plan
    finally:
        plan.set_block(0)
        plan.set_reach(0)


@pytest.mark.parametrize("block", [1, 2, 3, 4])
@pytest.mark.parametrize("pbc", [True, False])
def test_npairs_3d_any_block_matches_oracle(gpu, block, pbc):
    rng = np.random.default_rng(100 + block)
    L = 420.0
    s = clustered(rng, 30000, L, 1500)
    rb = np.logspace(-1, np.log10(20), 15)
    per = L if pbc else None
    want = oracle.npairs_3d(s, s, rb, period=per, num_threads=8)
    with forced(gpu, block) as plan:
        got = gpu.npairs_3d(s, s, rb, period=per)
        st = plan.stats()
    assert st["block"] == block
    assert np.array_equal(got, want)


@pytest.mark.parametrize("block", [2, 3])
def test_npairs_3d_blocks_cross_nonperiodic(gpu, block):
    # boxes whose cell counts are not multiples of the block factor
    rng = np.random.default_rng(7)
    s1 = rng.uniform(-30, 171, (25000, 3))
    s2 = rng.uniform(0, 137, (18000, 3))
    rb = np.logspace(-1, np.log10(9.5), 11)
    want = oracle.npairs_3d(s1, s2, rb, num_threads=8)
    with forced(gpu, block) as plan:
        got = gpu.npairs_3d(s1, s2, rb)
        assert plan.stats()["block"] == block
    assert np.array_equal(got, want)


def test_sparse_sample_chooses_blocks_by_default(gpu):
    rng = np.random.default_rng(8)
    L = 1000.0
    s = clustered(rng, 60000, L, 3000)
    rb = np.logspace(-1, np.log10(20), 15)
    got = gpu.npairs_3d(s, s, rb, period=L)
    assert gpu.default_plan().stats()["block"] > 1
    assert np.array_equal(got, oracle.npairs_3d(s, s, rb, period=L, num_threads=8))


@pytest.mark.parametrize("block", [2, 3])
def test_xy_z_and_s_mu_with_blocks(gpu, block):
    rng = np.random.default_rng(9)
    L = 500.0
    s = clustered(rng, 30000, L, 1500)
    rp = np.logspace(-1, np.log10(20), 15)
    pi = np.linspace(0, 25, 26)
    sb = np.logspace(np.log10(0.5), np.log10(20), 16)
    mu = np.linspace(0, 1, 11)
    w_xyz = oracle.npairs_xy_z(s, s, rp, pi, period=L, num_threads=8)
    w_smu = oracle.npairs_s_mu(s, s, sb, mu, period=L, num_threads=8)
    with forced(gpu, block) as plan:
        g_xyz = gpu.npairs_xy_z(s, s, rp, pi, period=L)
        assert plan.stats()["block"] == block
        g_smu = gpu.npairs_s_mu(s, s, sb, mu, period=L)
        assert plan.stats()["block"] == block
    assert np.array_equal(g_xyz, w_xyz)
    assert np.array_equal(g_smu, w_smu)


def test_marked_with_blocks(gpu):
    rng = np.random.default_rng(10)
    L = 500.0
    s = clustered(rng, 30000, L, 1500)
    w = rng.lognormal(0.0, 0.5, len(s))
    rb = np.logspace(np.log10(0.5), np.log10(20), 16)
    want = oracle.marked_npairs_3d(s, s, rb, 1, period=L, weights1=w, weights2=w, num_threads=8)
    with forced(gpu, 3) as plan:
        got = gpu.marked_npairs_3d(s, s, rb, 1, period=L, weights1=w, weights2=w)
        assert plan.stats()["block"] == 3
    np.testing.assert_allclose(got, want, rtol=1e-6)


def test_reach_two_with_blocks(gpu):
    rng = np.random.default_rng(11)
    L = 300.0
    s = clustered(rng, 40000, L, 2000)
    rb = np.logspace(-1, np.log10(25), 20)
    want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)
    with forced(gpu, 2, 2) as plan:
        got = gpu.npairs_3d(s, s, rb, period=L)
        st = plan.stats()
    assert (st["reach"], st["block"]) == (2, 2)
    assert np.array_equal(got, want)


def test_adjoint_with_blocks_matches_fp64_gradient(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    from halotools_gb300 import mocks
    L = 80.0
    pos, mass, _ = mocks.halo_table(5000, L, seed=12)
    w = 0.5 + np.random.default_rng(13).uniform(size=len(mass))
    rb = np.logspace(-1, np.log10(12), 10)
    gbar = np.random.default_rng(14).normal(size=len(rb))
    want = oracle.weighted_adjoint_3d(pos, w, rb, L, gbar)
    with forced(gpu, 3):
        wt = torch.from_numpy(w).cuda().requires_grad_(True)
        C = D.weighted_pair_counts(wt, torch.from_numpy(pos).cuda(), rb, L)
        (C * torch.from_numpy(gbar).cuda()).sum().backward()
    got = wt.grad.cpu().numpy()
    assert np.max(np.abs(got - want)) / np.abs(want).max() < 2e-6


@pytest.mark.parametrize("block", [2, 4])
def test_batched_with_blocks_equals_per_mock(gpu, block):
    from tests.test_gpu_parity import _mocks
    L = 400.0
    mocks = _mocks(41, [12000, 0, 25000, 3000, 1, 9000], L)
    rb = np.logspace(-1, np.log10(20), 15)
    bc = gpu.BatchedCounter(graph=True, autotune=False)
    bc.plan.set_block(block)
    got = bc(mocks, rb, L)
    assert bc.stats()["block"] == block
    for m, s in enumerate(mocks):
        want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8) if len(s) else \
            np.zeros(len(rb), np.int64)
        assert np.array_equal(got[m], want), m


# ---------------- product marks over several channels in one pass ----------------
@pytest.mark.parametrize("nch", [1, 2, 3, 8])
def test_marked_channels_match_oracle(gpu, nch):
    rng = np.random.default_rng(60 + nch)
    L = 400.0
    s = clustered(rng, 30000, L, 1500)
    w = np.stack([rng.lognormal(0.0, 0.5, len(s)) if c % 2 == 0 else rng.uniform(0, 1, len(s))
                  for c in range(nch)], axis=1)
    rb = np.logspace(np.log10(0.5), np.log10(25), 20)
    got = gpu.marked_npairs_3d_channels(s, s, rb, period=L, weights1=w, weights2=w)
    assert got.shape == (nch, len(rb))
    for c in range(nch):
        want = oracle.marked_npairs_3d(s, s, rb, 1, period=L, weights1=w[:, c],
                                       weights2=w[:, c], num_threads=8)
        np.testing.assert_allclose(got[c], want, rtol=1e-6)


def test_marked_channels_cross_nonperiodic_and_ones(gpu):
    rng = np.random.default_rng(70)
    s1 = rng.uniform(0, 150, (20000, 3))
    s2 = rng.uniform(10, 140, (15000, 3))
    w1 = rng.uniform(0.5, 2.0, (len(s1), 4))
    w2 = rng.uniform(0.5, 2.0, (len(s2), 4))
    rb = np.logspace(-1, np.log10(12), 12)
    got = gpu.marked_npairs_3d_channels(s1, s2, rb, weights1=w1, weights2=w2)
    for c in range(4):
        want = oracle.marked_npairs_3d(s1, s2, rb, 1, weights1=w1[:, c], weights2=w2[:, c],
                                       num_threads=8)
        np.testing.assert_allclose(got[c], want, rtol=1e-6)
    # unit marks give the integer counts
    ones = gpu.marked_npairs_3d_channels(s1, s2, rb, weights1=np.ones((len(s1), 2)),
                                         weights2=np.ones((len(s2), 2)))
    cnt = gpu.npairs_3d(s1, s2, rb).astype(np.float64)
    assert np.array_equal(ones[0], cnt) and np.array_equal(ones[1], cnt)


@pytest.mark.parametrize("pbc", [True, False])
def test_dense_sample_takes_reach_4_blocks_by_default(gpu, pbc):
    # 37 points per reach-2 cell: npairs_3d and npairs_s_mu choose reach 4 in
    # blocks of 2 on their own (periodic, and over the enclosing box)
    rng = np.random.default_rng(15)
    L = 100.0
    s = clustered(rng, 300000, L, 6000, mhi=13.5)
    rb = np.logspace(-1, 1, 12)
    per = L if pbc else None
    got = gpu.npairs_3d(s, s, rb, period=per)
    st = gpu.default_plan().stats()
    assert (st["reach"], st["block"]) == (4, 2)
    assert np.array_equal(got, oracle.npairs_3d(s, s, rb, period=per, num_threads=8))
    sb = np.logspace(np.log10(0.5), 1, 11)
    mu = np.linspace(0, 1, 11)
    got = gpu.npairs_s_mu(s, s, sb, mu, period=per)
    st = gpu.default_plan().stats()
    assert (st["reach"], st["block"]) == (4, 2)
    assert np.array_equal(got, oracle.npairs_s_mu(s, s, sb, mu, period=per, num_threads=8))


def test_reach_4_blocks_cross_counts(gpu):
    # two samples: the stencil covers the whole neighbourhood of each block
    rng = np.random.default_rng(16)
    L = 120.0
    s1 = clustered(rng, 40000, L, 2000)
    s2 = rng.uniform(0, L, (70000, 3))
    rb = np.logspace(-1, np.log10(12), 14)
    want = oracle.npairs_3d(s1, s2, rb, period=L, num_threads=8)
    with forced(gpu, 2, 4) as plan:
        got = gpu.npairs_3d(s1, s2, rb, period=L)
        st = plan.stats()
    assert (st["reach"], st["block"]) == (4, 2)
    assert np.array_equal(got, want)
