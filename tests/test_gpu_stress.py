"""Inputs at the edges of the work decomposition, against the oracle."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def test_everything_in_one_clump(gpu):
    # one cell holds 25,000 points: i-chunks of 64 and one stencil run far
    # longer than an item's j-group cap
    rng = np.random.default_rng(81)
    L = 200.0
    s = np.mod(100.0 + rng.normal(0, 0.3, (25000, 3)), L)
    rb = np.logspace(-2, np.log10(3.0), 14)
    want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_3d(s, s, rb, period=L), want)
    wr = oracle.npairs_xy_z(s, s, rb, np.linspace(0, 2, 9), period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_xy_z(s, s, rb, np.linspace(0, 2, 9), period=L), wr)


def test_clump_plus_sparse_background(gpu):
    rng = np.random.default_rng(82)
    L = 500.0
    s = np.concatenate([np.mod(250.0 + rng.normal(0, 1.0, (15000, 3)), L),
                        rng.uniform(0, L, (20000, 3))])
    rb = np.logspace(-1, np.log10(30), 18)
    want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_3d(s, s, rb, period=L), want)


@pytest.mark.parametrize("block", [0, 2, 3])
def test_noncubic_periodic_box(gpu, block):
    rng = np.random.default_rng(83)
    per = np.array([300.0, 120.0, 210.0])
    s = rng.uniform(0, 1, (30000, 3)) * per
    rb = np.logspace(-1, np.log10(25), 16)
    want = oracle.npairs_3d(s, s, rb, period=per, num_threads=8)
    plan = gpu.default_plan()
    plan.set_block(block)
    try:
        got = gpu.npairs_3d(s, s, rb, period=per)
    finally:
        plan.set_block(0)
    assert np.array_equal(got, want)


def test_search_at_a_third_of_the_box(gpu):
    # the largest search the reference allows (rectangular_mesh.py:376-417)
    rng = np.random.default_rng(84)
    L = 90.0
    s = rng.uniform(0, L, (8000, 3))
    rb = np.array([1.0, 10.0, 29.999999])
    want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_3d(s, s, rb, period=L), want)


def test_batched_uneven_mocks(gpu):
    rng = np.random.default_rng(85)
    L = 400.0
    mocks = [rng.uniform(0, L, (n, 3)) for n in (2, 60000, 0, 17, 5000, 1)]
    mocks.append(np.mod(200.0 + rng.normal(0, 0.5, (8000, 3)), L))
    rb = np.logspace(-1, np.log10(20), 12)
    bc = gpu.BatchedCounter(graph=True, autotune=True)
    got = bc(mocks, rb, L)
    for m, s in enumerate(mocks):
        want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8) if len(s) else \
            np.zeros(len(rb), np.int64)
        assert np.array_equal(got[m], want), m
