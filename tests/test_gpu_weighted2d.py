"""marked_npairs_xy_z, weighted_npairs_s_mu and npairs_jackknife_xy_z on the GPU
against the C oracle (a restatement of marked_npairs_xy_z_engine.pyx,
weighted_npairs_s_mu_engine.pyx and npairs_jackknife_xy_z_engine.pyx, itself
pinned to halotools' engines in test_oracle.py).

Sums are FP32 with an exact-error companion moved to FP64 every few thousand
pairs: 1e-6 relative of the FP64 reference for non-negative marks (signed marks:
1e-6 of the sum of magnitudes), exact for integer-valued marks.  Counts are
exact."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_blocks import forced
from tests.test_gpu_parity import clustered

pytestmark = pytest.mark.gpu

RTOL = 1e-6
NUMW = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 2, 11: 2,
        12: 4, 13: 4, 14: 3, 15: 3}


def _marks(rng, n, nw, integer=False):
    if integer:
        return rng.integers(0, 4, (n, nw)).astype(np.float64)
    w = rng.uniform(0.2, 2.0, (n, nw))
    w[:, 0] = rng.lognormal(0.0, 0.5, n)
    return w


def _close(got, want):
    scale = np.abs(want)
    assert np.all(np.abs(got - want) <= RTOL * scale + 1e-300), \
        np.max(np.abs(got - want) / np.maximum(scale, 1e-300))


@pytest.mark.parametrize("wid", sorted(NUMW))
def test_marked_xy_z_every_function_auto_pbc(gpu, wid):
    rng = np.random.default_rng(200 + wid)
    L = 250.0
    s = clustered(rng, 12000, L, 600)
    w = _marks(rng, len(s), NUMW[wid])
    if wid in (3, 4):
        w[:, 0] = rng.integers(0, 3, len(s))  # equality tests need ties
    rp = np.logspace(-1, np.log10(15), 12)
    pi = np.linspace(0, 20, 9)
    want = oracle.marked_npairs_xy_z(s, s, rp, pi, wid, period=L, weights1=w, weights2=w,
                                     num_threads=8)
    got = gpu.marked_npairs_xy_z(s, s, rp, pi, period=L, weights1=w, weights2=w,
                                 weight_func_id=wid)
    assert got.shape == want.shape and got.dtype == np.float64
    _close(got, want)  # (every mark here is positive)


@pytest.mark.parametrize("pbc", [True, False])
def test_marked_xy_z_cross(gpu, pbc):
    rng = np.random.default_rng(31)
    L = 200.0
    s1 = clustered(rng, 15000, L, 700)
    s2 = rng.uniform(0, L, (9000, 3))
    w1, w2 = _marks(rng, len(s1), 2), _marks(rng, len(s2), 2)
    rp = np.logspace(-1, np.log10(12), 10)
    pi = np.linspace(0, 15, 16)
    per = L if pbc else None
    for wid in (5, 9, 11):
        want = oracle.marked_npairs_xy_z(s1, s2, rp, pi, wid, period=per, weights1=w1,
                                         weights2=w2, num_threads=8)
        got = gpu.marked_npairs_xy_z(s1, s2, rp, pi, period=per, weights1=w1, weights2=w2,
                                     weight_func_id=wid)
        _close(got, want)


def test_marked_xy_z_integer_marks_exact_and_unit_marks_give_counts(gpu):
    rng = np.random.default_rng(32)
    L = 300.0
    s = clustered(rng, 40000, L, 1500)
    w = _marks(rng, len(s), 1, integer=True)[:, 0]
    rp = np.logspace(-1, np.log10(20), 14)
    pi = np.linspace(0, 25, 11)
    want = oracle.marked_npairs_xy_z(s, s, rp, pi, 1, period=L, weights1=w, weights2=w,
                                     num_threads=8)
    got = gpu.marked_npairs_xy_z(s, s, rp, pi, period=L, weights1=w, weights2=w, weight_func_id=1)
    assert np.array_equal(got, want)
    ones = gpu.marked_npairs_xy_z(s, s, rp, pi, period=L, weight_func_id=1)
    assert np.array_equal(ones, gpu.npairs_xy_z(s, s, rp, pi, period=L).astype(np.float64))


@pytest.mark.parametrize("block", [2, 3])
def test_marked_xy_z_with_blocks(gpu, block):
    rng = np.random.default_rng(33)
    L = 400.0
    s = clustered(rng, 30000, L, 1500)
    w = _marks(rng, len(s), 1)[:, 0]
    rp = np.logspace(-1, np.log10(15), 12)
    pi = np.linspace(0, 20, 11)
    want = oracle.marked_npairs_xy_z(s, s, rp, pi, 1, period=L, weights1=w, weights2=w,
                                     num_threads=8)
    with forced(gpu, block) as plan:
        got = gpu.marked_npairs_xy_z(s, s, rp, pi, period=L, weights1=w, weights2=w,
                                     weight_func_id=1)
        assert plan.stats()["block"] == block
    _close(got, want)


@pytest.mark.parametrize("pbc", [True, False])
def test_weighted_s_mu_matches_oracle(gpu, pbc):
    rng = np.random.default_rng(40)
    L = 250.0
    s = clustered(rng, 30000, L, 1200)
    w = rng.lognormal(0.0, 0.5, len(s))
    sb = np.logspace(np.log10(0.3), np.log10(20), 16)
    mu = np.linspace(0, 1, 11)
    per = L if pbc else None
    c0, w0 = oracle.weighted_npairs_s_mu(s, s, w, w, sb, mu, period=per, num_threads=8)
    c, wc = gpu.weighted_npairs_s_mu(s, s, w, w, sb, mu, period=per)
    assert c.dtype == np.int64 and wc.dtype == np.float64
    assert np.array_equal(c, c0)
    assert np.array_equal(c, gpu.npairs_s_mu(s, s, sb, mu, period=per))
    _close(wc, w0)


def test_weighted_s_mu_cross_and_unit_weights(gpu):
    rng = np.random.default_rng(41)
    L = 180.0
    s1 = clustered(rng, 20000, L, 900)
    s2 = rng.uniform(0, L, (12000, 3))
    w1, w2 = rng.uniform(0, 1, len(s1)), rng.uniform(0.5, 3, len(s2))
    sb = np.logspace(-1, np.log10(15), 12)
    mu = np.linspace(0, 1, 21)
    c0, w0 = oracle.weighted_npairs_s_mu(s1, s2, w1, w2, sb, mu, period=L, num_threads=8)
    c, wc = gpu.weighted_npairs_s_mu(s1, s2, w1, w2, sb, mu, period=L)
    assert np.array_equal(c, c0)
    _close(wc, w0)
    c1, wc1 = gpu.weighted_npairs_s_mu(s1, s2, np.ones(len(s1)), np.ones(len(s2)), sb, mu,
                                       period=L)
    assert np.array_equal(wc1, c1.astype(np.float64))


def test_weighted_2d_large_sample_many_moves(gpu):
    # ~2e8 pairs in each call: every warp moves its (hi, lo) sums to FP64 many times
    rng = np.random.default_rng(42)
    L = 500.0
    s = clustered(rng, 400000, L, 8000)
    w = rng.uniform(0.1, 1.0, len(s))
    sb = np.logspace(np.log10(0.5), np.log10(25), 12)
    mu = np.linspace(0, 1, 6)
    c0, w0 = oracle.weighted_npairs_s_mu(s, s, w, w, sb, mu, period=L, num_threads=16)
    c, wc = gpu.weighted_npairs_s_mu(s, s, w, w, sb, mu, period=L)
    assert np.array_equal(c, c0)
    _close(wc, w0)
    rp, pi = np.logspace(np.log10(0.5), np.log10(25), 12), np.linspace(0, 30, 7)
    _close(gpu.marked_npairs_xy_z(s, s, rp, pi, period=L, weights1=w, weights2=w, weight_func_id=1),
           oracle.marked_npairs_xy_z(s, s, rp, pi, 1, period=L, weights1=w, weights2=w,
                                     num_threads=16))
    # unit weights must still reproduce the counts exactly
    cf, wf = gpu.weighted_npairs_s_mu(s, s, np.ones(len(s)), np.ones(len(s)), sb, mu, period=L)
    assert np.array_equal(wf, cf.astype(np.float64))


def test_weighted_2d_empty_and_errors(gpu):
    rng = np.random.default_rng(43)
    s = rng.uniform(0, 100, (500, 3))
    rp, pi = np.logspace(-1, 1, 5), np.linspace(0, 10, 4)
    empty = np.zeros((0, 3))
    assert np.array_equal(gpu.marked_npairs_xy_z(empty, s, rp, pi, period=100, weight_func_id=1,
                                                 weights1=np.zeros(0)), np.zeros((5, 4)))
    c, w = gpu.weighted_npairs_s_mu(s, empty, np.ones(500), np.zeros(0), rp, np.linspace(0, 1, 3),
                                    period=100)
    assert not c.any() and not w.any()
    with pytest.raises(gpu.HalotoolsError):
        gpu.marked_npairs_xy_z(s, s, rp, pi, period=100, weight_func_id=16,
                               weights1=np.ones((500, 5)), weights2=np.ones((500, 5)))
    with pytest.raises(AssertionError):
        gpu.weighted_npairs_s_mu(s, s, np.ones(499), np.ones(500), rp, np.linspace(0, 1, 3))


# ---------------- npairs_jackknife_xy_z ----------------
def _cuboid_tags(s, L, n=3):
    c = np.minimum((s / (L / n)).astype(int), n - 1)
    return 1 + c[:, 0] * n * n + c[:, 1] * n + c[:, 2]


@pytest.mark.parametrize("pbc", [True, False])
def test_jackknife_xy_z_matches_oracle(gpu, pbc):
    rng = np.random.default_rng(50)
    L = 300.0
    s = clustered(rng, 30000, L, 1500)
    t = _cuboid_tags(s, L)
    rp = np.logspace(-1, np.log10(20), 12)
    pi = np.linspace(0, 25, 11)
    per = L if pbc else None
    want = oracle.npairs_jackknife_xy_z(s, s, rp, pi, t, t, 27, period=per, num_threads=8)
    got = gpu.npairs_jackknife_xy_z(s, s, rp, pi, t, t, 27, period=per)
    assert got.shape == (28, 12, 11)
    assert np.array_equal(got, want)
    assert np.array_equal(got[0], gpu.npairs_xy_z(s, s, rp, pi, period=per).astype(np.float64))


def test_jackknife_xy_z_cross_and_blocks(gpu):
    rng = np.random.default_rng(51)
    L = 250.0
    s1 = clustered(rng, 20000, L, 1000)
    s2 = rng.uniform(0, L, (15000, 3))
    t1, t2 = _cuboid_tags(s1, L), _cuboid_tags(s2, L)
    rp = np.logspace(-1, np.log10(15), 10)
    pi = np.linspace(0, 20, 21)
    want = oracle.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L), want)
    with forced(gpu, 2) as plan:
        got = gpu.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L)
        assert plan.stats()["block"] == 2
    assert np.array_equal(got, want)


# ---------------- weighted jackknife (3-D and (rp, pi)) ----------------
@pytest.mark.parametrize("pbc", [True, False])
def test_weighted_jackknife_3d_matches_oracle(gpu, pbc):
    rng = np.random.default_rng(90)
    L = 300.0
    s = clustered(rng, 30000, L, 1500)
    t = _cuboid_tags(s, L)
    w = rng.uniform(0.2, 2.0, len(s))
    rb = np.logspace(-1, np.log10(20), 12)
    per = L if pbc else None
    want = oracle.npairs_jackknife_3d(s, s, rb, t, t, 27, period=per, weights1=w, weights2=w,
                                      num_threads=8)
    got = gpu.npairs_jackknife_3d(s, s, rb, t, t, 27, period=per, weights1=w, weights2=w)
    assert got.shape == (28, 12)
    _close(got, want)


def test_weighted_jackknife_cross_and_integer_weights(gpu):
    rng = np.random.default_rng(91)
    L = 250.0
    s1 = clustered(rng, 20000, L, 1000)
    s2 = rng.uniform(0, L, (15000, 3))
    t1, t2 = _cuboid_tags(s1, L), _cuboid_tags(s2, L)
    w1, w2 = rng.uniform(0.2, 2.0, len(s1)), rng.uniform(0.2, 2.0, len(s2))
    rb = np.logspace(-1, np.log10(15), 10)
    rp, pi = np.logspace(-1, np.log10(15), 10), np.linspace(0, 20, 11)
    _close(gpu.npairs_jackknife_3d(s1, s2, rb, t1, t2, 27, period=L, weights1=w1, weights2=w2),
           oracle.npairs_jackknife_3d(s1, s2, rb, t1, t2, 27, period=L, weights1=w1,
                                      weights2=w2, num_threads=8))
    _close(gpu.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L, weights1=w1,
                                     weights2=w2),
           oracle.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L, weights1=w1,
                                        weights2=w2, num_threads=8))
    # weights of 2: every product is 4, so the weighted rows are exactly 4x the counts
    two1, two2 = np.full(len(s1), 2.0), np.full(len(s2), 2.0)
    assert np.array_equal(
        gpu.npairs_jackknife_3d(s1, s1, rb, t1, t1, 27, period=L, weights1=two1, weights2=two1),
        4.0 * gpu.npairs_jackknife_3d(s1, s1, rb, t1, t1, 27, period=L))
    assert np.array_equal(
        gpu.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L, weights1=two1,
                                  weights2=two2),
        4.0 * gpu.npairs_jackknife_xy_z(s1, s2, rp, pi, t1, t2, 27, period=L))


def test_weighted_jackknife_xy_z_auto_matches_oracle(gpu):
    rng = np.random.default_rng(92)
    L = 300.0
    s = clustered(rng, 25000, L, 1200)
    t = _cuboid_tags(s, L)
    w = rng.lognormal(0.0, 0.5, len(s))
    rp, pi = np.logspace(-1, np.log10(20), 12), np.linspace(0, 25, 11)
    _close(gpu.npairs_jackknife_xy_z(s, s, rp, pi, t, t, 27, period=L, weights1=w, weights2=w),
           oracle.npairs_jackknife_xy_z(s, s, rp, pi, t, t, 27, period=L, weights1=w,
                                        weights2=w, num_threads=8))
