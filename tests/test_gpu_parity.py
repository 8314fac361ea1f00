"""CUDA engines against the reference's golden vectors and the C oracle.

Integer counts must be bit-exact.  Run on a GB300 with ``pytest -m gpu``.
"""
import numpy as np
import pytest

from oracle import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu

INT_CASES = [n for n in G.names() if not n.startswith("marked")]


@pytest.mark.parametrize("name", INT_CASES)
def test_golden_exact(gpu, name):
    c = G.load(name)
    if c is None:
        pytest.skip("seeded generator differs on this platform")
    got = G.call(gpu, c)
    assert got.dtype == np.int64
    assert np.array_equal(got, c["out"]), (name, got, c["out"])


def clustered(rng, n, L, ncen, mlo=11.0, mhi=15.0):
    """Centres + NFW-like satellites + uniform fill, z displaced (RSD)."""
    cen = rng.uniform(0, L, (ncen, 3))
    m = 10 ** rng.uniform(mlo, mhi, ncen)
    nsat = rng.poisson((m / 1e12) ** 0.9)
    tot = min(int(nsat.sum()), n - ncen)
    host = np.repeat(np.arange(ncen), nsat)[:tot]
    rvir = (m[host] / 1e14) ** (1 / 3.0)
    r = rvir * rng.uniform(0, 1, tot) ** 1.5
    d = rng.normal(size=(tot, 3))
    d *= (r / np.linalg.norm(d, axis=1))[:, None]
    sat = cen[host] + d
    fill = rng.uniform(0, L, (n - ncen - tot, 3))
    pts = np.concatenate([cen, sat, fill])
    pts[:, 2] += rng.normal(0, 5.0, len(pts))
    return np.mod(pts, L)


@pytest.mark.parametrize("reach", [1, 2, 3])
def test_npairs_3d_matches_oracle_any_grid(gpu, reach):
    rng = np.random.default_rng(11)
    L = 300.0
    s = clustered(rng, 60000, L, 3000)
    rb = np.logspace(-1, np.log10(25), 20)
    want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)
    plan = gpu.default_plan()
    plan.set_reach(reach)
    try:
        got = gpu.npairs_3d(s, s, rb, period=L)
        assert plan.stats()["reach"] == reach
    finally:
        plan.set_reach(0)
    assert np.array_equal(got, want)


def test_npairs_3d_cross_nonperiodic_matches_oracle(gpu):
    rng = np.random.default_rng(12)
    s1 = rng.uniform(-50, 150, (40000, 3))
    s2 = rng.uniform(0, 120, (30000, 3))
    rb = np.logspace(-1, np.log10(15), 12)
    assert np.array_equal(gpu.npairs_3d(s1, s2, rb), oracle.npairs_3d(s1, s2, rb, num_threads=8))


def test_npairs_xy_z_matches_oracle(gpu):
    rng = np.random.default_rng(13)
    L = 400.0
    s = clustered(rng, 50000, L, 2500)
    rp = np.logspace(-1, np.log10(30), 20)
    pi = np.linspace(0, 40, 40)
    want = oracle.npairs_xy_z(s, s, rp, pi, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_xy_z(s, s, rp, pi, period=L), want)


def test_npairs_s_mu_matches_oracle(gpu):
    rng = np.random.default_rng(14)
    L = 400.0
    s = clustered(rng, 50000, L, 2500)
    sb = np.logspace(np.log10(0.5), np.log10(40), 30)
    mu = np.linspace(0, 1, 20)
    want = oracle.npairs_s_mu(s, s, sb, mu, period=L, num_threads=8)
    assert np.array_equal(gpu.npairs_s_mu(s, s, sb, mu, period=L), want)


def test_s_mu_last_column_equals_npairs_3d(gpu):
    # size-independent identity (test_npairs_s_mu.py:63-97): summing over mu
    rng = np.random.default_rng(15)
    L = 1000.0
    s = clustered(rng, 400000, L, 20000)
    sb = np.logspace(np.log10(0.5), np.log10(50), 30)
    a = gpu.npairs_s_mu(s, s, sb, np.linspace(0, 1, 20), period=L)
    b = gpu.npairs_3d(s, s, sb, period=L)
    assert np.array_equal(a[:, -1], b)


def test_auto_equals_cross_of_a_copy(gpu):
    rng = np.random.default_rng(16)
    s = rng.uniform(0, 200, (80000, 3))
    rb = np.logspace(-1, np.log10(20), 15)
    a = gpu.npairs_3d(s, s, rb, period=200.0)
    # a perturbed copy is not detected as identical, so this runs the cross path
    t = s.copy()
    t[0, 0] = np.nextafter(t[0, 0], 0.0)
    b = gpu.npairs_3d(s, t, rb, period=200.0)
    c = oracle.npairs_3d(s, t, rb, period=200.0, num_threads=8)
    assert np.array_equal(b, c)
    assert abs(int(a[-1]) - int(b[-1])) <= 2 * 1000


def test_repeat_runs_identical(gpu):
    rng = np.random.default_rng(17)
    s = clustered(rng, 100000, 500.0, 5000)
    rb = np.logspace(-1, np.log10(30), 20)
    a = gpu.npairs_3d(s, s, rb, period=500.0)
    b = gpu.npairs_3d(s, s, rb, period=500.0)
    assert np.array_equal(a, b)


def test_empty_and_single_point_samples(gpu):
    rb = np.array([0.1, 0.5])
    e = np.zeros((0, 3))
    one = np.array([[0.5, 0.5, 0.5]])
    assert np.array_equal(gpu.npairs_3d(e, one, rb, period=2.0), [0, 0])
    assert np.array_equal(gpu.npairs_3d(one, one, rb, period=2.0), [1, 1])
    assert np.array_equal(gpu.npairs_xy_z(one, e, rb, rb, period=2.0), np.zeros((2, 2)))


def test_points_on_box_faces(gpu):
    # coordinates exactly 0 and exactly L are legal and wrap
    pts = np.array([[0.0, 0.0, 0.0], [10.0, 10.0, 10.0], [10.0, 0.0, 5.0], [0.0, 10.0, 9.5]])
    rb = np.array([0.1, 0.6, 1.0, 3.0])
    want = oracle.npairs_3d(pts, pts, rb, period=10.0)
    assert np.array_equal(gpu.npairs_3d(pts, pts, rb, period=10.0), want)


def test_recheck_happens_and_counts_stay_exact(gpu):
    c = G.load("3d_ties0")
    got = gpu.npairs_3d(c["s1"], c["s2"], c["bins"], period=c["period"])
    assert gpu.default_plan().stats()["recheck_pairs"] >= len(c["bins"])
    assert np.array_equal(got, c["out"])


def test_wide_histogram_npairs_3d(gpu):
    # more edges than the lane-private histogram holds: shared-atomic variant
    rng = np.random.default_rng(18)
    s = rng.uniform(0, 100, (30000, 3))
    rb = np.linspace(0.05, 12.0, 150)
    assert np.array_equal(gpu.npairs_3d(s, s, rb, period=100.0),
                          oracle.npairs_3d(s, s, rb, period=100.0, num_threads=8))


def test_wide_2d_histogram_single_copy(gpu):
    rng = np.random.default_rng(19)
    s = rng.uniform(0, 100, (20000, 3))
    rp = np.linspace(0.1, 10.0, 60)
    pi = np.linspace(0.0, 12.0, 90)
    assert np.array_equal(gpu.npairs_xy_z(s, s, rp, pi, period=100.0),
                          oracle.npairs_xy_z(s, s, rp, pi, period=100.0, num_threads=8))


def test_out_of_box_and_nonfinite_positions_rejected(gpu):
    # the device digitiser flags them; the call raises instead of miscounting
    s = np.random.default_rng(20).uniform(0, 1, (500, 3))
    bad = s.copy()
    bad[0, 0] = 1.5
    with pytest.raises(ValueError):
        gpu.npairs_3d(bad, s, [0.1, 0.2], period=1)
    bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        gpu.npairs_3d(bad, s, [0.1, 0.2], period=1)
    with pytest.raises(ValueError):
        gpu.npairs_3d(bad, s, [0.1, 0.2])
    # the plan stays usable after a rejected call
    assert gpu.npairs_3d(s, s, [0.1, 0.2], period=1)[-1] >= 500


MARKED_CASES = G.names("marked")


@pytest.mark.parametrize("name", MARKED_CASES)
def test_marked_golden(gpu, name):
    # FP32 compensated sums: within 1e-6 relative of the reference's FP64 sums
    c = G.load(name)
    got = G.call(gpu, c)
    assert got.dtype == np.float64
    np.testing.assert_allclose(got, c["out"], rtol=1e-6, atol=1e-9)


def test_marked_product_clustered_matches_oracle(gpu):
    rng = np.random.default_rng(21)
    L = 400.0
    s = clustered(rng, 60000, L, 3000)
    w = rng.lognormal(0.0, 0.5, len(s))
    rb = np.logspace(np.log10(0.5), np.log10(40), 30)
    want = oracle.marked_npairs_3d(s, s, rb, 1, period=L, weights1=w, weights2=w, num_threads=8)
    got = gpu.marked_npairs_3d(s, s, rb, 1, period=L, weights1=w, weights2=w)
    np.testing.assert_allclose(got, want, rtol=1e-6)
    # the unweighted count with unit marks is exact
    ones = gpu.marked_npairs_3d(s, s, rb, 1, period=L)
    assert np.array_equal(ones, gpu.npairs_3d(s, s, rb, period=L).astype(np.float64))


# ---------------- batched mocks ----------------
def _mocks(seed, sizes, L):
    rng = np.random.default_rng(seed)
    return [clustered(rng, n, L, max(n // 20, 10)) if n >= 1000 else rng.uniform(0, L, (n, 3))
            for n in sizes]


@pytest.mark.parametrize("graph", [False, True])
def test_batched_equals_per_mock_counts(gpu, graph):
    L = 300.0
    mocks = _mocks(31, [20000, 0, 35000, 5000, 1, 27000], L)
    rb = np.logspace(-1, np.log10(20), 15)
    bc = gpu.BatchedCounter(graph=graph, autotune=False)
    got = bc(mocks, rb, L)
    got2 = bc(mocks, rb, L)  # second call: graph replayed / updated
    for m, s in enumerate(mocks):
        want = gpu.npairs_3d(s, s, rb, period=L) if len(s) else np.zeros(len(rb), np.int64)
        assert np.array_equal(got[m], want), m
    assert np.array_equal(got, got2)


def test_batched_float32_autotuned_matches_oracle(gpu):
    L = 250.0
    mocks = [m.astype(np.float32) for m in _mocks(32, [30000, 18000, 25000], L)]
    rb = np.logspace(-1, np.log10(15), 12)
    bc = gpu.BatchedCounter(graph=True, autotune=True)
    got = bc(mocks, rb, L)
    got_again = bc(mocks, rb, L)
    for m, s in enumerate(mocks):
        want = oracle.npairs_3d(s, s, rb, period=L, num_threads=8)  # exact FP64 upcast
        assert np.array_equal(got[m], want), m
    assert np.array_equal(got, got_again)


def test_batched_device_tensor_input(gpu):
    import torch
    L = 200.0
    mocks = _mocks(33, [15000, 22000], L)
    xyz = np.concatenate(mocks)
    offs = np.array([0, 15000, 37000])
    rb = np.logspace(-1, np.log10(12), 10)
    bc = gpu.BatchedCounter()
    got = bc.count_device(torch.from_numpy(xyz).cuda(), offs, rb, L)
    for m, s in enumerate(mocks):
        assert np.array_equal(got[m], gpu.npairs_3d(s, s, rb, period=L))
