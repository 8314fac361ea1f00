"""counts_in_cylinders and the isolation functions on the GPU against the C
oracle (a restatement of counts_in_cylinders_engine.pyx and the isolation
engines, pinned to halotools' engines in test_oracle.py); everything exact."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_blocks import forced
from tests.test_gpu_parity import clustered

pytestmark = pytest.mark.gpu


def _sample(seed, n, L, ncen):
    rng = np.random.default_rng(seed)
    return rng, clustered(rng, n, L, ncen)


@pytest.mark.parametrize("pbc", [True, False])
def test_counts_in_cylinders_matches_oracle(gpu, pbc):
    rng, s1 = _sample(80, 40000, 300.0, 2000)
    s2 = rng.uniform(0, 300.0, (25000, 3))
    rp = rng.uniform(0.2, 6.0, len(s1))
    pi = rng.uniform(0.5, 12.0, len(s1))
    per = 300.0 if pbc else None
    assert np.array_equal(gpu.counts_in_cylinders(s1, s2, rp, pi, period=per),
                          oracle.counts_in_cylinders(s1, s2, rp, pi, period=per, num_threads=8))
    # auto-correlation (sample2 None): a point does not count itself
    got = gpu.counts_in_cylinders(s1, None, rp, pi, period=per)
    assert got.dtype == np.int64
    assert np.array_equal(got, oracle.counts_in_cylinders(s1, None, rp, pi, period=per,
                                                          num_threads=8))


def test_counts_in_cylinders_mass_frac_blocks_and_zero_radii(gpu):
    rng, s1 = _sample(81, 30000, 250.0, 1500)
    rp = rng.uniform(0.0, 5.0, len(s1))
    rp[::7] = 0.0  # a zero cylinder holds nothing: -1 in the auto-correlation, as there
    pi = rng.uniform(0.0, 10.0, len(s1))
    m = 10 ** rng.uniform(10, 14, len(s1))
    for eq in [(True, False), (False, True)]:
        args = (m, m, (0.2, 3.0)) + eq
        want = oracle.counts_in_cylinders(s1, None, rp, pi, period=250.0, condition="mass_frac",
                                          condition_args=args, num_threads=8)
        got = gpu.counts_in_cylinders(s1, None, rp, pi, period=250.0, condition="mass_frac",
                                      condition_args=args)
        assert np.array_equal(got, want)
    want = oracle.counts_in_cylinders(s1, s1, rp, pi, period=250.0, num_threads=8)
    with forced(gpu, 2) as plan:
        got = gpu.counts_in_cylinders(s1, s1, rp, pi, period=250.0)
        assert plan.stats()["block"] == 2
    assert np.array_equal(got, want)
    assert np.all(gpu.counts_in_cylinders(s1, None, rp, pi, period=250.0)[::7] == -1)


def _brute_pairs(s1, s2, rp, pi, L):
    d = s1[:, None, :] - s2[None, :, :]
    if L is not None:
        d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
    inside = (d[..., 0] ** 2 + d[..., 1] ** 2 < rp[:, None] ** 2) & (d[..., 2] ** 2 < pi[:, None] ** 2)
    i1, i2 = np.nonzero(inside)
    return inside.sum(axis=1), np.stack([i1, i2], axis=1)


@pytest.mark.parametrize("auto", [False, True])
def test_counts_in_cylinders_indexes(gpu, auto):
    rng = np.random.default_rng(82)
    L = 60.0
    s1 = rng.uniform(0, L, (1500, 3))
    s2 = s1 if auto else rng.uniform(0, L, (1200, 3))
    rp = rng.uniform(0.5, 4.0, len(s1))
    pi = rng.uniform(1.0, 6.0, len(s1))
    counts, idx = gpu.counts_in_cylinders(s1, None if auto else s2, rp, pi, period=L,
                                          return_indexes=True)
    bc, bp = _brute_pairs(s1, s2, rp, pi, L)
    if auto:
        bc = bc - 1
        bp = bp[bp[:, 0] != bp[:, 1]]
    assert np.array_equal(counts, bc)
    assert idx.dtype.names == ("i1", "i2") and idx["i1"].dtype == np.uint32
    got = np.sort(idx, order=["i1", "i2"])
    assert np.array_equal(np.stack([got["i1"], got["i2"]], axis=1).astype(np.int64), bp)


@pytest.mark.parametrize("geo", ["sphere", "cylinder"])
@pytest.mark.parametrize("pbc", [True, False])
def test_isolation_matches_oracle(gpu, geo, pbc):
    rng, s1 = _sample(83, 30000, 300.0, 1500)
    s2 = clustered(rng, 20000, 300.0, 1000)
    r = rng.uniform(0.3, 6.0, len(s1))
    pi = rng.uniform(0.5, 10.0, len(s1))
    per = 300.0 if pbc else None
    if geo == "sphere":
        got = gpu.spherical_isolation(s1, s2, r, period=per)
        auto = gpu.spherical_isolation(s1, s1, r, period=per)
        want = oracle.isolation(s1, s2, r, None, period=per, num_threads=8)
        wauto = oracle.isolation(s1, s1, r, None, period=per, num_threads=8)
    else:
        got = gpu.cylindrical_isolation(s1, s2, r, pi, period=per)
        auto = gpu.cylindrical_isolation(s1, s1, r, pi, period=per)
        want = oracle.isolation(s1, s2, r, pi, period=per, num_threads=8)
        wauto = oracle.isolation(s1, s1, r, pi, period=per, num_threads=8)
    assert got.dtype == bool and np.array_equal(got, want)
    assert np.array_equal(auto, wauto)
    assert 0 < got.sum() < len(s1)


def test_isolation_duplicates_are_not_neighbours(gpu):
    # points at exactly the same position have separation 0: never neighbours
    rng = np.random.default_rng(84)
    s = rng.uniform(0, 100.0, (3000, 3))
    s = np.concatenate([s, s[:500]])
    r = np.full(len(s), 0.5)
    got = gpu.spherical_isolation(s, s, r, period=100.0)
    assert np.array_equal(got, oracle.isolation(s, s, r, None, period=100.0))
    assert np.array_equal(gpu.cylindrical_isolation(s, s, r, r, period=100.0),
                          oracle.isolation(s, s, r, r, period=100.0))


@pytest.mark.parametrize("func", list(range(7)))
def test_conditional_isolation_every_function(gpu, func):
    rng, s1 = _sample(85 + func, 20000, 250.0, 1000)
    s2 = rng.uniform(0, 250.0, (15000, 3))
    nm = 2 if func >= 5 else 1
    m1 = rng.uniform(0, 3, (len(s1), nm))
    m2 = rng.uniform(0, 3, (len(s2), nm))
    if func in (3, 4):
        m1, m2 = np.floor(m1), np.floor(m2)  # equality tests need ties
    r = rng.uniform(0.5, 6.0, len(s1))
    pi = rng.uniform(1.0, 8.0, len(s1))
    assert np.array_equal(
        gpu.conditional_spherical_isolation(s1, s2, r, m1, m2, func, period=250.0),
        oracle.isolation(s1, s2, r, None, period=250.0, marks1=m1, marks2=m2, cond_func=func,
                         num_threads=8))
    assert np.array_equal(
        gpu.conditional_cylindrical_isolation(s1, s2, r, pi, m1, m2, func, period=250.0),
        oracle.isolation(s1, s2, r, pi, period=250.0, marks1=m1, marks2=m2, cond_func=func,
                         num_threads=8))


def test_neighbours_empty(gpu):
    s = np.random.default_rng(86).uniform(0, 50, (100, 3))
    e = np.zeros((0, 3))
    assert np.array_equal(gpu.counts_in_cylinders(s, e, 1.0, 1.0, period=50.0), np.zeros(100))
    assert gpu.spherical_isolation(s, e, 1.0, period=50.0).all()
    assert len(gpu.counts_in_cylinders(e, s, 1.0, 1.0, period=50.0)) == 0
