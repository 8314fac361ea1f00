"""The seeded synthetic catalogues that stand in for the benchmark workloads
(CPU generators in halotools_gb300/mocks.py): shapes, bounds, determinism and
the distributions they follow (halotools' NFW enclosed mass, mass_profile.py:31;
Zheng07 mean occupations, zheng07_components.py:149-153, 455-470)."""
import math

import numpy as np

from halotools_gb300 import mocks


def test_clustered_points_shape_bounds_and_seed():
    a = mocks.clustered_points(20000, 100.0, 800, seed=3)
    b = mocks.clustered_points(20000, 100.0, 800, seed=3)
    c = mocks.clustered_points(20000, 100.0, 800, seed=4)
    assert a.shape == (20000, 3) and a.dtype == np.float64
    assert np.all(a >= 0.0) and np.all(a < 100.0)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)


def test_clustered_points_are_clustered():
    # satellites sit within a virial radius of their centre (z smeared by the
    # 5 Mpc/h displacement): many more close pairs than a uniform sample
    from scipy.spatial import cKDTree
    x = mocks.clustered_points(20000, 100.0, 2000, seed=5)
    u = np.random.default_rng(5).uniform(0, 100.0, (20000, 3))

    def close(p):  # ordered pairs within 1, self pairs left out
        t = cKDTree(p, boxsize=100.0)
        return t.count_neighbors(t, 1.0) - len(p)
    assert close(x) > 5 * close(u)


def test_nfw_radii_follow_the_enclosed_mass_profile():
    from scipy import stats
    rng = np.random.default_rng(6)
    conc, rvir = 8.0, 2.0
    r = mocks.nfw_radii(rng, np.full(20000, conc), np.full(20000, rvir))
    assert np.all(r > 0.0) and np.all(r <= rvir)
    m = lambda x: np.log1p(x) - x / (1.0 + x)
    cdf = lambda s: m(conc * np.clip(s, 0.0, rvir) / rvir) / m(conc)
    assert stats.kstest(r, cdf).pvalue > 1e-3


def test_halo_table_mass_function_and_concentration():
    pos, mass, conc = mocks.halo_table(400000, 500.0, seed=7)
    assert pos.shape == (400000, 3) and np.all((pos >= 0) & (pos < 500.0))
    logm = np.log10(mass)
    assert logm.min() >= 11.0 and logm.max() <= 15.0
    # dN/dlog10M ~ M^-0.9: counts per dex fall by 10^-0.9 per dex
    h, e = np.histogram(logm, bins=np.linspace(11.0, 15.0, 9))
    slope = np.polyfit(0.5 * (e[1:] + e[:-1]), np.log10(h), 1)[0]
    assert abs(slope + 0.9) < 0.03, slope
    np.testing.assert_allclose(conc, 10.0 * (mass / 1e12) ** -0.1, rtol=1e-12)


def test_zheng07_mean_occupations():
    logm = np.array([11.5, 12.0, 12.5])
    np.testing.assert_allclose(mocks.zheng07_mean_ncen(logm, 12.0, 0.3)[1], 0.5)
    assert np.all(np.diff(mocks.zheng07_mean_ncen(logm, 12.0, 0.3)) > 0)
    m0, m1 = 10.0 ** 12.0, 10.0 ** 13.3
    mass = np.array([0.5 * m0, m0, m0 + m1, m0 + 4 * m1])
    np.testing.assert_allclose(mocks.zheng07_mean_nsat(mass, 12.0, 13.3, 1.0),
                               [0.0, 0.0, 1.0, 4.0])
    np.testing.assert_allclose(mocks.zheng07_mean_nsat(mass, 12.0, 13.3, 0.5)[3], 2.0)


def test_hod_mock_galaxy_count_matches_the_occupations():
    pos, mass, conc = mocks.halo_table(200000, 300.0, seed=8)
    theta = (12.0, 0.3, 12.0, 13.3, 1.0)
    pc = mocks.zheng07_mean_ncen(np.log10(mass), theta[0], theta[1])
    ns = mocks.zheng07_mean_nsat(mass, theta[2], theta[3], theta[4])
    mean = pc.sum() + ns.sum()
    sd = math.sqrt((pc * (1 - pc)).sum() + ns.sum())
    g = mocks.hod_mock(pos, mass, conc, 300.0, theta, seed=9)
    assert g.shape[1] == 3 and np.all((g >= 0) & (g < 300.0))
    assert abs(len(g) - mean) < 5 * sd, (len(g), mean, sd)
