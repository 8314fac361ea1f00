"""Zheng07 mocks drawn by the GPU kernels (gbp_hod_mocks): exact where the draws
are forced, statistical where they are random (the reference draws with numpy's
generators, which a counter-based GPU stream does not reproduce), and the
batched counter fed by them without a host round trip."""
import numpy as np
import pytest

from halotools_gb300 import mocks
from oracle import oracle

pytestmark = pytest.mark.gpu

L = 500.0


def _grid_halos(n_side, mass, conc, rvir):
    g = (np.arange(n_side) + 0.5) * (L / n_side)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    n = len(pos)
    return pos, np.full(n, mass), np.full(n, conc), np.full(n, rvir)


def test_deterministic_and_seeded(gpu):
    pos, mass, conc = mocks.halo_table(200000, L, seed=3)
    th = np.array([[12.0, 0.3, 12.0, 13.3, 1.0], [12.5, 0.5, 12.2, 13.0, 0.8]])
    a, oa = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=11)
    b, ob = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=11)
    c, oc = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=12)
    assert np.array_equal(oa, ob) and bool((a == b).all())
    assert not (np.array_equal(oa, oc) and bool((a == c).all()))
    x = a.cpu().numpy()
    assert x.dtype == np.float32 and np.all(x >= 0) and np.all(x < L)


def test_forced_centrals_are_the_halos(gpu):
    # <Ncen> = 1 (logMmin far below), no satellites (M0 above every halo)
    pos, mass, conc = mocks.halo_table(50000, L, seed=4)
    th = np.array([[5.0, 0.1, 20.0, 21.0, 1.0]] * 3)
    x, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=1)
    assert list(offs) == [0, 50000, 100000, 150000]
    got = x.cpu().numpy()
    for m in range(3):
        assert np.array_equal(got[offs[m]:offs[m + 1]], pos.astype(np.float32))


@pytest.mark.parametrize("lam", [3.0, 40.0])
def test_satellite_counts_are_poisson(gpu, lam):
    # no centrals; <Nsat> = lam for every halo: ((M - M0) / M1)^1 with M - M0 = lam M1
    pos, mass, conc, rvir = _grid_halos(24, 1e14, 6.0, 0.5)
    logM1 = 12.0
    M0 = 1e14 - lam * 10 ** logM1
    th = np.array([[30.0, 0.1, np.log10(M0), logM1, 1.0]])
    x, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=5, rvir=rvir)
    g = x.cpu().numpy().astype(np.float64)
    # assign each satellite to its halo (halos L/24 apart, satellites within 0.5)
    cell = np.floor(g / (L / 24)).astype(int).clip(0, 23)
    idx = (cell[:, 0] * 24 + cell[:, 1]) * 24 + cell[:, 2]
    k = np.bincount(idx, minlength=len(pos))
    n = len(k)
    assert abs(k.mean() - lam) < 5 * np.sqrt(lam / n)
    assert abs(k.var() - lam) < 6 * lam * np.sqrt(2.0 / n)


def test_satellite_radii_follow_nfw_and_are_isotropic(gpu):
    c, rv = 7.0, 1.0
    pos = np.array([[L / 2, L / 2, L / 2]])
    th = np.array([[30.0, 0.1, 13.0, 10.0, 1.0]])  # <Nsat> = (1e14 - 1e13) / 1e10 = 9000
    x, offs = mocks.hod_mocks_gpu(pos, np.array([1e14]), np.array([c]), L, th, seed=6,
                                  rvir=np.array([rv]))
    d = x.cpu().numpy().astype(np.float64) - pos
    r = np.linalg.norm(d, axis=1)
    n = len(r)
    assert 8500 < n < 9500
    assert np.all(r <= rv + 1e-4)  # (float32 positions near 250: ulp 1.5e-5)

    def m(t):
        return np.log1p(t) - t / (1 + t)
    rs = np.sort(r / rv)
    cdf = m(rs * c) / m(c)
    ks = np.max(np.abs(cdf - (np.arange(1, n + 1) / n)))
    assert ks < 1.63 * 1.5 / np.sqrt(n)
    u = d / r[:, None]
    assert np.all(np.abs(u.mean(axis=0)) < 5 / np.sqrt(3 * n))


def test_mock_sizes_match_zheng07_means(gpu):
    pos, mass, conc = mocks.halo_table(300000, L, seed=7)
    th = np.array([[12.0, 0.3, 12.0, 13.3, 1.0], [11.5, 0.2, 11.8, 12.9, 1.1],
                   [13.0, 0.6, 12.5, 13.8, 0.7]])
    _, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=8)
    for m, t in enumerate(th):
        nc = mocks.zheng07_mean_ncen(np.log10(mass), t[0], t[1])
        ns = mocks.zheng07_mean_nsat(mass, t[2], t[3], t[4])
        mean, var = nc.sum() + ns.sum(), (nc * (1 - nc)).sum() + ns.sum()
        assert abs((offs[m + 1] - offs[m]) - mean) < 5 * np.sqrt(var), m


def test_batched_counter_on_gpu_mocks(gpu):
    pos, mass, conc = mocks.halo_table(100000, L, seed=9)
    th = np.array([[12.0, 0.3, 12.0, 13.3, 1.0], [11.8, 0.4, 12.1, 13.1, 0.9]])
    x, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=10)
    rb = np.logspace(-1, np.log10(20), 15)
    bc = gpu.BatchedCounter(graph=False, autotune=False)
    got = bc.count_device(x, offs, rb, L) if hasattr(bc, "count_device") else \
        bc([x[offs[m]:offs[m + 1]] for m in range(len(th))], rb, L)
    xs = x.cpu().numpy().astype(np.float64)
    for m in range(len(th)):
        s = xs[offs[m]:offs[m + 1]]
        assert np.array_equal(got[m], oracle.npairs_3d(s, s, rb, period=L, num_threads=8))


def test_offsets_only_and_errors(gpu):
    from halotools_gb300 import _native as N
    plan = N.default_plan()
    pos, mass, conc = mocks.halo_table(1000, L, seed=2)
    rvir = (mass / 1e14) ** (1 / 3)
    th = np.array([[12.0, 0.3, 12.0, 13.3, 1.0]])
    offs = np.zeros(2, dtype=np.int64)
    plan.check(plan.lib.gbp_hod_mocks(plan.handle, N.dptr(pos), N.dptr(mass), N.dptr(conc),
                                      N.dptr(rvir), len(mass), N.pd(th), 1, L, 3,
                                      N.GBP_MEM_HOST, None, 0, N.pi64(offs)))
    assert offs[0] == 0 and offs[1] > 0
    gal = np.zeros((int(offs[1]), 3), dtype=np.float32)
    plan.check(plan.lib.gbp_hod_mocks(plan.handle, N.dptr(pos), N.dptr(mass), N.dptr(conc),
                                      N.dptr(rvir), len(mass), N.pd(th), 1, L, 3,
                                      N.GBP_MEM_HOST, N.dptr(gal), len(gal), N.pi64(offs)))
    xd, od = mocks.hod_mocks_gpu(pos, mass, conc, L, th, seed=3)
    assert np.array_equal(od, offs) and np.array_equal(xd.cpu().numpy(), gal)
    bad = np.array([[12.0, 0.0, 12.0, 13.3, 1.0]])
    rc = plan.lib.gbp_hod_mocks(plan.handle, N.dptr(pos), N.dptr(mass), N.dptr(conc),
                                N.dptr(rvir), len(mass), N.pd(bad), 1, L, 3, N.GBP_MEM_HOST,
                                None, 0, N.pi64(offs))
    assert rc != 0
