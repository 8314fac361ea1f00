"""The C oracle against the reference's golden vectors (CPU only)."""
import numpy as np
import pytest

from oracle import oracle
from tests import golden_cases as G


@pytest.mark.parametrize("name", G.names())
def test_oracle_matches_reference_golden(name):
    c = G.load(name)
    if c is None:
        pytest.skip("seeded generator differs on this platform")
    got = G.call(oracle, c)
    if c["kind"] == "marked":
        np.testing.assert_allclose(got, c["out"], rtol=1e-12, atol=1e-12)
    else:
        assert np.array_equal(got, c["out"]), (got, c["out"])


def test_tie_fixtures_pin_left_to_right_unfused_order():
    # every partner sits exactly on its own edge under ((dx*dx + dy*dy) + dz*dz)
    for name in G.names("3d_ties"):
        c = G.load(name)
        assert np.array_equal(c["out"], np.arange(1, len(c["bins"]) + 1))


@pytest.mark.parametrize("period", [None, 50.0])
def test_cell_walk_equals_brute_force(period):
    rng = np.random.default_rng(7)
    s1 = rng.uniform(0, 50, (700, 3))
    s2 = rng.uniform(0, 50, (600, 3))
    rb = np.logspace(-1, np.log10(12), 9)
    assert np.array_equal(oracle.npairs_3d(s1, s2, rb, period=period),
                          oracle.brute_force_npairs_3d(s1, s2, rb, period=period))


def test_threads_do_not_change_counts():
    rng = np.random.default_rng(8)
    s = rng.uniform(0, 100, (5000, 3))
    rb = np.logspace(-1, np.log10(20), 10)
    a = oracle.npairs_3d(s, s, rb, period=100.0, num_threads=1)
    b = oracle.npairs_3d(s, s, rb, period=100.0, num_threads=4)
    assert np.array_equal(a, b)


def test_oracle_planted_error_is_caught():
    # a mistake planted in the oracle's inputs (one partner nudged past its
    # edge) must change the count, so the tie fixtures are sensitive
    c = G.load("3d_ties0")
    s2 = c["s2"].copy()
    s2[0, 0] = np.nextafter(s2[0, 0], np.inf if s2[0, 0] < c["s1"][0, 0] else -np.inf) + 1e-9
    got = oracle.npairs_3d(c["s1"], s2, c["bins"], period=c["period"])
    assert not np.array_equal(got, c["out"])


def test_oracle_adjoint_matches_marked_identity():
    rng = np.random.default_rng(9)
    x = rng.uniform(0, 40, (1500, 3))
    w = rng.uniform(0, 1, 1500)
    rb = np.array([1.0, 3.0, 7.0])
    g = np.array([0.3, -1.0, 2.0])
    grad = oracle.weighted_adjoint_3d(x, w, rb, 40.0, g)
    for m in (0, 700, 1499):
        c = oracle.marked_npairs_3d(x[m:m + 1], x, rb, 1, period=40.0, weights1=np.ones(1),
                                    weights2=w)
        assert abs(grad[m] - 2 * np.dot(g, c)) < 1e-9 * max(1.0, abs(grad[m]))


# ---- the oracle's sibling walks against halotools' own engines ----
from tests.golden import make_sibling_golden as S  # noqa: E402

# (the oracle has no pair list: the index cases are checked on the GPU only)
_W2_CASES = sorted(n for n in S.CASES
                   if S.CASES[n][0] in ("marked_npairs_xy_z", "weighted_npairs_s_mu",
                                        "npairs_jackknife_xy_z", "npairs_jackknife_3d",
                                        "counts_in_cylinders",
                                        "spherical_isolation", "cylindrical_isolation",
                                        "conditional_spherical_isolation",
                                        "conditional_cylindrical_isolation")
                   and "indexes" not in n)


@pytest.mark.parametrize("name", _W2_CASES)
def test_oracle_weighted_2d_matches_reference_golden(name):
    import os
    d = np.load(os.path.join(S.OUT, name + ".npz"))
    if str(d["sha"]) != S.input_sha():
        pytest.skip("seeded generator differs on this platform")
    got = S.run_case(oracle, name)
    if isinstance(got, tuple):
        assert np.array_equal(got[0], d["out"])
        got, want = got[1], d["out_w"]
    else:
        want = d["out"]
    if want.dtype.kind in "biu":
        assert got.dtype.kind == want.dtype.kind and np.array_equal(got, want)
    else:
        # the reference engines are built with -Ofast: sums agree to a few ulps
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


def test_oracle_weighted_2d_unit_marks_give_counts():
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 60, (1500, 3))
    rp, pi = np.logspace(-1, 1, 6), np.linspace(0, 12, 5)
    cnt = oracle.npairs_xy_z(x, x, rp, pi, period=60)
    assert np.array_equal(oracle.marked_npairs_xy_z(x, x, rp, pi, 1, period=60), cnt.astype(float))
    sb, mu = np.logspace(-1, 1, 6), np.linspace(0, 1, 7)
    c, w = oracle.weighted_npairs_s_mu(x, x, np.ones(1500), np.ones(1500), sb, mu, period=60)
    assert np.array_equal(c, oracle.npairs_s_mu(x, x, sb, mu, period=60))
    assert np.array_equal(w, c.astype(float))
