"""The parity summaries and the FP64 Zheng07 Jacobian used by the full-size checks
(oracle/parity.py): exactness, per-bin relative errors, and the analytic
derivatives of the Zheng07 occupations against central differences."""
import numpy as np

from oracle import oracle, parity


def test_exact_and_relative_summaries():
    a = np.array([1, 2, 3, 10], dtype=np.int64)
    assert parity.exact(a, a.copy()) == {"exact": True, "bins": 4, "mismatched_bins": 0,
                                         "in_range_pairs": 10}
    b = a.copy()
    b[1] += 1
    assert parity.exact(b, a)["mismatched_bins"] == 1
    r = parity.rel_per_bin([1.0, 2.0, 0.5], [1.0, 2.0 + 2e-6, 0.0])
    assert r[0] == 0.0 and abs(r[1] - 1e-6) < 1e-11 and r[2] == 0.5
    s = parity.rel_summary([1.0, 2.0], [1.0, 2.0 * (1 + 5e-7)], 1e-6)
    assert s["ok"] and s["max_rel_err"] < 1e-6


def test_zheng07_jacobian_matches_central_differences():
    from halotools_gb300 import mocks
    _, mass, _ = mocks.halo_table(20000, 100.0, seed=7)
    th = np.array([12.1, 0.35, 11.9, 13.2, 1.05])
    J = parity.zheng07_jacobian_fp64(th, mass)
    h = 1e-6
    fd = np.stack([(parity.zheng07_fp64(th + h * e, mass) - parity.zheng07_fp64(th - h * e, mass))
                   / (2 * h) for e in np.eye(5)], axis=1)
    assert np.max(np.abs(J - fd)) < 1e-6 * max(1.0, np.abs(J).max())


def test_weighted_table_gives_marked_counts_and_adjoint():
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 80.0, (3000, 3))
    w = rng.uniform(0.5, 2.0, 3000)
    rb = np.logspace(-1, np.log10(12), 8)
    S = oracle.weighted_per_object_3d(x, w, rb, 80.0, 4)
    C, _ = parity.weighted_counts_and_jacobian(S, w, np.zeros((3000, 5)))
    want = oracle.marked_npairs_3d(x, x, rb, 1, period=80.0, weights1=w, weights2=w)
    assert np.max(np.abs(C - want) / want) < 1e-12
    g = rng.normal(size=len(rb))
    assert np.allclose(2 * S @ g, oracle.weighted_adjoint_3d(x, w, rb, 80.0, g), rtol=1e-12,
                       atol=1e-9)
