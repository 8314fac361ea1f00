"""Estimator-layer argument checks (raised before any pair is counted)."""
import numpy as np
import pytest

from halotools_gb300 import estimators as E
from halotools_gb300 import HalotoolsError


S = np.random.default_rng(0).uniform(0, 100, (50, 3))
R = np.logspace(-1, 1, 5)


def test_unknown_estimator():
    with pytest.raises(ValueError, match="estimator"):
        E.tpcf(S, R, period=100.0, estimator="Peebles")


def test_randoms_required_without_period():
    with pytest.raises(ValueError, match="randoms must be provided"):
        E.tpcf(S, R)
    with pytest.raises(ValueError, match="randoms must be provided"):
        E.wp(S, R, 10.0)


def test_rr_precomputed_needs_nr_and_matching_randoms():
    with pytest.raises(ValueError, match="both"):
        E.tpcf(S, R, period=100.0, RR_precomputed=np.ones(4))
    with pytest.raises(HalotoolsError, match="length of ``rbins``"):
        E.tpcf(S, R, randoms=S, period=100.0, RR_precomputed=np.ones(3), NR_precomputed=50)
    with pytest.raises(HalotoolsError, match="NR_precomputed"):
        E.tpcf(S, R, randoms=S, period=100.0, RR_precomputed=np.ones(4), NR_precomputed=49)


def test_bad_period_and_shape():
    with pytest.raises(ValueError, match="period"):
        E.tpcf(S, R, period=[100.0, -1.0, 100.0])
    with pytest.raises(TypeError, match="shape"):
        E.tpcf(S[:, :2], R, period=100.0)


def test_estimator_formulas_on_known_counts():
    # xi = (NR^2 / N^2) DD / RR - 1 (Natural) and Landy-Szalay with DR = RR N / NR
    DD, RR = np.array([10.0, 20.0]), np.array([5.0, 5.0])
    xi = E._xi(DD, None, RR, 10, 10, 20, 20, "Natural")
    np.testing.assert_allclose(xi, 4.0 * DD / RR - 1.0)
    DR = RR * 10 / 20
    ls = E._xi(DD, DR, RR, 10, 10, 20, 20, "Landy-Szalay")
    np.testing.assert_allclose(ls, 4.0 * DD / RR - 2.0 * 2.0 * DR / RR + 1.0)
