"""Two-point estimators on the GB300 pair counters: ``tpcf``, ``rp_pi_tpcf``,
``wp``, ``s_mu_tpcf`` and ``marked_tpcf``.

halotools' estimator layer (two_point_clustering/tpcf.py, rp_pi_tpcf.py, wp.py,
tpcf_estimators.py) is plain Python around ``npairs_3d`` / ``npairs_xy_z``; the
pair counts are where the time goes. Here the same estimators run with every
data-data, data-random and random-random count on the GPU engines of this
package. Signatures, defaults and return shapes follow halotools:

* ``tpcf(sample1, rbins, sample2=None, randoms=None, period=None, do_auto=True,
  do_cross=True, estimator="Natural", num_threads=1, approx_cell1_size=None,
  approx_cell2_size=None, approx_cellran_size=None, RR_precomputed=None,
  NR_precomputed=None, seed=None)`` (tpcf.py:212-228);
* ``rp_pi_tpcf(sample1, rp_bins, pi_bins, sample2=None, randoms=None, ...)``
  (rp_pi_tpcf.py);
* ``wp(sample1, rp_bins, pi_max, sample2=None, randoms=None, ...)`` (wp.py:20-23);
* ``s_mu_tpcf(sample1, s_bins, mu_bins, sample2=None, randoms=None, ...)``
  (s_mu_tpcf.py), analytic randoms from spherical sectors (s_mu_tpcf.py:323-334);
* ``tpcf_jackknife(sample1, randoms, rbins, Nsub=[5, 5, 5], ...)``
  (tpcf_jackknife.py:33-45): xi and its jackknife covariance over cuboid
  subvolumes, from the GPU jackknife counter (DD, DR, RR);
* ``marked_tpcf(sample1, rbins, sample2=None, marks1=None, marks2=None, ...)``
  (marked_tpcf.py). Its random-mark normalisation draws ``iterations`` mark
  permutations; with the product weight (id 1) they are counted as channels of
  one launch (``marked_npairs_3d_channels``), otherwise one call each.

With a periodic box and no randoms, random counts are analytic: ``N_R N dV / V``
with spherical shells for ``tpcf`` (tpcf.py:120-144) and cylindrical annuli of
height ``2 pi`` for ``rp_pi_tpcf`` (rp_pi_tpcf.py:359-363, 440-460). The five
estimators (Natural, Davis-Peebles, Hewett, Hamilton, Landy-Szalay) are the
published pair-count ratios, with halotools' normalisations
(tpcf_estimators.py:14-113).
"""
from __future__ import annotations

import math
import warnings

import numpy as np

from .pair_counters import (HalotoolsError, marked_npairs_3d, marked_npairs_3d_channels,
                            npairs_3d, npairs_jackknife_3d, npairs_s_mu, npairs_xy_z)

__all__ = ("tpcf", "rp_pi_tpcf", "wp", "s_mu_tpcf", "marked_tpcf", "tpcf_jackknife",
           "ESTIMATORS")

ESTIMATORS = ("Natural", "Davis-Peebles", "Hewett", "Hamilton", "Landy-Szalay")
# which of DD, DR, RR each estimator needs (tpcf_estimators.py:126-160)
_NEEDS = {"Natural": (True, False, True), "Davis-Peebles": (True, True, False),
          "Hewett": (True, True, True), "Hamilton": (True, True, True),
          "Landy-Szalay": (True, True, True)}

_ZERO_MSG = ("When calculating the two-point function, there was at least one \n"
             "separation bin with zero {0} pairs. Since the ``{1}`` estimator you chose \n"
             "divides by {0}, you will have at least one NaN returned value.\n")


def _shape(sample, name="sample1"):
    s = np.asarray(sample)
    if s.ndim != 2 or s.shape[1] != 3:
        raise TypeError("Input ``%s`` must have shape (Npts, 3)" % name)
    return s


def _period(period):
    if period is None:
        return None, False
    p = np.atleast_1d(period).astype(float)
    if len(p) == 1:
        p = np.array([p[0]] * 3)
    if len(p) != 3 or not (np.all(p < np.inf) and np.all(p > 0)):
        raise ValueError("Input ``period`` must be either a scalar or a 3-element sequence.\n"
                         "All values must bounded positive numbers.\n")
    return p, True


def _sample2(sample1, sample2, do_cross):
    """sample2 defaults to sample1; an identical sample2 means auto only."""
    if sample2 is None:
        return sample1, True, do_cross
    sample2 = _shape(sample2, "sample2")
    if sample1.shape == sample2.shape and np.all(sample1 == sample2):
        if do_cross:
            warnings.warn("\n `sample1` and `sample2` are exactly the same, \n"
                          "only the auto-correlation will be returned.\n")
        return sample2, True, False
    return sample2, False, do_cross


def _check_common(estimator, do_auto, do_cross, randoms, pbc):
    if estimator not in ESTIMATORS:
        raise ValueError("Input `estimator` must be one of the following:{0}".format(
            list(ESTIMATORS)))
    if randoms is None and not pbc:
        raise ValueError("If no PBCs are specified, randoms must be provided.\n")
    if do_auto != bool(do_auto) or do_cross != bool(do_cross):
        raise ValueError("`do_auto` and `do_cross` keywords must be boolean-valued.")


def _zero_check(DR, RR, estimator):
    if estimator in ("Natural", "Davis-Peebles", "Hewett", "Landy-Szalay") and np.any(RR == 0):
        raise ValueError(_ZERO_MSG.format("RR", estimator))
    if estimator == "Hamilton" and np.any(DR == 0):
        raise ValueError(_ZERO_MSG.format("DR", estimator))


def _mult(x, y):
    """A per-sample factor times each row (jackknife subsamples), or plain product."""
    return (x * y.T).T if np.ndim(x) > 0 else x * y


def _xi(DD, DR, RR, ND1, ND2, NR1, NR2, estimator):
    """Auto-type estimator from differential counts (tpcf_estimators.py:14-58);
    the N's may be per-subsample arrays (rows of DD, DR, RR)."""
    _zero_check(DR, RR, estimator)
    with np.errstate(divide="ignore", invalid="ignore"):
        if estimator == "Natural":
            return _mult(1.0 / (ND1 * ND2 / (NR1 * NR2)), DD / RR) - 1.0
        if estimator == "Davis-Peebles":
            return _mult(1.0 / (ND1 * ND2 / (ND1 * NR2)), DD / DR) - 1.0
        if estimator == "Hewett":
            f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
            return _mult(1.0 / f1, DD / RR) - _mult(1.0 / f2, DR / RR)
        if estimator == "Hamilton":
            return (DD * RR) / (DR * DR) - 1.0
        f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
        return _mult(1.0 / f1, DD / RR) - _mult(1.0 / f2, 2.0 * DR / RR) + 1.0


def _xi_cross(DD, D1R, D2R, RR, ND1, ND2, NR1, NR2, estimator):
    """Cross estimator (tpcf_estimators.py:61-99): Natural, Hamilton, Landy-Szalay."""
    _zero_check(D1R, RR, estimator)
    _zero_check(D2R, RR, estimator)
    with np.errstate(divide="ignore", invalid="ignore"):
        if estimator == "Natural":
            return _mult(1.0 / (ND1 * ND2 / (NR1 * NR2)), DD / RR) - 1.0
        if estimator == "Hamilton":
            return (DD * RR) / (D1R * D2R) - 1.0
        if estimator == "Landy-Szalay":
            f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
            return (_mult(1.0 / f1, DD / RR) - _mult(1.0 / f2, D1R / RR) -
                    _mult(1.0 / f2, D2R / RR) + 1.0)
    raise ValueError("{0} estimator is not supported for cross-correlations".format(estimator))


def _combine(auto, cross, s1_is_s2, do_auto, do_cross):
    """Return what halotools returns for the auto/cross switches (tpcf.py:458-476)."""
    if s1_is_s2:
        return auto(1)
    if do_auto and do_cross:
        return auto(1), cross(), auto(2)
    if do_cross:
        return cross()
    if do_auto:
        return auto(1), auto(2)
    return None


# ---------------- 3-D ----------------
def tpcf(sample1, rbins, sample2=None, randoms=None, period=None, do_auto=True, do_cross=True,
         estimator="Natural", num_threads=1, approx_cell1_size=None, approx_cell2_size=None,
         approx_cellran_size=None, RR_precomputed=None, NR_precomputed=None, seed=None):
    """Real-space two-point correlation function xi(r) (halotools tpcf.py:212),
    every pair count on the GPU."""
    sample1 = _shape(sample1)
    sample2, s1_is_s2, do_cross = _sample2(sample1, sample2, do_cross)
    rbins = np.atleast_1d(rbins).astype(float)
    period, pbc = _period(period)
    _check_common(estimator, do_auto, do_cross, randoms, pbc)
    if (RR_precomputed is None) != (NR_precomputed is None):
        raise ValueError("\nYou must either provide both ``RR_precomputed`` and "
                         "``NR_precomputed`` arguments, or neither\n")
    if RR_precomputed is not None:
        # tpcf.py:560-584
        RR_precomputed = np.atleast_1d(RR_precomputed)
        if len(RR_precomputed) != len(rbins) - 1:
            raise HalotoolsError("\nLength of ``RR_precomputed`` must match length of ``rbins``\n")
        if np.any(RR_precomputed == 0):
            warnings.warn("RR_precomputed has radial bin(s) which contain no pairs. \n"
                          "Consider increasing the number of randoms, or using larger bins.")
        if randoms is None or len(randoms) != NR_precomputed:
            raise HalotoolsError("If passing in randoms and also NR_precomputed, \n"
                                 "the value of NR_precomputed must agree with the number of "
                                 "randoms\n")
    do_dd, do_dr, do_rr = _NEEDS[estimator]
    if RR_precomputed is not None:
        do_rr = False
    N1, N2 = len(sample1), len(sample2)
    NR = len(randoms) if randoms is not None else (
        NR_precomputed if NR_precomputed is not None else N1)
    kw = dict(period=period, num_threads=num_threads)

    def diff(a, b, c1, c2):
        return np.diff(npairs_3d(a, b, rbins, approx_cell1_size=c1, approx_cell2_size=c2, **kw))

    D11 = diff(sample1, sample1, approx_cell1_size, approx_cell1_size) if do_auto else None
    if s1_is_s2:
        D12 = D22 = D11
    else:
        D12 = diff(sample1, sample2, approx_cell1_size, approx_cell2_size) if do_cross else None
        D22 = diff(sample2, sample2, approx_cell2_size, approx_cell2_size) if do_auto else None

    if randoms is not None:
        randoms = _shape(randoms, "randoms")
        RR = diff(randoms, randoms, approx_cellran_size, approx_cellran_size) if do_rr else None
        D1R = diff(sample1, randoms, approx_cell1_size, approx_cellran_size) if do_dr else None
        D2R = None if s1_is_s2 else (
            diff(sample2, randoms, approx_cell2_size, approx_cellran_size) if do_dr else None)
    else:
        # analytic randoms in the periodic box: N_R N dV / V (tpcf.py:120-144)
        v = (math.pi ** 1.5 / math.gamma(2.5)) * rbins ** 3
        dv = np.diff(v)
        vol = period.prod()
        D1R = NR * (dv * (N1 / vol))
        D2R = NR * (dv * (N2 / vol))
        RR = dv * (NR ** 2 / vol)
    if RR_precomputed is not None:
        RR = RR_precomputed

    def auto(k):
        return _xi(D11, D1R, RR, N1, N1, NR, NR, estimator) if k == 1 else \
            _xi(D22, D2R, RR, N2, N2, NR, NR, estimator)

    def cross():
        return _xi_cross(D12, D1R, D2R, RR, N1, N2, NR, NR, estimator)

    return _combine(auto, cross, s1_is_s2, do_auto, do_cross)


# ---------------- (rp, pi) ----------------
def rp_pi_tpcf(sample1, rp_bins, pi_bins, sample2=None, randoms=None, period=None,
               do_auto=True, do_cross=True, estimator="Natural", num_threads=1,
               approx_cell1_size=None, approx_cell2_size=None, approx_cellran_size=None,
               seed=None):
    """Redshift-space xi(rp, pi) (halotools rp_pi_tpcf.py), every pair count on the
    GPU. Returns arrays of shape (len(rp_bins) - 1, len(pi_bins) - 1)."""
    sample1 = _shape(sample1)
    sample2, s1_is_s2, do_cross = _sample2(sample1, sample2, do_cross)
    rp_bins = np.atleast_1d(rp_bins).astype(float)
    pi_bins = np.atleast_1d(pi_bins).astype(float)
    period, pbc = _period(period)
    _check_common(estimator, do_auto, do_cross, randoms, pbc)
    do_dd, do_dr, do_rr = _NEEDS[estimator]
    N1, N2 = len(sample1), len(sample2)
    NR = len(randoms) if randoms is not None else N1
    kw = dict(period=period, num_threads=num_threads)

    def diff2(a, b, c1, c2):
        c = npairs_xy_z(a, b, rp_bins, pi_bins, approx_cell1_size=c1, approx_cell2_size=c2, **kw)
        return np.diff(np.diff(c, axis=0), axis=1)

    D11 = diff2(sample1, sample1, approx_cell1_size, approx_cell1_size) if do_auto else None
    if s1_is_s2:
        D12 = D22 = D11
    else:
        D12 = diff2(sample1, sample2, approx_cell1_size, approx_cell2_size) if do_cross else None
        D22 = diff2(sample2, sample2, approx_cell2_size, approx_cell2_size) if do_auto else None

    if randoms is not None:
        randoms = _shape(randoms, "randoms")
        RR = diff2(randoms, randoms, approx_cellran_size, approx_cellran_size) if do_rr else None
        D1R = diff2(sample1, randoms, approx_cell1_size, approx_cellran_size) if do_dr else None
        D2R = None if s1_is_s2 else (
            diff2(sample2, randoms, approx_cell2_size, approx_cellran_size) if do_dr else None)
    else:
        # analytic randoms: cylinders of radius rp and height 2 pi (rp_pi_tpcf.py:359-363, 440-460)
        v = math.pi * np.outer(rp_bins ** 2.0, 2.0 * pi_bins)
        dv = np.diff(np.diff(v, axis=0), axis=1)
        vol = period.prod()
        D1R = N1 * (dv * (N1 / vol))
        D2R = N2 * (dv * (N2 / vol))
        RR = dv * (NR ** 2 / vol)

    def auto(k):
        return _xi(D11, D1R, RR, N1, N1, NR, NR, estimator) if k == 1 else \
            _xi(D22, D2R, RR, N2, N2, NR, NR, estimator)

    def cross():
        return _xi_cross(D12, D1R, D2R, RR, N1, N2, NR, NR, estimator)

    return _combine(auto, cross, s1_is_s2, do_auto, do_cross)


def wp(sample1, rp_bins, pi_max, sample2=None, randoms=None, period=None, do_auto=True,
       do_cross=True, estimator="Natural", num_threads=1, approx_cell1_size=None,
       approx_cell2_size=None, approx_cellran_size=None, seed=None):
    """Projected correlation function w_p(rp) = 2 pi_max xi(rp, 0 < pi < pi_max)
    (halotools wp.py:20), from one GPU (rp, pi) count per sample pair."""
    pi_max = float(pi_max)
    res = rp_pi_tpcf(sample1, rp_bins, np.array([0.0, pi_max]), sample2=sample2,
                     randoms=randoms, period=period, do_auto=do_auto, do_cross=do_cross,
                     estimator=estimator, num_threads=num_threads,
                     approx_cell1_size=approx_cell1_size, approx_cell2_size=approx_cell2_size,
                     approx_cellran_size=approx_cellran_size)
    if isinstance(res, tuple):
        return tuple(2.0 * r[:, 0] * pi_max for r in res)
    return 2.0 * res[:, 0] * pi_max


# ---------------- (s, mu) ----------------
def s_mu_tpcf(sample1, s_bins, mu_bins, sample2=None, randoms=None, period=None, do_auto=True,
              do_cross=True, estimator="Natural", num_threads=1, approx_cell1_size=None,
              approx_cell2_size=None, approx_cellran_size=None, seed=None):
    """xi(s, mu) (halotools s_mu_tpcf.py), every pair count on the GPU. Returns
    arrays of shape (len(s_bins) - 1, len(mu_bins) - 1) in increasing mu."""
    sample1 = _shape(sample1)
    sample2, s1_is_s2, do_cross = _sample2(sample1, sample2, do_cross)
    s_bins = np.atleast_1d(s_bins).astype(float)
    mu_bins = np.atleast_1d(mu_bins).astype(float)
    if np.min(mu_bins) < 0.0 or np.max(mu_bins) > 1.0:
        raise ValueError("`mu_bins` must be in the range [0,1].")
    period, pbc = _period(period)
    _check_common(estimator, do_auto, do_cross, randoms, pbc)
    do_dd, do_dr, do_rr = _NEEDS[estimator]
    N1, N2 = len(sample1), len(sample2)
    NR = len(randoms) if randoms is not None else N1
    kw = dict(period=period, num_threads=num_threads)

    def diff2(a, b, c1, c2):
        c = npairs_s_mu(a, b, s_bins, mu_bins, approx_cell1_size=c1, approx_cell2_size=c2, **kw)
        return np.diff(np.diff(c, axis=0), axis=1)

    D11 = diff2(sample1, sample1, approx_cell1_size, approx_cell1_size) if do_auto else None
    if s1_is_s2:
        D12 = D22 = D11
    else:
        D12 = diff2(sample1, sample2, approx_cell1_size, approx_cell2_size) if do_cross else None
        D22 = diff2(sample2, sample2, approx_cell2_size, approx_cell2_size) if do_auto else None

    if randoms is not None:
        randoms = _shape(randoms, "randoms")
        RR = diff2(randoms, randoms, approx_cellran_size, approx_cellran_size) if do_rr else None
        D1R = diff2(sample1, randoms, approx_cell1_size, approx_cellran_size) if do_dr else None
        D2R = None if s1_is_s2 else (
            diff2(sample2, randoms, approx_cell2_size, approx_cellran_size) if do_dr else None)
    else:
        # wedges of spherical sectors, doubled for the reflection (s_mu_tpcf.py:323-334, 418-440)
        mu_rev = np.sort(mu_bins)[::-1]
        v = (2.0 * np.pi / 3.0) * np.outer(s_bins ** 3.0, 1.0 - np.cos(np.arccos(mu_rev))) * 2.0
        dv = np.diff(np.diff(v, axis=1), axis=0)
        vol = period.prod()
        D1R = (N1 - 1.0) * (dv * (N1 / vol))
        D2R = (N2 - 1.0) * (dv * (N2 / vol))
        RR = dv * (NR ** 2 / vol)

    # counts run in increasing sin(theta_LOS), i.e. decreasing mu: reverse the last axis
    def auto(k):
        x = _xi(D11, D1R, RR, N1, N1, NR, NR, estimator) if k == 1 else \
            _xi(D22, D2R, RR, N2, N2, NR, NR, estimator)
        return x[:, ::-1]

    def cross():
        return _xi_cross(D12, D1R, D2R, RR, N1, N2, NR, NR, estimator)[:, ::-1]

    return _combine(auto, cross, s1_is_s2, do_auto, do_cross)


# ---------------- marked ----------------
class _LegacySeed:
    """Seed numpy's legacy global generator inside a ``with`` block and restore
    it afterwards (the permutation draws of marked_tpcf.py:150-165)."""

    def __init__(self, seed):
        self.seed = seed

    def __enter__(self):
        self.state = np.random.get_state()
        np.random.seed(self.seed)

    def __exit__(self, *exc):
        np.random.set_state(self.state)


def _marks(m, n, name):
    m = np.ones(n) if m is None else np.atleast_1d(m).astype(float)
    if m.ndim == 1:
        m = m.reshape((len(m), 1))
    elif m.ndim != 2:
        raise HalotoolsError("\n You must either pass in a 1-D or 2-D array \n"
                             "for the input `%s`." % name)
    if len(m) != n:
        raise HalotoolsError("\n `%s` must have same length as `%s`." %
                             (name, "sample1" if name == "marks1" else "sample2"))
    return m


def marked_tpcf(sample1, rbins, sample2=None, marks1=None, marks2=None, period=None,
                do_auto=True, do_cross=True, num_threads=1, weight_func_id=1,
                normalize_by="random_marks", iterations=1, randomize_marks=None, seed=None):
    """Marked correlation function M(r) = W(r) / R(r) (halotools marked_tpcf.py),
    every weighted count on the GPU.

    ``normalize_by="random_marks"`` divides by the weighted counts with the marks
    permuted among the points, ``iterations`` times (the median is kept);
    ``"number_counts"`` by the plain pair counts. As in halotools, each iteration
    re-seeds the permutation draws with ``seed`` and permutes the already
    permuted marks, and both sides of a random auto count use the permuted
    marks (marked_tpcf.py:150-221).
    """
    sample1 = _shape(sample1)
    sample2, s1_is_s2, do_cross = _sample2(sample1, sample2, do_cross)
    try:
        int(weight_func_id) == weight_func_id
    except Exception:
        raise ValueError("\n `wfunc` parameter must be an integer ID of the desired function.")
    if normalize_by not in ("random_marks", "number_counts"):
        raise ValueError("\n `normalize_by` parameter not recognized.")
    marks1 = _marks(marks1, len(sample1), "marks1")
    marks2 = _marks(marks2, len(sample2), "marks2")
    randomize = np.atleast_1d(randomize_marks) if randomize_marks is not None else \
        np.array([True] * marks1.shape[1])
    if randomize.ndim != 1:
        raise HalotoolsError("\n `randomize_marks` must be one dimensional.")
    if len(randomize) != marks1.shape[1]:
        raise HalotoolsError("\n `randomize_marks` must have same length \n"
                             " as the number of weights per point.")
    rbins = np.atleast_1d(rbins).astype(float)
    period, _ = _period(period)
    if do_auto != bool(do_auto) or do_cross != bool(do_cross):
        raise ValueError("`do_auto` and `do_cross` keywords must be boolean-valued.")
    wid = int(weight_func_id)
    kw = dict(period=period, num_threads=num_threads)

    def w(a, b, m1, m2):
        return np.diff(marked_npairs_3d(a, b, rbins, wid, weights1=m1, weights2=m2, **kw))

    W11 = w(sample1, sample1, marks1, marks1) if do_auto else None
    if s1_is_s2:
        W12 = W22 = W11
    else:
        W12 = w(sample1, sample2, marks1, marks2) if do_cross else None
        W22 = w(sample2, sample2, marks2, marks2) if do_auto else None

    if normalize_by == "number_counts":
        def c(a, b):
            return np.diff(npairs_3d(a, b, rbins, **kw))
        R11 = c(sample1, sample1) if do_auto else None
        if s1_is_s2:
            R12 = R22 = R11
        else:
            R12 = c(sample1, sample2) if do_cross else None
            R22 = c(sample2, sample2) if do_auto else None
    else:
        # the marks of every iteration, drawn and composed as halotools does
        p1s, p2s = [], []
        m1, m2 = marks1.copy(), marks2.copy()
        for _ in range(int(iterations)):
            with _LegacySeed(seed):
                perm1 = np.random.permutation(np.arange(0, len(sample1)))
                perm2 = np.random.permutation(np.arange(0, len(sample2)))
            for k in range(m1.shape[1]):
                if randomize[k]:
                    m1[:, k] = m1[perm1, k]
            for k in range(m2.shape[1]):
                if randomize[k]:
                    m2[:, k] = m2[perm2, k]
            p1s.append(m1.copy())
            p2s.append(m2.copy())
        R11, R12, R22 = _random_marked(sample1, sample2, rbins, wid, p1s, p2s, s1_is_s2,
                                       do_auto, do_cross, kw)
        if int(iterations) > 1:
            R11 = None if R11 is None else np.median(R11, axis=0)
            R12 = None if R12 is None else np.median(R12, axis=0)
            R22 = None if R22 is None else np.median(R22, axis=0)
        else:
            R11 = None if R11 is None else R11[0]
            R12 = None if R12 is None else R12[0]
            R22 = None if R22 is None else R22[0]

    with np.errstate(divide="ignore", invalid="ignore"):
        def auto(k):
            return W11 / R11 if k == 1 else W22 / R22

        def cross():
            return W12 / R12

        return _combine(auto, cross, s1_is_s2, do_auto, do_cross)


def _random_marked(sample1, sample2, rbins, wid, p1s, p2s, s1_is_s2, do_auto, do_cross, kw):
    """Weighted counts with permuted marks, one row per iteration: product marks
    (id 1, one weight per point) as channels of one launch (32 per launch),
    other marking functions one call per iteration."""
    its = len(p1s)

    def rows(a, b, ma, mb):
        if wid == 1 and ma[0].shape[1] == 1:
            out = []
            for c0 in range(0, its, 32):
                wa = np.ascontiguousarray(np.concatenate(ma[c0:c0 + 32], axis=1))
                wb = wa if mb is ma else np.ascontiguousarray(np.concatenate(mb[c0:c0 + 32], axis=1))
                out.append(np.diff(marked_npairs_3d_channels(a, b, rbins, weights1=wa, weights2=wb,
                                                             **kw), axis=1))
            return np.concatenate(out, axis=0)
        return np.stack([np.diff(marked_npairs_3d(a, b, rbins, wid, weights1=x, weights2=y, **kw))
                         for x, y in zip(ma, mb)])

    R11 = rows(sample1, sample1, p1s, p1s) if do_auto else None
    if s1_is_s2:
        return R11, R11, R11
    R12 = rows(sample1, sample2, p1s, p2s) if do_cross else None
    R22 = rows(sample2, sample2, p2s, p2s) if do_auto else None
    return R11, R12, R22


# ---------------- jackknife ----------------
def _cuboid_labels(sample, Nsub, Lbox):
    """Labels 1..prod(Nsub) of the cuboid subvolumes holding the points, points
    on the upper face in the last subvolume (catalog_analysis_helpers.py:330-384)."""
    Nsub = np.atleast_1d(Nsub).astype("i4")
    if len(Nsub) == 1:
        Nsub = np.array([Nsub[0]] * 3)
    elif len(Nsub) != 3:
        raise TypeError("Input ``Nsub`` must be a scalar or length-3 sequence")
    Lbox = np.atleast_1d(Lbox).astype("f8")
    if len(Lbox) == 1:
        Lbox = np.array([Lbox[0]] * 3)
    dL = Lbox / Nsub
    n_sub = int(np.prod(Nsub))
    ids = np.arange(1, n_sub + 1).reshape(Nsub[0], Nsub[1], Nsub[2])
    idx = np.floor(sample / dL).astype(int)
    for d in range(3):
        idx[:, d] = np.where(idx[:, d] == Nsub[d], Nsub[d] - 1, idx[:, d])
    return ids[idx[:, 0], idx[:, 1], idx[:, 2]].astype(int), n_sub


def _enclose3(a, b, c):
    """Shift three samples by their smallest coordinate; cube of the largest extent
    (tpcf_jackknife.py:403-440)."""
    lo = np.min([np.min(x[:, d]) for x in (a, b, c) for d in range(3)])
    hi = np.max([np.max(x[:, d]) for x in (a, b, c) for d in range(3)]) - lo
    return a - lo, b - lo, c - lo, np.array([hi, hi, hi])


def tpcf_jackknife(sample1, randoms, rbins, Nsub=[5, 5, 5], sample2=None, period=None,
                   do_auto=True, do_cross=True, estimator="Natural", num_threads=1, seed=None):
    """xi(r) and its jackknife covariance (halotools tpcf_jackknife.py:33): the
    box is cut into ``Nsub`` cuboids, each pair counted once per subsample with
    the GPU jackknife counter, and the covariance is (N - 1) times the biased
    covariance of the leave-one-out estimates. ``randoms`` may be a 1-element
    array giving the number of uniform randoms to draw (periodic boxes)."""
    sample1 = _shape(sample1)
    sample2, s1_is_s2, do_cross = _sample2(sample1, sample2, do_cross)
    period, pbc = _period(period)
    if np.shape(randoms) == (1,):
        n_ran = randoms[0]
        if not pbc:
            raise HalotoolsError("\n When no `period` parameter is passed, \n"
                                 "the user must provide true randoms, and \n"
                                 "not just the number of randoms desired.")
        with _LegacySeed(seed):
            randoms = np.random.random((n_ran, 3)) * period
    randoms = _shape(randoms, "randoms")
    rbins = np.atleast_1d(rbins).astype(float)
    _check_common(estimator, do_auto, do_cross, randoms, pbc)
    if pbc:
        lbox = period
    else:
        sample1, sample2, randoms, lbox = _enclose3(sample1, sample2, randoms)
        if s1_is_s2:
            sample2 = sample1
    do_dd, do_dr, do_rr = _NEEDS[estimator]
    N1, N2, NR = len(sample1), len(sample2), len(randoms)
    j1, nsv = _cuboid_labels(sample1, Nsub, lbox)
    j2, _ = _cuboid_labels(sample2, Nsub, lbox)
    jr, _ = _cuboid_labels(randoms, Nsub, lbox)

    def per_sub(j):  # points in each subvolume (tpcf_jackknife.py:443-457)
        return np.bincount(j, minlength=nsv + 1)[1:]
    N1s, N2s, NRs = N1 - per_sub(j1), N2 - per_sub(j2), NR - per_sub(jr)
    kw = dict(period=period, num_threads=num_threads)

    def jk(a, b, ta, tb):
        return np.diff(npairs_jackknife_3d(a, b, rbins, ta, tb, nsv, **kw), axis=1)

    D11 = jk(sample1, sample1, j1, j1) if do_auto else None
    if s1_is_s2:
        D12 = D22 = D11
    else:
        D12 = jk(sample1, sample2, j1, j2) if do_cross else None
        D22 = jk(sample2, sample2, j2, j2) if do_auto else None
    D1R = jk(sample1, randoms, j1, jr) if do_dr else None
    RR = jk(randoms, randoms, jr, jr) if do_rr else None
    D2R = D1R if s1_is_s2 else (jk(sample2, randoms, j2, jr) if do_dr else None)

    def full(x):
        return None if x is None else x[0, :]

    def sub(x):
        return None if x is None else x[1:, :]

    out_full, out_cov = {}, {}
    if do_auto:
        out_full[11] = _xi(full(D11), full(D1R), full(RR), N1, N1, NR, NR, estimator)
        out_full[22] = _xi(full(D22), full(D2R), full(RR), N2, N2, NR, NR, estimator)
        x11 = _xi(sub(D11), sub(D1R), sub(RR), N1s, N1s, NRs, NRs, estimator)
        x22 = _xi(sub(D22), sub(D2R), sub(RR), N2s, N2s, NRs, NRs, estimator)
        out_cov[11] = np.array(np.cov(x11.T, bias=True)) * (nsv - 1.0)
        out_cov[22] = np.array(np.cov(x22.T, bias=True)) * (nsv - 1.0)
    if do_cross:
        out_full[12] = _xi_cross(full(D12), full(D1R), full(D2R), full(RR), N1, N2, NR, NR,
                                 estimator)
        x12 = _xi_cross(sub(D12), sub(D1R), sub(D2R), sub(RR), N1s, N2s, NRs, NRs, estimator)
        out_cov[12] = np.array(np.cov(x12.T, bias=True)) * (nsv - 1.0)
    if s1_is_s2:
        return out_full[11], out_cov[11]
    if do_auto and do_cross:
        return (out_full[11], out_full[12], out_full[22], out_cov[11], out_cov[12], out_cov[22])
    if do_auto:
        return out_full[11], out_full[22], out_cov[11], out_cov[22]
    return out_full[12], out_cov[12]
