"""Two-point estimators on the GB300 pair counters: ``tpcf``, ``rp_pi_tpcf``, ``wp``.

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
* ``wp(sample1, rp_bins, pi_max, sample2=None, randoms=None, ...)`` (wp.py:20-23).

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

from .pair_counters import HalotoolsError, npairs_3d, npairs_xy_z

__all__ = ("tpcf", "rp_pi_tpcf", "wp", "ESTIMATORS")

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


def _xi(DD, DR, RR, ND1, ND2, NR1, NR2, estimator):
    """Auto-type estimator from differential counts (tpcf_estimators.py:14-58)."""
    _zero_check(DR, RR, estimator)
    with np.errstate(divide="ignore", invalid="ignore"):
        if estimator == "Natural":
            return (1.0 / (ND1 * ND2 / (NR1 * NR2))) * (DD / RR) - 1.0
        if estimator == "Davis-Peebles":
            return (1.0 / (ND1 * ND2 / (ND1 * NR2))) * (DD / DR) - 1.0
        if estimator == "Hewett":
            f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
            return (1.0 / f1) * (DD / RR) - (1.0 / f2) * (DR / RR)
        if estimator == "Hamilton":
            return (DD * RR) / (DR * DR) - 1.0
        f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
        return (1.0 / f1) * (DD / RR) - (1.0 / f2) * (2.0 * DR / RR) + 1.0


def _xi_cross(DD, D1R, D2R, RR, ND1, ND2, NR1, NR2, estimator):
    """Cross estimator (tpcf_estimators.py:61-99): Natural, Hamilton, Landy-Szalay."""
    _zero_check(D1R, RR, estimator)
    _zero_check(D2R, RR, estimator)
    with np.errstate(divide="ignore", invalid="ignore"):
        if estimator == "Natural":
            return (1.0 / (ND1 * ND2 / (NR1 * NR2))) * (DD / RR) - 1.0
        if estimator == "Hamilton":
            return (DD * RR) / (D1R * D2R) - 1.0
        if estimator == "Landy-Szalay":
            f1, f2 = ND1 * ND2 / (NR1 * NR2), ND1 * NR2 / (NR1 * NR2)
            return (1.0 / f1) * (DD / RR) - (1.0 / f2) * (D1R / RR) - (1.0 / f2) * (D2R / RR) + 1.0
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
