"""Parity summaries of GPU results against the oracle, at full workload sizes.

TEST INFRASTRUCTURE: used by the ``-m gpu`` tests and by the benchmark's CPU
leg, which run the oracle (``oracle/oracle.py``, or the reference's own
compiled engines through ``oracle/ref_driver.py``) beside the CUDA path and
report what these functions return.  Nothing on the product path imports it.

* Integer counts: bit-exact or not, with the number of differing bins.
* Weighted / marked sums and gradients: the relative error of every bin
  against the FP64 oracle, |got - want| / |want| (bins whose FP64 value is 0
  report the absolute error instead).
* The FP64 Zheng07 weights and their Jacobian in theta, the oracle side of the
  adjoint checks (zheng07_components.py:149-153 for the centrals,
  :455-470 for the satellites; halotools has no derivatives, so the Jacobian
  is the analytic derivative of those formulas).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

LN10 = math.log(10.0)


def exact(got, want) -> dict:
    """Bit-exact comparison of integer counts."""
    got = np.asarray(got)
    want = np.asarray(want)
    same = got.shape == want.shape and bool(np.array_equal(got, want))
    bad = int(np.count_nonzero(got != want)) if got.shape == want.shape else int(want.size)
    return {"exact": same, "bins": int(want.size), "mismatched_bins": bad,
            "in_range_pairs": int(np.asarray(want).reshape(-1)[-1]) if want.size else 0}


def rel_per_bin(got, want) -> list:
    """|got - want| / |want| per bin (absolute error where want == 0)."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    d = np.abs(got - want)
    den = np.abs(want)
    r = np.where(den > 0, d / np.where(den > 0, den, 1.0), d)
    return [float(v) for v in r.reshape(-1)]


def rel_summary(got, want, tol) -> dict:
    r = rel_per_bin(got, want)
    return {"max_rel_err": max(r) if r else 0.0, "tol": tol, "ok": bool(max(r, default=0.0) <= tol),
            "rel_err_per_bin": r}


def zheng07_fp64(theta, mass):
    """<Ncen> + <Nsat> in FP64 for one theta = (logMmin, sigma, logM0, logM1, alpha)."""
    lmin, sig, lm0, lm1, alpha = (float(t) for t in theta)
    mass = np.asarray(mass, dtype=np.float64)
    ncen = 0.5 * (1.0 + erf((np.log10(mass) - lmin) / sig))
    m0, m1 = 10.0 ** lm0, 10.0 ** lm1
    u = np.maximum(mass - m0, 0.0) / m1
    nsat = np.where(mass > m0, u ** alpha, 0.0)
    return ncen + nsat


def zheng07_jacobian_fp64(theta, mass):
    """dw/dtheta, (N, 5), FP64: derivatives of the centrals' erf term in
    (logMmin, sigma) and of the satellites' power law in (logM0, logM1, alpha)."""
    lmin, sig, lm0, lm1, alpha = (float(t) for t in theta)
    mass = np.asarray(mass, dtype=np.float64)
    x = (np.log10(mass) - lmin) / sig
    g = np.exp(-x * x) / math.sqrt(math.pi)  # d/dx of erf(x) / 2
    m0, m1 = 10.0 ** lm0, 10.0 ** lm1
    sat = mass > m0
    u = np.where(sat, (mass - m0) / m1, 1.0)
    ua = np.where(sat, u ** alpha, 0.0)
    J = np.zeros((len(mass), 5))
    J[:, 0] = -g / sig
    J[:, 1] = -g * x / sig
    J[:, 2] = np.where(sat, -alpha * u ** (alpha - 1.0) * m0 * LN10 / m1, 0.0)
    J[:, 3] = -alpha * LN10 * ua
    J[:, 4] = np.where(sat, ua * np.log(u), 0.0)
    return J


def weighted_counts_and_jacobian(S, w, J):
    """From the per-point table S[m, k] = sum_j w_j [d_mj <= r_k] (the oracle's
    ``weighted_per_object_3d``): C_k = sum_m w_m S[m, k] and
    dC_k/dtheta = 2 sum_m S[m, k] J[m, :], shapes (nb,) and (nb, 5)."""
    return w @ S, 2.0 * (S.T @ J)
