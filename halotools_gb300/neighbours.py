"""Per-object neighbour counts on the GB300 engines: counts in cylinders and the
isolation functions.

Signatures, defaults, argument checks and messages follow the reference
front-ends:

* ``counts_in_cylinders``     counts_in_cells/counts_in_cylinders.py:27-300
* ``spherical_isolation``     isolation_functions/spherical_isolation.py:27-209
* ``cylindrical_isolation``   isolation_functions/cylindrical_isolation.py:28-245
* ``conditional_spherical_isolation``   conditional_spherical_isolation.py:25-220
* ``conditional_cylindrical_isolation`` conditional_cylindrical_isolation.py:25-240

All of them run ``gbp_counts_in_cylinders`` / ``gbp_cylinder_pairs`` /
``gbp_isolation`` (``include/gbpairs.h``): a full-stencil gather over the GPU
cell grid, FP32 with a guard band and an FP64 decision in the reference's
operation order near each point's radius.

Differences, for inputs the reference does not handle consistently:

* ``num_threads`` is validated and ignored.  (With ``num_threads > 1`` the
  reference's isolation front-ends add up per-process flags in which the points
  a process did not visit count as isolated, so every point comes back
  isolated; the GPU gives the single-process answer.)
* Without a period, ``counts_in_cylinders`` encloses the points from the
  (x, z, z) columns and then keeps the unshifted positions
  (counts_in_cylinders.py:241-263); here the points are shifted into the
  enclosing box as the pair counters do, which changes nothing but the last
  bit of a separation.
"""
from __future__ import annotations

import numpy as np

from . import _native
from .pair_counters import (HalotoolsError, _approx_cells, _check_num_threads, _columns,
                            _positions)

__all__ = ("counts_in_cylinders", "spherical_isolation", "cylindrical_isolation",
           "conditional_spherical_isolation", "conditional_cylindrical_isolation")


def _per_point(values, n1, msg):
    # counts_in_cylinders.py:207-223: a scalar or one value per sample-1 point;
    # a scalar is broadcast in one pass (v + 0.0, the bits of zeros(n1) + v).
    # Returns the per-point array and its maximum (0.0 with no points).
    v = np.atleast_1d(values).astype("f8", copy=False)  # read only
    if len(v) == 1:
        return np.full(n1, v[0] + 0.0), (v[0] + 0.0 if n1 else 0.0)
    if len(v) == n1:
        return v, (np.max(v) if n1 else 0.0)
    raise ValueError(msg)


def _get_r_max(n1, r_max):
    # isolation_functions_helpers.py:11-35; a scalar is checked once, then
    # broadcast (with no points every value passes, as the empty array does)
    r = np.atleast_1d(r_max).astype(float, copy=False)  # read only
    msg = "Input ``r_max`` must be an array of bounded positive numbers."
    if len(r) == 1:
        if n1 > 0 and not (r[0] < np.inf and r[0] > 0):
            raise ValueError(msg)
        return np.full(n1, r[0])
    if len(r) != n1:
        raise ValueError("Input ``r_max`` must be the same length as ``sample1``.")
    if not (np.all(r < np.inf) and np.all(r > 0)):
        raise ValueError(msg)
    return r


def _cond(kind=0, func=0, marks1=None, marks2=None, lim=(0.0, 0.0), eq=(False, False)):
    c = _native.NeighCond()
    c.kind = kind
    c.func = func
    keep = []
    if marks1 is not None:
        m1 = np.ascontiguousarray(marks1, dtype=np.float64)
        m2 = np.ascontiguousarray(marks2, dtype=np.float64)
        keep = [m1, m2]
        c.marks1 = _native.dptr(m1)
        c.marks2 = _native.dptr(m2)
        c.nmarks = 1 if m1.ndim == 1 else m1.shape[1]
    c.lower_inclusive = int(bool(eq[0]))
    c.upper_inclusive = int(bool(eq[1]))
    c.lim[0], c.lim[1] = float(lim[0]), float(lim[1])
    return c, keep


def counts_in_cylinders(sample1, sample2, proj_search_radius, cylinder_half_length, period=None,
                        verbose=False, num_threads=1, approx_cell1_size=None,
                        approx_cell2_size=None, return_indexes=False, condition=None,
                        condition_args=()):
    """Number of ``sample2`` points in each ``sample1`` point's cylinder of radius
    ``proj_search_radius`` (xy) and half-length ``cylinder_half_length`` (z).

    Same inputs and outputs as halotools ``counts_in_cylinders``
    (counts_in_cylinders.py:27): int64 counts per ``sample1`` point, and with
    ``return_indexes`` a structured array of ``(i1, i2)`` uint32 pairs (in no
    particular order).  ``sample2=None`` is the auto-correlation, which does not
    count a point in its own cylinder.  ``condition="mass_frac"`` with
    ``condition_args = (mass1, mass2, (fmin, fmax)[, lower_equality[,
    upper_equality]])`` counts only pairs with fmin < mass2[j] / mass1[i] < fmax.
    """
    _check_num_threads(num_threads)
    autocorr = sample2 is None
    s1 = _columns(np.asarray(sample1, dtype=np.float64))
    s2 = s1 if autocorr else _columns(np.asarray(sample2, dtype=np.float64))
    n1 = len(s1)
    if return_indexes and (len(s1) > 2 ** 32 or len(s2) > 2 ** 32):
        raise ValueError("Return indexes uses a uint32 and so can only handle inputs shorter "
                         "than 2^32 (~4 Billion).")
    rp, rpm = _per_point(proj_search_radius, n1,
                         "Input ``proj_search_radius`` must be a scalar or length-Npts1 array")
    pi, pim = _per_point(cylinder_half_length, n1,
                         "Input ``cylinder_half_length`` must be a scalar or length-Npts1 array")
    _approx_cells(approx_cell1_size, [rpm, rpm, pim], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rpm, rpm, pim], "approx_cell2_size")
    # conditions.pyx choose_condition
    if condition is None or condition == "always_true":
        cond, keep = _cond()
    elif condition == "mass_frac":
        m1 = np.asarray(condition_args[0], dtype=np.float64)
        m2 = np.asarray(condition_args[1], dtype=np.float64)
        lims = [float(a) for a in condition_args[2]]
        eq = list(condition_args[3:]) + [False, False]
        cond, keep = _cond(1, 0, m1, m2, lims, eq[:2])
    else:
        raise ValueError("'condition' must be None or a permitted descriptive string")
    x1, x2, box, pbc = _positions(s1, s2, period, [rpm, rpm, pim],
                                  [rpm * 3.0, rpm * 3.0, pim * 3.0])
    plan = _native.default_plan()
    rp = np.ascontiguousarray(rp)
    pi = np.ascontiguousarray(pi)
    counts = np.zeros(n1, dtype=np.int64)
    plan.check(plan.lib.gbp_counts_in_cylinders(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.pd(rp),
        _native.pd(pi), _native.pd(box), pbc, _native.ref(cond), _native.pi64(counts)))
    if return_indexes:
        pairs = np.zeros(2 * max(int(counts.sum()), 1), dtype=np.uint32)
        plan.check(plan.lib.gbp_cylinder_pairs(
            plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.pd(rp),
            _native.pd(pi), _native.pd(box), pbc, _native.ref(cond), _native.pi64(counts),
            _native.pu32(pairs)))
        pairs = pairs[:2 * int(counts.sum())].reshape(-1, 2)
        indexes = np.zeros(len(pairs), dtype=[("i1", np.uint32), ("i2", np.uint32)])
        indexes["i1"], indexes["i2"] = pairs[:, 0], pairs[:, 1]
    del keep
    # counts_in_cylinders.py:190-195: a point always matches itself
    if autocorr:
        counts -= 1
        if return_indexes:
            indexes = indexes[indexes["i1"] != indexes["i2"]]
    if return_indexes:
        return counts, indexes
    return counts


def _isolation(sample1, sample2, r, pi, period, num_threads, approx_cell1_size,
               approx_cell2_size, marks=None):
    _check_num_threads(num_threads)
    s1 = _columns(sample1)
    s2 = s1 if sample2 is sample1 else _columns(sample2)
    rm = np.amax(r) if len(r) else 0.0
    pm = (np.amax(pi) if len(pi) else 0.0) if pi is not None else rm
    _approx_cells(approx_cell1_size, [rm, rm, pm], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rm, rm, pm], "approx_cell2_size")
    if marks is None:
        cond, keep = _cond()
    else:
        cond, keep = _cond(2, marks[2], marks[0], marks[1])
    x1, x2, box, pbc = _positions(s1, s2, period, [rm, rm, pm], [rm * 3.0, rm * 3.0, pm * 3.0])
    plan = _native.default_plan()
    out = np.ones(len(x1), dtype=np.uint8)
    r = np.ascontiguousarray(r, dtype=np.float64)
    pic = np.ascontiguousarray(pi, dtype=np.float64) if pi is not None else None
    pip = _native.pd(pic) if pic is not None else None
    plan.check(plan.lib.gbp_isolation(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.pd(r), pip,
        _native.pd(box), pbc, _native.ref(cond), _native.pu8(out)))
    del keep
    return out.astype(bool)


def spherical_isolation(sample1, sample2, r_max, period=None, num_threads=1,
                        approx_cell1_size=None, approx_cell2_size=None):
    """True for each ``sample1`` point with no ``sample2`` point at separation
    0 < s < r_max (spherical_isolation.py:27)."""
    r = _get_r_max(len(_columns(sample1)), r_max)
    return _isolation(sample1, sample2, r, None, period, num_threads, approx_cell1_size,
                      approx_cell2_size)


def cylindrical_isolation(sample1, sample2, rp_max, pi_max, period=None, num_threads=1,
                          approx_cell1_size=None, approx_cell2_size=None):
    """True for each ``sample1`` point with no ``sample2`` point in its cylinder
    dxy < rp_max, |dz| < pi_max at separation > 0 (cylindrical_isolation.py:28)."""
    n1 = len(_columns(sample1))
    return _isolation(sample1, sample2, _get_r_max(n1, rp_max), _get_r_max(n1, pi_max), period,
                      num_threads, approx_cell1_size, approx_cell2_size)


# isolation_functions_helpers.py:73-107: marks per point of each marking function
_COND_NMARKS = {0: 1, 1: 1, 2: 1, 3: 1, 4: 1, 5: 2, 6: 2}


def _func_signature_int_from_cond_func(cond_func):
    try:
        assert int(cond_func) == cond_func
    except Exception:
        raise ValueError("Your input ``cond_func`` parameter must be one of the integer values \n"
                         "associated with one of the marking functions for conditional "
                         "isolation.\n")
    if cond_func not in _COND_NMARKS:
        raise HalotoolsError("Your input ``cond_func`` = %i parameter must be one of the integer "
                             "values \nassociated with one of the marking functions for "
                             "conditional isolation.\n" % cond_func)
    return _COND_NMARKS[int(cond_func)]


def _reshape_input_marks(marks, npts, nm, cond_func):
    # isolation_functions_helpers.py:110-139
    if marks is None:
        return np.ones((npts, nm), dtype=np.float64)
    marks = np.atleast_1d(marks).astype(np.float64, copy=False)  # read only
    if len(marks.shape) == 1:
        marks = np.reshape(marks, (len(marks), 1))
    if marks.shape[0] != npts:
        raise ValueError("You must pass in an array of marks whose length \n"
                         "matches the number of points in your sample.\n"
                         "Your input sample has %i points, but your marks array has length = %i.\n"
                         % (npts, marks.shape[0]))
    if marks.shape[1] != nm:
        raise ValueError("The input value of ``cond_func`` = %i. "
                         "For this choice for the conditional isolation function,\n"
                         "there should be %i marks per point. \n"
                         "However, your input marks has %i points per mark.\n"
                         % (cond_func, nm, marks.shape[1]))
    return marks


def _marks(sample1, sample2, marks1, marks2, cond_func):
    nm = _func_signature_int_from_cond_func(cond_func)
    m1 = _reshape_input_marks(marks1, len(_columns(sample1)), nm, cond_func)
    m2 = _reshape_input_marks(marks2, len(_columns(sample2)), nm, cond_func)
    return m1, m2, int(cond_func)


def conditional_spherical_isolation(sample1, sample2, r_max, marks1=None, marks2=None,
                                    cond_func=0, period=None, num_threads=1,
                                    approx_cell1_size=None, approx_cell2_size=None):
    """As ``spherical_isolation``, counting only neighbours j with
    cond_func(marks1[i], marks2[j]) true (conditional_spherical_isolation.py:25)."""
    marks = _marks(sample1, sample2, marks1, marks2, cond_func)
    r = _get_r_max(len(_columns(sample1)), r_max)
    return _isolation(sample1, sample2, r, None, period, num_threads, approx_cell1_size,
                      approx_cell2_size, marks)


def conditional_cylindrical_isolation(sample1, sample2, rp_max, pi_max, marks1=None,
                                      marks2=None, cond_func=0, period=None, num_threads=1,
                                      approx_cell1_size=None, approx_cell2_size=None):
    """As ``cylindrical_isolation``, counting only neighbours j with
    cond_func(marks1[i], marks2[j]) true (conditional_cylindrical_isolation.py:25)."""
    marks = _marks(sample1, sample2, marks1, marks2, cond_func)
    n1 = len(_columns(sample1))
    return _isolation(sample1, sample2, _get_r_max(n1, rp_max), _get_r_max(n1, pi_max), period,
                      num_threads, approx_cell1_size, approx_cell2_size, marks)
