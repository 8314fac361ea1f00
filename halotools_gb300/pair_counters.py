"""Drop-in front-ends for halotools' pair counters, running on the GB300 engines.

Signatures, defaults, argument checks and error messages follow the
reference front-ends:

* ``npairs_3d``        halotools mock_observables/pair_counters/npairs_3d.py:20-213
* ``npairs_xy_z``      npairs_xy_z.py:20-237
* ``npairs_s_mu``      npairs_s_mu.py:20-209
* ``marked_npairs_3d`` marked_npairs_3d.py:25-326
* ``marked_npairs_xy_z`` marked_npairs_xy_z.py:23-333
* ``weighted_npairs_s_mu`` weighted_npairs_s_mu.py:22-230
* ``npairs_jackknife_xy_z`` npairs_jackknife_xy_z.py:23-170

``num_threads`` is validated as the reference does and then ignored (the GPU
is the parallel engine).  ``approx_cell1_size`` / ``approx_cell2_size`` are
validated and used only as hints: the GPU chooses its own cell grid, and the
counts do not depend on it.

Two deliberate differences, both for inputs the reference does not define:
periodic positions outside ``[0, period]`` and non-finite positions raise
``ValueError`` (the reference's mesh silently drops or mis-files them), and
bin edges must be non-negative with a positive maximum.
"""
from __future__ import annotations

import multiprocessing
import warnings

import numpy as np

from . import _native
from ._native import GBP_MEM_HOST

__all__ = ("npairs_3d", "npairs_xy_z", "npairs_s_mu", "marked_npairs_3d", "npairs_projected",
           "npairs_jackknife_3d", "npairs_per_object_3d", "marked_npairs_3d_channels",
           "HalotoolsError")


class HalotoolsError(Exception):
    """Raised for weight-shape errors, as halotools.custom_exceptions.HalotoolsError."""


_NUM_THREADS_MSG = "Input ``num_threads`` argument must be an integer or the string 'max'"
_PERIOD_MSG = "Input ``period`` must be a bounded positive number in all dimensions"


def _check_num_threads(num_threads):
    # npairs_3d.py:157-162
    if num_threads != 1 or not isinstance(num_threads, int):
        if isinstance(num_threads, str) and num_threads == "max":
            return multiprocessing.cpu_count()
        if not isinstance(num_threads, int):
            raise ValueError(_NUM_THREADS_MSG)
    return num_threads


def _is_strictly_increasing(a):
    # array_is_monotonic(a, strict=True) == 1 (utils/array_utils.py)
    return bool(np.all(np.diff(a) > 0))


def _bins(b, msg):
    b = np.atleast_1d(b).astype("f8")
    if not (b.ndim == 1 and len(b) > 1 and (len(b) <= 2 or _is_strictly_increasing(b))):
        raise ValueError(msg)
    return b


def _columns(sample):
    s = np.asarray(sample)
    if s.ndim != 2 or s.shape[1] < 3:
        raise ValueError("Input sample of points must be a Numpy ndarray of shape (Npts, 3).")
    return s


def _enclosing_box(s1, s2, min_size, same=False):
    # mesh_helpers.py:17-64: the smallest coordinate over both samples and all
    # three dimensions (in the input dtype) and the box = largest extent, padded
    # to min_size.  One reduction over each sample's three columns gives the same
    # minimum and maximum as the reference's six per-column reductions.
    x1 = s1[:, :3]
    x2 = x1 if same else s2[:, :3]
    lo = [np.min(x1)] if same else [np.min(x1), np.min(x2)]
    hi = [np.max(x1)] if same else [np.max(x1), np.max(x2)]
    xyzmin = np.min(lo)
    xyzmax = np.max(hi) - xyzmin
    lbox = np.array([xyzmax, xyzmax, xyzmax])
    min_size = np.atleast_1d(min_size)
    if np.any(lbox < min_size):
        lbox[(lbox < min_size)] = min_size[(lbox < min_size)]
    return xyzmin, lbox.astype(np.float64)


def _enclose_in_box(s1, s2, min_size, same=False):
    # mesh_helpers.py:17-64: both samples shifted by the smallest coordinate, in
    # the input dtype (a sample given twice is shifted once), and the box
    xyzmin, lbox = _enclosing_box(s1, s2, min_size, same)
    x1 = s1[:, :3] - xyzmin
    x2 = x1 if same else s2[:, :3] - xyzmin
    return x1, x2, lbox


def _period(period):
    p = np.atleast_1d(period).astype(float)
    if len(p) == 1:
        p = np.array([p[0]] * 3)
    if len(p) != 3 or not (np.all(p < np.inf) and np.all(p > 0)):
        raise ValueError(_PERIOD_MSG)
    return p


def _approx_cells(a, default, name):
    # npairs_3d.py:202-209 then mesh_helpers._set_approximate_cell_sizes
    if a is None:
        a = default
    elif np.size(a) == 1:
        a = [a, a, a]
    a = np.atleast_1d(a)
    if len(a) != 3 or a.ndim != 1:
        raise ValueError("Input ``%s`` must be a length-3 sequence" % name)
    return a


def _search_check(search, period):
    # rectangular_mesh.py:376-417
    for d, ax in enumerate("xyz"):
        if not (search[d] <= period[d] / 3.0):
            msg = ("\n The maximum length over which you search for pairs of points \n"
                   "cannot be larger than Lbox/3 in any dimension. \n"
                   "You tried to search for pairs out to a length of search_%slength = %.2f,\n"
                   "but the size of your box in this dimension is %speriod = %.2f.\n"
                   "If you need to count pairs on these length scales, \n"
                   "you should use a larger simulation.\n" % (ax, search[d], ax, period[d]))
            raise ValueError(msg)


def _positions(sample1, sample2, period, search, pbc_min_size):
    """Return contiguous float64 (N,3) arrays, box, pbc flag, auto flag."""
    s1 = _columns(sample1)
    same = sample2 is sample1
    s2 = s1 if same else _columns(sample2)
    if period is None:
        pbc = 0
        x1, x2, box = _enclose_in_box(s1, s2, pbc_min_size, same)
    else:
        pbc = 1
        box = _period(period)
        x1, x2 = s1[:, :3], s2[:, :3]
    x1 = np.ascontiguousarray(x1, dtype=np.float64)
    x2 = x1 if same else np.ascontiguousarray(x2, dtype=np.float64)
    if not same and x1.shape == x2.shape and np.array_equal(x1, x2):
        x2 = x1  # identical samples: the auto-correlation path gives the same counts
    _search_check(search, box)
    return x1, x2, np.ascontiguousarray(box, dtype=np.float64), pbc


def _nonneg(b, what):
    if np.any(b < 0) or not np.max(b) > 0:
        raise ValueError("Input ``%s`` must be non-negative with a positive maximum" % what)


def npairs_3d(sample1, sample2, rbins, period=None, num_threads=1, approx_cell1_size=None,
              approx_cell2_size=None):
    """Cumulative pair counts ``counts[k] = #(i, j)`` with separation ``<= rbins[k]``.

    Same inputs and output as halotools ``npairs_3d`` (npairs_3d.py:20): an
    int64 array of length ``len(rbins)``; ordered pairs, so auto-counts are
    doubled and include self-pairs.
    """
    _check_num_threads(num_threads)
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    rmax = np.max(rbins)
    _approx_cells(approx_cell1_size, [rmax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rmax] * 3, "approx_cell2_size")
    _nonneg(rbins, "rbins")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rmax] * 3, [rmax * 3.0] * 3)
    plan = _native.default_plan()
    out = np.zeros(len(rbins), dtype=np.int64)
    plan.check(plan.lib.gbp_npairs_3d(plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2),
                                      len(x2), _native.pd(rbins), len(rbins), _native.pd(box),
                                      pbc, GBP_MEM_HOST, _native.pi64(out)))
    return out


def npairs_xy_z(sample1, sample2, rp_bins, pi_bins, period=None, num_threads=1,
                approx_cell1_size=None, approx_cell2_size=None):
    """Cumulative (r_p, pi) pair counts, shape ``(len(rp_bins), len(pi_bins))``.

    Same inputs and output as halotools ``npairs_xy_z`` (npairs_xy_z.py:20);
    z is the line of sight.
    """
    _check_num_threads(num_threads)
    rp_bins = _bins(rp_bins, "Input ``rp_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    pi_bins = _bins(pi_bins, "Input ``pi_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    rpm, pim = np.max(rp_bins), np.max(pi_bins)
    _approx_cells(approx_cell1_size, [rpm, rpm, pim], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rpm, rpm, pim], "approx_cell2_size")
    _nonneg(rp_bins, "rp_bins")
    _nonneg(pi_bins, "pi_bins")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rpm, rpm, pim],
                                  [rpm * 3.0, rpm * 3.0, pim * 3.0])
    plan = _native.default_plan()
    out = np.zeros((len(rp_bins), len(pi_bins)), dtype=np.int64)
    plan.check(plan.lib.gbp_npairs_xy_z(plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2),
                                        len(x2), _native.pd(rp_bins), len(rp_bins),
                                        _native.pd(pi_bins), len(pi_bins), _native.pd(box), pbc,
                                        GBP_MEM_HOST, _native.pi64(out)))
    return out


def npairs_projected(sample1, sample2, rp_bins, pi_max, period=None, num_threads=1,
                     approx_cell1_size=None, approx_cell2_size=None):
    """Cumulative projected pair counts, length ``len(rp_bins)``: pairs with
    ``r_p <= rp_bins[k]`` and ``|pi| <= pi_max``.

    Same inputs and output as halotools ``npairs_projected``
    (npairs_projected.py:20-21). It is the ``pi_max`` column of the (r_p, pi)
    count with pi edges ``[0, pi_max]``: the projected engine tests the same
    squared quantities, ``dx*dx + dy*dy <= rp^2`` and ``dz*dz <= pi_max^2``
    (npairs_projected_engine.pyx), with the same cumulative walk over rp.
    """
    _check_num_threads(num_threads)
    rp_bins = _bins(rp_bins, "Input ``rp_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    rpm = np.max(rp_bins)
    _approx_cells(approx_cell1_size, [rpm, rpm, rpm], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rpm, rpm, rpm], "approx_cell2_size")
    msg = "Input ``pi_max`` must be a positive scalar less than period[2]/3"
    if period is None:
        pi_max_f = float(pi_max)
        _, box = _enclosing_box(_columns(sample1), _columns(sample2),
                                [rpm * 3.0, rpm * 3.0, pi_max_f * 3.0], sample2 is sample1)
    else:
        box = _period(period)
    if not (pi_max > 0.0 and pi_max < box[2] / 3.0):
        raise ValueError(msg)
    _nonneg(rp_bins, "rp_bins")
    counts = npairs_xy_z(sample1, sample2, rp_bins, np.array([0.0, float(pi_max)]), period=period,
                         num_threads=num_threads)
    return np.ascontiguousarray(counts[:, -1])


def npairs_s_mu(sample1, sample2, s_bins, mu_bins, period=None, num_threads=1,
                approx_cell1_size=None, approx_cell2_size=None):
    """Cumulative (s, mu) pair counts, shape ``(len(s_bins), len(mu_bins))``.

    Same inputs and output as halotools ``npairs_s_mu`` (npairs_s_mu.py:20):
    the second axis runs over ``sort(sin(arccos(mu_bins)))``
    (npairs_s_mu.py:174-175), i.e. increasing angle from the line of sight z.
    """
    _check_num_threads(num_threads)
    s_bins = _bins(s_bins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                           "least two entries")
    smax = np.max(s_bins)
    mu_bins = np.atleast_1d(mu_bins)
    if not (mu_bins.ndim == 1 and len(mu_bins) > 1 and
            (len(mu_bins) <= 2 or _is_strictly_increasing(mu_bins))):
        raise ValueError("\n Input `mu_bins` must be a monotonically increasing \n"
                         "1D array with at least two entries")
    _approx_cells(approx_cell1_size, [smax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [smax] * 3, "approx_cell2_size")
    _nonneg(s_bins, "s_bins")
    mu_prime = np.ascontiguousarray(np.sort(np.sin(np.arccos(mu_bins))), dtype=np.float64)
    x1, x2, box, pbc = _positions(sample1, sample2, period, [smax] * 3, [smax * 3.0] * 3)
    plan = _native.default_plan()
    out = np.zeros((len(s_bins), len(mu_prime)), dtype=np.int64)
    plan.check(plan.lib.gbp_npairs_s_mu(plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2),
                                        len(x2), _native.pd(s_bins), len(s_bins),
                                        _native.pd(mu_prime), len(mu_prime), _native.pd(box),
                                        pbc, GBP_MEM_HOST, _native.pi64(out)))
    return out


# marked_npairs_3d.py:281-326
_NUM_WEIGHTS = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 2, 11: 2,
                12: 4, 13: 4, 14: 3, 15: 3, 16: 5, 17: 5}


def _func_signature_int_from_wfunc(weight_func_id, known=None):
    known = _NUM_WEIGHTS if known is None else known
    if type(weight_func_id) != int:
        raise ValueError("\n weight_func_id parameter must be an integer ID of a weighting function.")
    if weight_func_id not in known:
        raise HalotoolsError("The value ``weight_func_id`` = %i is not recognized" % weight_func_id)
    return known[weight_func_id]


# marked_npairs_xy_z.py:292-333 knows ids 1-15 only
_NUM_WEIGHTS_XY_Z = {k: v for k, v in _NUM_WEIGHTS.items() if k <= 15}


def _process_weights(sample1, sample2, weights1, weights2, weight_func_id, known=None):
    """marked_npairs_3d.py:186-276 (and the same checks in marked_npairs_xy_z.py:
    192-289): shape checks and float64 (N, n_w) arrays."""
    nw = _func_signature_int_from_wfunc(weight_func_id, known)
    out = []
    for which, sample, w in ((1, sample1, weights1), (2, sample2, weights2)):
        npts = np.shape(sample)[0]
        shape = (npts, nw)
        conv = False
        if w is None:
            w = np.ones(shape, dtype=np.float64)
        else:
            w = np.atleast_1d(w).astype("float64", copy=False)  # read only
            if w.ndim == 1:
                conv = True
                w = w.reshape((len(w), 1))
            elif w.ndim != 2:
                raise HalotoolsError("\n You must either pass in a 1-D or 2-D array \n"
                                     "for the input `weights%d`. Instead, an array of \n"
                                     "dimension %i was received." % (which, w.ndim))
        if np.shape(w) != shape:
            if conv:
                raise HalotoolsError("\n You passed in a 1-D array for `weights%d` that \n"
                                     "does not have the correct length. The number of \n"
                                     "points in `sample%d` = %i, while the number of points \n"
                                     "in your input 1-D `weights%d` array = %i"
                                     % (which, which, npts, which, np.shape(w)[0]))
            raise HalotoolsError("\n You passed in a 2-D array for `weights%d` that \n"
                                 "does not have a consistent shape with `sample%d`. \n"
                                 "`sample%d` has length %i. The input value of `weight_func_id` = %i \n"
                                 "For this value of `weight_func_id`, there should be %i weights \n"
                                 "per point. The shape of your input `weights%d` is (%i, %i)\n"
                                 % (which, which, which, npts, weight_func_id, nw, which,
                                    np.shape(w)[0], np.shape(w)[1]))
        out.append(np.ascontiguousarray(w, dtype=np.float64))
    return out[0], out[1], nw


def marked_npairs_3d(sample1, sample2, rbins, weight_func_id, period=None, weights1=None,
                     weights2=None, num_threads=1, approx_cell1_size=None,
                     approx_cell2_size=None):
    """Cumulative weighted pair counts ``W(<r)`` (float64, length ``len(rbins)``).

    Same inputs and output as halotools ``marked_npairs_3d``
    (marked_npairs_3d.py:25); weights accumulate in FP32 with compensated
    (Kahan) partial sums, within 1e-6 relative of the FP64 reference for
    non-negative marks.
    """
    _check_num_threads(num_threads)
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    rmax = np.max(rbins)
    _approx_cells(approx_cell1_size, [rmax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rmax] * 3, "approx_cell2_size")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rmax] * 3, [rmax * 3.0] * 3)
    w1, w2, nw = _process_weights(sample1, sample2, weights1, weights2, weight_func_id)
    _nonneg(rbins, "rbins")
    if x2 is x1 and not (weights2 is weights1 or np.array_equal(w1, w2)):
        x2 = x1.copy()  # same points, different marks: count as a cross-correlation
    if x2 is x1:
        w2 = w1
    plan = _native.default_plan()
    out = np.zeros(len(rbins), dtype=np.float64)
    plan.check(plan.lib.gbp_marked_npairs_3d(plan.handle, _native.dptr(x1), len(x1),
                                             _native.dptr(x2), len(x2), _native.dptr(w1),
                                             _native.dptr(w2), nw, int(weight_func_id),
                                             _native.pd(rbins), len(rbins), _native.pd(box), pbc,
                                             GBP_MEM_HOST, _native.pd(out)))
    return out


def marked_npairs_xy_z(sample1, sample2, rp_bins, pi_bins, period=None, weights1=None,
                       weights2=None, weight_func_id=0, num_threads=1, approx_cell1_size=None,
                       approx_cell2_size=None):
    """Cumulative (r_p, pi) sums of a marking function, float64, shape
    ``(len(rp_bins), len(pi_bins))``.

    Same inputs and output as halotools ``marked_npairs_xy_z``
    (marked_npairs_xy_z.py:23); ``weight_func_id`` 1-15 as there.  Each pair's
    weight is added in FP32 with an exact-error companion (moved to FP64 every
    few thousand pairs): within 1e-6 relative of the FP64 reference, exact for
    integer-valued weights.
    """
    _check_num_threads(num_threads)
    rp_bins = _bins(rp_bins, "Input ``rp_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    pi_bins = _bins(pi_bins, "Input ``pi_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    rpm, pim = np.max(rp_bins), np.max(pi_bins)
    _approx_cells(approx_cell1_size, [rpm, rpm, pim], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rpm, rpm, pim], "approx_cell2_size")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rpm, rpm, pim],
                                  [rpm * 3.0, rpm * 3.0, pim * 3.0])
    w1, w2, nw = _process_weights(sample1, sample2, weights1, weights2, weight_func_id,
                                  _NUM_WEIGHTS_XY_Z)
    _nonneg(rp_bins, "rp_bins")
    _nonneg(pi_bins, "pi_bins")
    if x2 is x1 and not (weights2 is weights1 or np.array_equal(w1, w2)):
        x2 = x1.copy()  # same points, different marks: count as a cross-correlation
    if x2 is x1:
        w2 = w1
    plan = _native.default_plan()
    out = np.zeros((len(rp_bins), len(pi_bins)), dtype=np.float64)
    plan.check(plan.lib.gbp_marked_npairs_xy_z(plan.handle, _native.dptr(x1), len(x1),
                                               _native.dptr(x2), len(x2), _native.dptr(w1),
                                               _native.dptr(w2), nw, int(weight_func_id),
                                               _native.pd(rp_bins), len(rp_bins),
                                               _native.pd(pi_bins), len(pi_bins),
                                               _native.pd(box), pbc, GBP_MEM_HOST,
                                               _native.pd(out)))
    return out


def weighted_npairs_s_mu(sample1, sample2, weights1, weights2, s_bins, mu_bins, period=None,
                         num_threads=1, approx_cell1_size=None, approx_cell2_size=None):
    """Cumulative (s, mu) pair counts and w1 * w2 sums: ``(counts, weighted_counts)``,
    int64 and float64, each of shape ``(len(s_bins), len(mu_bins))``.

    Same inputs and outputs as halotools ``weighted_npairs_s_mu``
    (weighted_npairs_s_mu.py:22); the second axis runs over
    ``sort(sin(arccos(mu_bins)))`` (weighted_npairs_s_mu.py:192-193).  Counts are
    exact; sums within 1e-6 relative of the FP64 reference.
    """
    _check_num_threads(num_threads)
    s_bins = _bins(s_bins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                           "least two entries")
    smax = np.max(s_bins)
    _approx_cells(approx_cell1_size, [smax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [smax] * 3, "approx_cell2_size")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [smax] * 3, [smax * 3.0] * 3)
    # weighted_npairs_s_mu.py:171-176
    w1 = np.atleast_1d(weights1)
    w2 = np.atleast_1d(weights2)
    assert w1.shape == (len(x1),), "``weights1`` should have shape ({0}, )".format(len(x1))
    assert w2.shape == (len(x2),), "``weights2`` should have shape ({0}, )".format(len(x2))
    mu_bins = np.atleast_1d(mu_bins)
    if not (mu_bins.ndim == 1 and len(mu_bins) > 1 and
            (len(mu_bins) <= 2 or _is_strictly_increasing(mu_bins))):
        raise ValueError("\n Input `mu_bins` must be a monotonically increasing \n"
                         "1D array with at least two entries")
    _nonneg(s_bins, "s_bins")
    w1 = np.ascontiguousarray(w1, dtype=np.float64)
    w2 = np.ascontiguousarray(w2, dtype=np.float64)
    if x2 is x1 and not (weights2 is weights1 or np.array_equal(w1, w2)):
        x2 = x1.copy()  # same points, different weights: count as a cross-correlation
    if x2 is x1:
        w2 = w1
    mu_prime = np.ascontiguousarray(np.sort(np.sin(np.arccos(mu_bins))), dtype=np.float64)
    plan = _native.default_plan()
    counts = np.zeros((len(s_bins), len(mu_prime)), dtype=np.int64)
    wcounts = np.zeros((len(s_bins), len(mu_prime)), dtype=np.float64)
    plan.check(plan.lib.gbp_weighted_npairs_s_mu(plan.handle, _native.dptr(x1), len(x1),
                                                 _native.dptr(x2), len(x2), _native.dptr(w1),
                                                 _native.dptr(w2), _native.pd(s_bins),
                                                 len(s_bins), _native.pd(mu_prime),
                                                 len(mu_prime), _native.pd(box), pbc,
                                                 GBP_MEM_HOST, _native.pi64(counts),
                                                 _native.pd(wcounts)))
    return counts, wcounts


def marked_npairs_3d_channels(sample1, sample2, rbins, period=None, weights1=None,
                              weights2=None, num_threads=1, approx_cell1_size=None,
                              approx_cell2_size=None):
    """Product-mark counts over several mark channels in one pass.

    ``weights1`` / ``weights2``: (N, nch) arrays, nch <= 32 (a 1-D array is one
    channel). Returns (nch, len(rbins)) float64 whose row c equals
    ``marked_npairs_3d(sample1, sample2, rbins, 1, period, weights1[:, c],
    weights2[:, c])`` (marked_npairs_3d.py:25 with the product weight function,
    marking_functions.pyx:36-43): e.g. the random-mark draws of marked_tpcf
    (marked_tpcf.py:327-345) evaluated together. Each pair is binned once.
    """
    _check_num_threads(num_threads)
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    rmax = np.max(rbins)
    _approx_cells(approx_cell1_size, [rmax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rmax] * 3, "approx_cell2_size")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rmax] * 3, [rmax * 3.0] * 3)
    _nonneg(rbins, "rbins")

    def marks(w, n, name):
        if w is None:
            return np.ones((n, 1))
        w = np.asarray(w, dtype=np.float64)
        if w.ndim == 1:
            w = w[:, None]
        if w.ndim != 2 or w.shape[0] != n:
            raise HalotoolsError("``%s`` must have shape (N, nch) with N the number of "
                                 "points" % name)
        return np.ascontiguousarray(w)
    w1 = marks(weights1, len(x1), "weights1")
    w2 = marks(weights2, len(x2), "weights2") if weights2 is not None or x2 is not x1 else w1
    if w1.shape[1] != w2.shape[1]:
        raise HalotoolsError("``weights1`` and ``weights2`` must have the same number of channels")
    nch = w1.shape[1]
    if not 1 <= nch <= 32:
        raise ValueError("1 to 32 mark channels are supported, got %d" % nch)
    if x2 is x1 and not (w2 is w1 or np.array_equal(w1, w2)):
        x2 = x1.copy()  # same points, different marks: count as a cross-correlation
    if x2 is x1:
        w2 = w1
    plan = _native.default_plan()
    out = np.zeros((nch, len(rbins)), dtype=np.float64)
    plan.check(plan.lib.gbp_marked_npairs_3d_channels(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.dptr(w1),
        _native.dptr(w2), nch, _native.pd(rbins), len(rbins), _native.pd(box), pbc,
        GBP_MEM_HOST, _native.pd(out)))
    return out


def _jackknife_inputs(sample1, sample2, jtags1, jtags2, N_samples, weights1, weights2):
    """npairs_jackknife_3d.py / npairs_jackknife_xy_z.py weight and tag checks
    (_npairs_jackknife_xy_z_process_weights_jtags).  Returns the samples, tags and
    float64 weights (None when every weight is 1: the exact integer path)."""
    s1 = _columns(sample1)
    s2 = s1 if sample2 is sample1 else _columns(sample2)
    ws = []
    for w, s, name in ((weights1, s1, "weights1"), (weights2, s2, "weights2")):
        if w is not None:
            w = np.asarray(w).astype("float64", copy=False)  # read only
            if np.shape(w)[0] != np.shape(s)[0]:
                raise HalotoolsError("%s should have same len as %s" % (name, name.replace(
                    "weights", "sample")))
        ws.append(w)
    # (read only; one array given for both sides is converted and checked once)
    t1 = np.asarray(jtags1).astype("int", copy=False)
    t2 = t1 if jtags2 is jtags1 else np.asarray(jtags2).astype("int", copy=False)
    if np.shape(t1)[0] != np.shape(s1)[0]:
        raise HalotoolsError("jtags1 should have same len as sample1")
    if np.shape(t2)[0] != np.shape(s2)[0]:
        raise HalotoolsError("jtags2 should have same len as sample2")
    lo1 = np.min(t1) if len(t1) else None
    hi1 = np.max(t1) if len(t1) else None
    lo2, hi2 = (lo1, hi1) if t2 is t1 else ((np.min(t2), np.max(t2)) if len(t2) else (None, None))
    if lo1 is not None and lo1 < 1:
        raise HalotoolsError("jtags1 must be >= 1")
    if lo2 is not None and lo2 < 1:
        raise HalotoolsError("jtags2 must be >= 1")
    if hi1 is not None and hi1 > N_samples:
        raise HalotoolsError("jtags1 must be <= N_samples")
    if hi2 is not None and hi2 > N_samples:
        raise HalotoolsError("jtags2 must be <= N_samples")
    # np.unique(t1) == arange(1, N_samples + 1): with the tags checked to lie in
    # [1, N_samples], every subsample present (a count per tag when N_samples is
    # a whole number)
    if float(N_samples).is_integer():
        present = np.bincount(np.ravel(t1), minlength=int(N_samples) + 1)[1:] > 0
        every = len(present) == int(N_samples) and bool(np.all(present))
    else:
        every = np.array_equal(np.unique(t1), np.arange(1, N_samples + 1))
    if not every:
        warnings.warn("Warning: sample1 does not contain points in every jackknife sample.")
    w1, w2 = ws
    if (w1 is None or np.all(w1 == 1.0)) and (w2 is None or np.all(w2 == 1.0)):
        return s1, s2, t1, t2, None
    w1 = np.ones(len(s1)) if w1 is None else np.ascontiguousarray(w1.reshape(len(s1)))
    w2 = np.ones(len(s2)) if w2 is None else np.ascontiguousarray(w2.reshape(len(s2)))
    return s1, s2, t1, t2, (w1, w2)


def _jackknife_tags(x1, x2, t1, t2, wts=None):
    """int32 tag arrays; the same points with different tags (or weights) count as a
    cross-correlation."""
    j1 = np.ascontiguousarray(t1, dtype=np.int32)
    same_w = wts is None or np.array_equal(wts[0], wts[1])
    j2 = j1 if (x2 is x1 and (t2 is t1 or np.array_equal(t1, t2)) and same_w) else \
        np.ascontiguousarray(t2, dtype=np.int32)
    if x2 is x1 and j2 is not j1:
        x2 = x1.copy()
    return x1, x2, j1, j2


def _jackknife_weights(x1, x2, wts):
    """float64 weight arrays, shared when the auto-correlation shares its samples."""
    wa = np.ascontiguousarray(wts[0], dtype=np.float64)
    wb = wa if x2 is x1 else np.ascontiguousarray(wts[1], dtype=np.float64)
    return wa, wb


def npairs_jackknife_3d(sample1, sample2, rbins, jtags1, jtags2, N_samples, period=None,
                        weights1=None, weights2=None, num_threads=1, approx_cell1_size=None,
                        approx_cell2_size=None):
    """Jackknife pair counts, shape ``(N_samples + 1, len(rbins))``, float64.

    Same inputs and output as halotools ``npairs_jackknife_3d``
    (npairs_jackknife_3d.py:29-31): row 0 is the cumulative count of all pairs,
    row s the count with subsample s removed, where a pair with one end in s
    counts one half (npairs_jackknife_3d_engine.pyx:238-289). Exact for unit
    weights (the ``tpcf_jackknife`` case); other weights are summed per pair as
    w1 w2, within 1e-6 relative of the FP64 reference.
    """
    _check_num_threads(num_threads)
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    rmax = np.max(rbins)
    _approx_cells(approx_cell1_size, [rmax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rmax] * 3, "approx_cell2_size")
    s1, s2, t1, t2, wts = _jackknife_inputs(sample1, sample2, jtags1, jtags2, N_samples,
                                            weights1, weights2)
    _nonneg(rbins, "rbins")
    x1, x2, box, pbc = _positions(s1, s2, period, [rmax] * 3, [rmax * 3.0] * 3)
    x1, x2, j1, j2 = _jackknife_tags(x1, x2, t1, t2, wts)
    plan = _native.default_plan()
    out = np.zeros((int(N_samples) + 1, len(rbins)), dtype=np.float64)
    if wts is not None:
        wa, wb = _jackknife_weights(x1, x2, wts)
        plan.check(plan.lib.gbp_npairs_jackknife_3d_weighted(
            plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2),
            _native.dptr(wa), _native.dptr(wb), _native.dptr(j1), _native.dptr(j2),
            int(N_samples), _native.pd(rbins), len(rbins), _native.pd(box), pbc, GBP_MEM_HOST,
            _native.pd(out)))
        return out
    plan.check(plan.lib.gbp_npairs_jackknife_3d(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.dptr(j1),
        _native.dptr(j2), int(N_samples), _native.pd(rbins), len(rbins), _native.pd(box), pbc,
        GBP_MEM_HOST, _native.pd(out)))
    return out


def npairs_jackknife_xy_z(sample1, sample2, rp_bins, pi_bins, jtags1, jtags2, N_samples,
                          period=None, weights1=None, weights2=None, num_threads=1,
                          approx_cell1_size=None, approx_cell2_size=None):
    """Jackknife (r_p, pi) pair counts, shape ``(N_samples + 1, len(rp_bins),
    len(pi_bins))``, float64.

    Same inputs and output as halotools ``npairs_jackknife_xy_z``
    (npairs_jackknife_xy_z.py:23-26): row 0 counts all pairs, row s the pairs
    without subsample s, a pair with one end in s counting one half
    (npairs_jackknife_xy_z_engine.pyx:250-281).  Exact for unit weights; other
    weights are summed per pair as w1 w2, within 1e-6 relative of the FP64
    reference.
    """
    _check_num_threads(num_threads)
    rp_bins = _bins(rp_bins, "Input ``rp_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    pi_bins = _bins(pi_bins, "Input ``pi_bins`` must be a monotonically increasing 1D array "
                             "with at least two entries")
    rpm, pim = np.max(rp_bins), np.max(pi_bins)
    _approx_cells(approx_cell1_size, [rpm, rpm, pim], "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rpm, rpm, pim], "approx_cell2_size")
    s1, s2, t1, t2, wts = _jackknife_inputs(sample1, sample2, jtags1, jtags2, N_samples,
                                            weights1, weights2)
    _nonneg(rp_bins, "rp_bins")
    _nonneg(pi_bins, "pi_bins")
    x1, x2, box, pbc = _positions(s1, s2, period, [rpm, rpm, pim],
                                  [rpm * 3.0, rpm * 3.0, pim * 3.0])
    x1, x2, j1, j2 = _jackknife_tags(x1, x2, t1, t2, wts)
    plan = _native.default_plan()
    out = np.zeros((int(N_samples) + 1, len(rp_bins), len(pi_bins)), dtype=np.float64)
    if wts is not None:
        wa, wb = _jackknife_weights(x1, x2, wts)
        plan.check(plan.lib.gbp_npairs_jackknife_xy_z_weighted(
            plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2),
            _native.dptr(wa), _native.dptr(wb), _native.dptr(j1), _native.dptr(j2),
            int(N_samples), _native.pd(rp_bins), len(rp_bins), _native.pd(pi_bins),
            len(pi_bins), _native.pd(box), pbc, GBP_MEM_HOST, _native.pd(out)))
        return out
    plan.check(plan.lib.gbp_npairs_jackknife_xy_z(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.dptr(j1),
        _native.dptr(j2), int(N_samples), _native.pd(rp_bins), len(rp_bins),
        _native.pd(pi_bins), len(pi_bins), _native.pd(box), pbc, GBP_MEM_HOST,
        _native.pd(out)))
    return out


def npairs_per_object_3d(sample1, sample2, rbins, period=None, num_threads=1,
                         approx_cell1_size=None, approx_cell2_size=None):
    """Counts of ``sample2`` points around each point of ``sample1``, shape
    ``(Npts1, len(rbins))`` int64, as halotools ``npairs_per_object_3d``
    (npairs_per_object_3d.py:20-21): entry [i, k] counts j with separation
    <= rbins[k] (self pairs included when the samples coincide)."""
    _check_num_threads(num_threads)
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    rmax = np.max(rbins)
    _approx_cells(approx_cell1_size, [rmax] * 3, "approx_cell1_size")
    _approx_cells(approx_cell2_size, [rmax] * 3, "approx_cell2_size")
    x1, x2, box, pbc = _positions(sample1, sample2, period, [rmax] * 3, [rmax * 3.0] * 3)
    _nonneg(rbins, "rbins")
    plan = _native.default_plan()
    out = np.zeros((len(x1), len(rbins)), dtype=np.int64)
    plan.check(plan.lib.gbp_npairs_per_object_3d(
        plan.handle, _native.dptr(x1), len(x1), _native.dptr(x2), len(x2), _native.pd(rbins),
        len(rbins), _native.pd(box), pbc, GBP_MEM_HOST, _native.pi64(out)))
    return out
