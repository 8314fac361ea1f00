"""ctypes front-end of the C oracle (``oracle/pairs_oracle.c``).

TEST INFRASTRUCTURE: only the tests, the smoke check and the benchmark's CPU
baseline leg use this module.  It restates the argument processing of the
reference front-ends (halotools mock_observables/pair_counters/npairs_3d.py:153-213,
npairs_xy_z.py:166-237, npairs_s_mu.py:154-175, marked_npairs_3d.py:186-326)
just far enough to drive the C cell walks with the same inputs the reference
engines see, without validating user errors (the product's front-end does that).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pairs_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C oracle (unfused, left-to-right FP64) into ``oracle/liboracle.so``."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                        "-pthread", SRC, "-o", tmp, "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        d, i64, i = ctypes.c_double, ctypes.c_int64, ctypes.c_int
        pd, pi64 = P(d), P(i64)
        L.orc_npairs_3d.argtypes = [pd, i64, pd, i64, pd, i, pd, i, pd, pd, i, pi64]
        L.orc_npairs_xy_z.argtypes = [pd, i64, pd, i64, pd, i, pd, i, pd, i, pd, pd, i, pi64]
        L.orc_npairs_s_mu.argtypes = [pd, i64, pd, i64, pd, i, pd, i, pd, i, pd, pd, i, pi64]
        L.orc_marked_npairs_3d.argtypes = [pd, i64, pd, i64, pd, pd, i, i, pd, i, pd, i, pd, pd, i, pd]
        L.orc_marked_npairs_xy_z.argtypes = [pd, i64, pd, i64, pd, pd, i, i, pd, i, pd, i, pd,
                                             i, pd, pd, i, pd]
        L.orc_weighted_npairs_s_mu.argtypes = [pd, i64, pd, i64, pd, pd, pd, i, pd, i, pd, i,
                                               pd, pd, i, pi64, pd]
        L.orc_npairs_jackknife_xy_z.argtypes = [pd, i64, pd, i64, pd, pd, pi64, pi64, i, pd, i,
                                                pd, i, pd, i, pd, pd, i, pd]
        L.orc_npairs_jackknife_3d.argtypes = [pd, i64, pd, i64, pd, pd, pi64, pi64, i, pd, i,
                                              pd, i, pd, pd, i, pd]
        L.orc_neighbours.argtypes = [pd, i64, pd, i64, pd, pd, pd, pd, i, i, i, d, d, i, i, i,
                                     pd, i, pd, pd, i, pi64]
        L.orc_bf_npairs_3d.argtypes = [pd, i64, pd, i64, pd, i, pd, i, pi64]
        L.orc_weighted_adjoint_3d.argtypes = [pd, i64, pd, pd, i, pd, i, pd, i, pd]
        L.orc_weighted_per_object_3d.argtypes = [pd, i64, pd, i64, pd, pd, i, pd, i, i, pd]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _pi(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _geometry(sample1, sample2, search_max, period):
    """Columns, optional enclosing box (mesh_helpers.py:17-64), period array."""
    s1 = np.asarray(sample1)
    s2 = np.asarray(sample2)
    if period is None:
        pbc = 0
        x1, x2 = s1[:, :3], s2[:, :3]
        xyzmin = np.min([np.min(x1[:, 0]), np.min(x2[:, 0]), np.min(x1[:, 1]), np.min(x2[:, 1]),
                         np.min(x1[:, 2]), np.min(x2[:, 2])])
        xyzmax = np.max([np.max(x1), np.max(x2)]) - xyzmin
        x1 = x1 - xyzmin
        x2 = x2 - xyzmin
        lbox = np.array([xyzmax] * 3, dtype=np.float64)
        mins = np.asarray(search_max, dtype=np.float64) * 3.0
        lbox = np.where(lbox < mins, mins, lbox)
    else:
        pbc = 1
        x1, x2 = s1[:, :3], s2[:, :3]
        lbox = np.atleast_1d(period).astype(np.float64)
        if len(lbox) == 1:
            lbox = np.array([lbox[0]] * 3)
    x1 = np.ascontiguousarray(x1, dtype=np.float64)
    x2 = np.ascontiguousarray(x2, dtype=np.float64)
    return x1, x2, np.ascontiguousarray(lbox, dtype=np.float64), pbc


def _approx(a, default):
    if a is None:
        return np.asarray(default, dtype=np.float64)
    a = np.atleast_1d(a).astype(np.float64)
    if len(a) == 1:
        a = np.array([a[0]] * 3)
    return np.ascontiguousarray(a)


def _check(rc):
    if rc == -2:
        raise ValueError("cannot be larger than Lbox/3")
    if rc != 0:
        raise RuntimeError("oracle failure %d" % rc)


def npairs_3d(sample1, sample2, rbins, period=None, num_threads=1,
              approx_cell1_size=None, approx_cell2_size=None):
    rbins = np.ascontiguousarray(np.atleast_1d(rbins), dtype=np.float64)
    rmax = np.max(rbins)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rmax] * 3, period)
    a1 = _approx(approx_cell1_size, [rmax] * 3)
    a2 = _approx(approx_cell2_size, [rmax] * 3)
    out = np.zeros(len(rbins), dtype=np.int64)
    _check(lib().orc_npairs_3d(_p(x1), len(x1), _p(x2), len(x2), _p(rbins), len(rbins),
                               _p(lbox), pbc, _p(a1), _p(a2), int(num_threads), _pi(out)))
    return out


def npairs_xy_z(sample1, sample2, rp_bins, pi_bins, period=None, num_threads=1,
                approx_cell1_size=None, approx_cell2_size=None):
    rp = np.ascontiguousarray(np.atleast_1d(rp_bins), dtype=np.float64)
    pi = np.ascontiguousarray(np.atleast_1d(pi_bins), dtype=np.float64)
    rpm, pim = np.max(rp), np.max(pi)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rpm, rpm, pim], period)
    a1 = _approx(approx_cell1_size, [rpm, rpm, pim])
    a2 = _approx(approx_cell2_size, [rpm, rpm, pim])
    out = np.zeros((len(rp), len(pi)), dtype=np.int64)
    _check(lib().orc_npairs_xy_z(_p(x1), len(x1), _p(x2), len(x2), _p(rp), len(rp), _p(pi),
                                 len(pi), _p(lbox), pbc, _p(a1), _p(a2), int(num_threads),
                                 _pi(out)))
    return out


def npairs_s_mu(sample1, sample2, s_bins, mu_bins, period=None, num_threads=1,
                approx_cell1_size=None, approx_cell2_size=None):
    s = np.ascontiguousarray(np.atleast_1d(s_bins), dtype=np.float64)
    smax = np.max(s)
    mu_prime = np.ascontiguousarray(np.sort(np.sin(np.arccos(np.atleast_1d(mu_bins)))),
                                    dtype=np.float64)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [smax] * 3, period)
    a1 = _approx(approx_cell1_size, [smax] * 3)
    a2 = _approx(approx_cell2_size, [smax] * 3)
    out = np.zeros((len(s), len(mu_prime)), dtype=np.int64)
    _check(lib().orc_npairs_s_mu(_p(x1), len(x1), _p(x2), len(x2), _p(s), len(s), _p(mu_prime),
                                 len(mu_prime), _p(lbox), pbc, _p(a1), _p(a2), int(num_threads),
                                 _pi(out)))
    return out


NUM_WEIGHTS = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 2, 11: 2,
               12: 4, 13: 4, 14: 3, 15: 3, 16: 5, 17: 5}


def marked_npairs_3d(sample1, sample2, rbins, weight_func_id, period=None, weights1=None,
                     weights2=None, num_threads=1, approx_cell1_size=None, approx_cell2_size=None):
    rbins = np.ascontiguousarray(np.atleast_1d(rbins), dtype=np.float64)
    rmax = np.max(rbins)
    nw = NUM_WEIGHTS[weight_func_id]
    n1, n2 = len(sample1), len(sample2)
    w1 = np.ones((n1, nw)) if weights1 is None else np.asarray(weights1, dtype=np.float64).reshape(n1, nw)
    w2 = np.ones((n2, nw)) if weights2 is None else np.asarray(weights2, dtype=np.float64).reshape(n2, nw)
    w1 = np.ascontiguousarray(w1)
    w2 = np.ascontiguousarray(w2)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rmax] * 3, period)
    a1 = _approx(approx_cell1_size, [rmax] * 3)
    a2 = _approx(approx_cell2_size, [rmax] * 3)
    out = np.zeros(len(rbins), dtype=np.float64)
    _check(lib().orc_marked_npairs_3d(_p(x1), n1, _p(x2), n2, _p(w1), _p(w2), nw,
                                      int(weight_func_id), _p(rbins), len(rbins), _p(lbox), pbc,
                                      _p(a1), _p(a2), int(num_threads), _p(out)))
    return out


def marked_npairs_xy_z(sample1, sample2, rp_bins, pi_bins, weight_func_id, period=None,
                       weights1=None, weights2=None, num_threads=1, approx_cell1_size=None,
                       approx_cell2_size=None):
    """marked_npairs_xy_z.py:160-189 driving marked_npairs_xy_z_engine.pyx:209-224."""
    rp = np.ascontiguousarray(np.atleast_1d(rp_bins), dtype=np.float64)
    pi = np.ascontiguousarray(np.atleast_1d(pi_bins), dtype=np.float64)
    rpm, pim = np.max(rp), np.max(pi)
    nw = NUM_WEIGHTS[weight_func_id]
    n1, n2 = len(sample1), len(sample2)
    w1 = np.ones((n1, nw)) if weights1 is None else np.asarray(weights1, dtype=np.float64).reshape(n1, nw)
    w2 = np.ones((n2, nw)) if weights2 is None else np.asarray(weights2, dtype=np.float64).reshape(n2, nw)
    w1 = np.ascontiguousarray(w1)
    w2 = np.ascontiguousarray(w2)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rpm, rpm, pim], period)
    a1 = _approx(approx_cell1_size, [rpm, rpm, pim])
    a2 = _approx(approx_cell2_size, [rpm, rpm, pim])
    out = np.zeros((len(rp), len(pi)), dtype=np.float64)
    _check(lib().orc_marked_npairs_xy_z(_p(x1), n1, _p(x2), n2, _p(w1), _p(w2), nw,
                                        int(weight_func_id), _p(rp), len(rp), _p(pi), len(pi),
                                        _p(lbox), pbc, _p(a1), _p(a2), int(num_threads), _p(out)))
    return out


def weighted_npairs_s_mu(sample1, sample2, weights1, weights2, s_bins, mu_bins, period=None,
                         num_threads=1, approx_cell1_size=None, approx_cell2_size=None):
    """weighted_npairs_s_mu.py:175-230 driving weighted_npairs_s_mu_engine.pyx:186-255:
    returns (counts, weighted counts), both cumulative in s and mu'."""
    s = np.ascontiguousarray(np.atleast_1d(s_bins), dtype=np.float64)
    smax = np.max(s)
    mu_prime = np.ascontiguousarray(np.sort(np.sin(np.arccos(np.atleast_1d(mu_bins)))),
                                    dtype=np.float64)
    n1, n2 = len(sample1), len(sample2)
    w1 = np.ascontiguousarray(np.asarray(weights1, dtype=np.float64).reshape(n1))
    w2 = np.ascontiguousarray(np.asarray(weights2, dtype=np.float64).reshape(n2))
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [smax] * 3, period)
    a1 = _approx(approx_cell1_size, [smax] * 3)
    a2 = _approx(approx_cell2_size, [smax] * 3)
    out = np.zeros((len(s), len(mu_prime)), dtype=np.int64)
    wout = np.zeros((len(s), len(mu_prime)), dtype=np.float64)
    _check(lib().orc_weighted_npairs_s_mu(_p(x1), n1, _p(x2), n2, _p(w1), _p(w2), _p(s), len(s),
                                          _p(mu_prime), len(mu_prime), _p(lbox), pbc, _p(a1),
                                          _p(a2), int(num_threads), _pi(out), _p(wout)))
    return out, wout


def npairs_jackknife_xy_z(sample1, sample2, rp_bins, pi_bins, jtags1, jtags2, N_samples,
                          period=None, weights1=None, weights2=None, num_threads=1,
                          approx_cell1_size=None, approx_cell2_size=None):
    """npairs_jackknife_xy_z.py:23-170 driving npairs_jackknife_xy_z_engine.pyx:231-281:
    (N_samples + 1, len(rp_bins), len(pi_bins)) float64."""
    rp = np.ascontiguousarray(np.atleast_1d(rp_bins), dtype=np.float64)
    pi = np.ascontiguousarray(np.atleast_1d(pi_bins), dtype=np.float64)
    rpm, pim = np.max(rp), np.max(pi)
    n1, n2 = len(sample1), len(sample2)
    w1 = np.ones(n1) if weights1 is None else np.asarray(weights1, dtype=np.float64)
    w2 = np.ones(n2) if weights2 is None else np.asarray(weights2, dtype=np.float64)
    w1, w2 = np.ascontiguousarray(w1), np.ascontiguousarray(w2)
    t1 = np.ascontiguousarray(jtags1, dtype=np.int64)
    t2 = np.ascontiguousarray(jtags2, dtype=np.int64)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rpm, rpm, pim], period)
    a1 = _approx(approx_cell1_size, [rpm, rpm, pim])
    a2 = _approx(approx_cell2_size, [rpm, rpm, pim])
    out = np.zeros((int(N_samples) + 1, len(rp), len(pi)), dtype=np.float64)
    _check(lib().orc_npairs_jackknife_xy_z(_p(x1), n1, _p(x2), n2, _p(w1), _p(w2), _pi(t1),
                                           _pi(t2), int(N_samples), _p(rp), len(rp), _p(pi),
                                           len(pi), _p(lbox), pbc, _p(a1), _p(a2),
                                           int(num_threads), _p(out)))
    return out


def npairs_jackknife_3d(sample1, sample2, rbins, jtags1, jtags2, N_samples, period=None,
                        weights1=None, weights2=None, num_threads=1, approx_cell1_size=None,
                        approx_cell2_size=None):
    """npairs_jackknife_3d.py:29-160 driving npairs_jackknife_3d_engine.pyx:
    (N_samples + 1, len(rbins)) float64."""
    rb = np.ascontiguousarray(np.atleast_1d(rbins), dtype=np.float64)
    rmax = np.max(rb)
    n1, n2 = len(sample1), len(sample2)
    w1 = np.ones(n1) if weights1 is None else np.asarray(weights1, dtype=np.float64)
    w2 = np.ones(n2) if weights2 is None else np.asarray(weights2, dtype=np.float64)
    w1, w2 = np.ascontiguousarray(w1), np.ascontiguousarray(w2)
    t1 = np.ascontiguousarray(jtags1, dtype=np.int64)
    t2 = np.ascontiguousarray(jtags2, dtype=np.int64)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rmax] * 3, period)
    a1 = _approx(approx_cell1_size, [rmax] * 3)
    a2 = _approx(approx_cell2_size, [rmax] * 3)
    out = np.zeros((int(N_samples) + 1, len(rb)), dtype=np.float64)
    _check(lib().orc_npairs_jackknife_3d(_p(x1), n1, _p(x2), n2, _p(w1), _p(w2), _pi(t1), _pi(t2),
                                         int(N_samples), _p(rb), len(rb), _p(lbox), pbc, _p(a1),
                                         _p(a2), int(num_threads), _p(out)))
    return out


def _neighbours(sample1, sample2, r, pi, period, marks1=None, marks2=None, ckind=0, cfunc=0,
                lim=(0.0, 0.0), eq=(False, False), excl0=0, num_threads=1):
    n1, n2 = len(sample1), len(sample2)
    r = np.ascontiguousarray(r, dtype=np.float64)
    pic = None if pi is None else np.ascontiguousarray(pi, dtype=np.float64)
    rm = float(np.max(r)) if n1 else 0.0
    pm = (float(np.max(pic)) if n1 else 0.0) if pic is not None else rm
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rm, rm, pm], period)
    a1 = _approx(None, [rm, rm, pm])
    nm = 0
    m1 = m2 = np.zeros(1)
    if marks1 is not None:
        m1 = np.ascontiguousarray(marks1, dtype=np.float64).reshape(n1, -1)
        m2 = np.ascontiguousarray(marks2, dtype=np.float64).reshape(n2, -1)
        nm = m1.shape[1]
    out = np.zeros(max(n1, 1), dtype=np.int64)
    _check(lib().orc_neighbours(_p(x1), n1, _p(x2), n2, _p(r),
                                _p(pic) if pic is not None else None, _p(m1), _p(m2), nm,
                                int(ckind), int(cfunc), float(lim[0]), float(lim[1]),
                                int(bool(eq[0])), int(bool(eq[1])), int(excl0), _p(lbox), pbc,
                                _p(a1), _p(a1), int(num_threads), _pi(out)))
    return out[:n1]


def counts_in_cylinders(sample1, sample2, proj_search_radius, cylinder_half_length,
                        period=None, num_threads=1, condition=None, condition_args=()):
    """counts_in_cylinders.py:27-195 driving counts_in_cylinders_engine.pyx:255-281."""
    autocorr = sample2 is None
    s2 = sample1 if autocorr else sample2
    n1 = len(sample1)
    rp = np.zeros(n1) + np.atleast_1d(proj_search_radius).astype("f8") if \
        np.size(proj_search_radius) == 1 else np.asarray(proj_search_radius, dtype=np.float64)
    pi = np.zeros(n1) + np.atleast_1d(cylinder_half_length).astype("f8") if \
        np.size(cylinder_half_length) == 1 else np.asarray(cylinder_half_length, dtype=np.float64)
    kw = {}
    if condition == "mass_frac":
        eq = list(condition_args[3:]) + [False, False]
        kw = dict(marks1=condition_args[0], marks2=condition_args[1], ckind=1,
                  lim=condition_args[2], eq=eq[:2])
    c = _neighbours(sample1, s2, rp, pi, period, num_threads=num_threads, **kw)
    return c - 1 if autocorr else c


def isolation(sample1, sample2, r, pi=None, period=None, marks1=None, marks2=None, cond_func=None,
              num_threads=1):
    """spherical / cylindrical isolation (pi None: spheres), conditional with a
    marking function id when cond_func is given (isolation_functions/engines)."""
    kw = {}
    if cond_func is not None:
        kw = dict(marks1=marks1, marks2=marks2, ckind=2, cfunc=cond_func)
    c = _neighbours(sample1, sample2, r, pi, period, excl0=1, num_threads=num_threads, **kw)
    return c == 0


def spherical_isolation(sample1, sample2, r_max, period=None, num_threads=1):
    """spherical_isolation.py:27-113 driving spherical_isolation_engine.pyx:190-199."""
    r = np.zeros(len(sample1)) + np.asarray(r_max, dtype=np.float64)
    return isolation(sample1, sample2, r, None, period, num_threads=num_threads)


def cylindrical_isolation(sample1, sample2, rp_max, pi_max, period=None, num_threads=1):
    """cylindrical_isolation.py:28-137 driving cylindrical_isolation_engine.pyx:198-208."""
    n = len(sample1)
    return isolation(sample1, sample2, np.zeros(n) + np.asarray(rp_max, dtype=np.float64),
                     np.zeros(n) + np.asarray(pi_max, dtype=np.float64), period,
                     num_threads=num_threads)


def conditional_spherical_isolation(sample1, sample2, r_max, marks1=None, marks2=None,
                                    cond_func=0, period=None, num_threads=1):
    """conditional_spherical_isolation.py:25-150 (marked_spherical_isolation_engine.pyx)."""
    r = np.zeros(len(sample1)) + np.asarray(r_max, dtype=np.float64)
    return isolation(sample1, sample2, r, None, period, marks1, marks2, cond_func, num_threads)


def conditional_cylindrical_isolation(sample1, sample2, rp_max, pi_max, marks1=None, marks2=None,
                                      cond_func=0, period=None, num_threads=1):
    """conditional_cylindrical_isolation.py:25-160 (marked_cylindrical_isolation_engine.pyx)."""
    n = len(sample1)
    return isolation(sample1, sample2, np.zeros(n) + np.asarray(rp_max, dtype=np.float64),
                     np.zeros(n) + np.asarray(pi_max, dtype=np.float64), period, marks1, marks2,
                     cond_func, num_threads)


def brute_force_npairs_3d(sample1, sample2, rbins, period=None):
    """Mesh-free O(N1*N2) count; small inputs only."""
    rbins = np.ascontiguousarray(np.atleast_1d(rbins), dtype=np.float64)
    rmax = np.max(rbins)
    x1, x2, lbox, pbc = _geometry(sample1, sample2, [rmax] * 3, period)
    out = np.zeros(len(rbins), dtype=np.int64)
    _check(lib().orc_bf_npairs_3d(_p(x1), len(x1), _p(x2), len(x2), _p(rbins), len(rbins),
                                  _p(lbox), pbc, _pi(out)))
    return out


def weighted_adjoint_3d(xyz, w, rbins, period, gbar, num_threads=8):
    """FP64 dL/dw of sum_ij w_i w_j [d_ij <= r_k] for upstream gradient gbar (brute force)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    rbins = np.ascontiguousarray(rbins, dtype=np.float64)
    gbar = np.ascontiguousarray(gbar, dtype=np.float64)
    box = np.ascontiguousarray(np.broadcast_to(np.atleast_1d(period).astype(np.float64), (3,)))
    out = np.zeros(len(xyz), dtype=np.float64)
    _check(lib().orc_weighted_adjoint_3d(_p(xyz), len(xyz), _p(w), _p(rbins), len(rbins), _p(box),
                                         1, _p(gbar), int(num_threads), _p(out)))
    return out


def weighted_per_object_3d(xyz, w, rbins, period, num_threads=8):
    """FP64 (N, nb) table S[m, k] = sum_j w_j [d_mj <= r_k] over the cell walk
    (j = m included), auto-correlation of ``xyz`` in a periodic box.  From it:
    C_k = sum_m w_m S[m, k], dL/dw_m = 2 sum_k gbar_k S[m, k] and
    dC_k/dtheta = 2 sum_m S[m, k] dw_m/dtheta."""
    rbins = np.ascontiguousarray(np.atleast_1d(rbins), dtype=np.float64)
    x, _, lbox, pbc = _geometry(xyz, xyz, [np.max(rbins)] * 3, period)
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros((len(x), len(rbins)), dtype=np.float64)
    _check(lib().orc_weighted_per_object_3d(_p(x), len(x), _p(x), len(x), _p(w), _p(rbins),
                                            len(rbins), _p(lbox), pbc, int(num_threads), _p(out)))
    return out
