"""ctypes binding of ``libgbpairs.so`` (declared in ``include/gbpairs.h``).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every counting call raises ``GBPairsUnavailable``.  There
is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

GBP_OK = 0
GBP_ERR_INVALID = -1
GBP_ERR_CUDA = -2
GBP_ERR_NOMEM = -3
GBP_ERR_RANGE = -4
GBP_ERR_NODEVICE = -5
GBP_MEM_HOST = 0
GBP_MEM_DEVICE = 1

EXPORTED = (
    "gbp_plan_create", "gbp_plan_destroy", "gbp_plan_set_stream", "gbp_plan_set_reach",
    "gbp_plan_last_error", "gbp_plan_stats", "gbp_npairs_3d", "gbp_npairs_xy_z",
    "gbp_npairs_s_mu", "gbp_marked_npairs_3d", "gbp_measure_fp32_peak",
    "gbp_npairs_3d_static", "gbp_batched_npairs_3d", "gbp_plan_set_graph", "gbp_plan_set_autotune",
    "gbp_plan_set_block", "gbp_marked_npairs_3d_channels", "gbp_npairs_jackknife_3d",
    "gbp_npairs_per_object_3d", "gbp_marked_npairs_xy_z", "gbp_weighted_npairs_s_mu",
    "gbp_npairs_jackknife_xy_z", "gbp_counts_in_cylinders", "gbp_cylinder_pairs",
    "gbp_isolation", "gbp_hod_mocks", "gbp_npairs_jackknife_3d_weighted",
    "gbp_npairs_jackknife_xy_z_weighted", "gbp_weighted_adjoint_3d_channels",
    "gbp_zheng07_weights_batched", "gbp_zheng07_vjp_batched",
    "gbp_weighted_adjoint_3d", "gbp_zheng07_weights", "gbp_zheng07_vjp", "gbp_plan_set_limits",
    "gbp_grid_describe", "gbp_npairs_3d_thresholds", "gbp_npairs_xy_z_thresholds",
    "gbp_npairs_3d_lut", "gbp_stencil_describe", "gbp_npairs_s_mu_tables",
)


class GBPairsUnavailable(RuntimeError):
    """The CUDA library or a GPU is missing; no fallback exists."""


class GBPairsError(RuntimeError):
    """A CUDA-side failure reported by the library."""


class Stats(ctypes.Structure):
    _fields_ = [
        ("candidate_pairs", ctypes.c_int64),
        ("recheck_pairs", ctypes.c_int64),
        ("cells", ctypes.c_int64 * 3),
        ("reach", ctypes.c_int32),
        ("stencil_cells", ctypes.c_int32),
        ("work_items", ctypes.c_int64),
        ("ms_build", ctypes.c_float),
        ("ms_count", ctypes.c_float),
        ("ms_total", ctypes.c_float),
        ("count_launches", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int32),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
        ("block", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["cells"] = list(self.cells)
        return d


class NeighCond(ctypes.Structure):
    """gbp_neigh_cond: the condition a neighbour pair must meet (include/gbpairs.h)."""
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("func", ctypes.c_int32),
        ("marks1", ctypes.c_void_p),
        ("marks2", ctypes.c_void_p),
        ("nmarks", ctypes.c_int32),
        ("lower_inclusive", ctypes.c_int32),
        ("upper_inclusive", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("lim", ctypes.c_double * 2),
    ]


_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and type the C-ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            # rebuilds only when a source changed (fingerprint stamp)
            try:
                path = _build.build()
            except Exception as exc:  # nvcc missing, compile error ...
                if not os.path.exists(path):
                    raise GBPairsUnavailable("cannot build libgbpairs.so: %s" % exc) from exc
                raise
        elif not os.path.exists(path):
            raise GBPairsUnavailable("libgbpairs.so not built: run halotools_gb300.build")
        try:
            L = ctypes.CDLL(path)
        except OSError as exc:
            raise GBPairsUnavailable("cannot load %s: %s" % (path, exc)) from exc
        P = ctypes.POINTER
        pd, pi64 = P(ctypes.c_double), P(ctypes.c_int64)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.gbp_plan_create.argtypes = [ctypes.c_int, P(vp)]
        L.gbp_plan_destroy.argtypes = [vp]
        L.gbp_plan_set_stream.argtypes = [vp, vp]
        L.gbp_plan_set_reach.argtypes = [vp, ctypes.c_int]
        L.gbp_plan_last_error.argtypes = [vp]
        L.gbp_plan_last_error.restype = ctypes.c_char_p
        L.gbp_plan_stats.argtypes = [vp, P(Stats)]
        L.gbp_npairs_3d.argtypes = [vp, vp, i64, vp, i64, pd, i32, pd, i32, i32, pi64]
        L.gbp_npairs_xy_z.argtypes = [vp, vp, i64, vp, i64, pd, i32, pd, i32, pd, i32, i32, pi64]
        L.gbp_npairs_s_mu.argtypes = [vp, vp, i64, vp, i64, pd, i32, pd, i32, pd, i32, i32, pi64]
        L.gbp_marked_npairs_3d.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, i32, pd, i32, pd,
                                           i32, i32, pd]
        L.gbp_marked_npairs_3d_channels.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, pd, i32,
                                                    pd, i32, i32, pd]
        L.gbp_npairs_jackknife_3d.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, pd, i32, pd, i32,
                                              i32, pd]
        L.gbp_npairs_per_object_3d.argtypes = [vp, vp, i64, vp, i64, pd, i32, pd, i32, i32, pi64]
        L.gbp_npairs_jackknife_3d_weighted.argtypes = [vp, vp, i64, vp, i64, vp, vp, vp, vp, i32,
                                                       pd, i32, pd, i32, i32, pd]
        L.gbp_npairs_jackknife_xy_z_weighted.argtypes = [vp, vp, i64, vp, i64, vp, vp, vp, vp,
                                                         i32, pd, i32, pd, i32, pd, i32, i32, pd]
        L.gbp_weighted_adjoint_3d_channels.argtypes = [vp, vp, i64, vp, i32, pd, i32, pd, i32,
                                                       i32, pd, vp]
        L.gbp_zheng07_weights_batched.argtypes = [vp, vp, i64, pd, i32, i32, vp]
        L.gbp_zheng07_vjp_batched.argtypes = [vp, vp, i64, pd, i32, vp, i32, pd]
        L.gbp_hod_mocks.argtypes = [vp, vp, vp, vp, vp, i64, pd, i32, ctypes.c_double,
                                    ctypes.c_uint64, i32, vp, i64, pi64]
        pcond = P(NeighCond)
        L.gbp_counts_in_cylinders.argtypes = [vp, vp, i64, vp, i64, pd, pd, pd, i32, pcond, pi64]
        L.gbp_cylinder_pairs.argtypes = [vp, vp, i64, vp, i64, pd, pd, pd, i32, pcond, pi64,
                                         P(ctypes.c_uint32)]
        L.gbp_isolation.argtypes = [vp, vp, i64, vp, i64, pd, pd, pd, i32, pcond,
                                    P(ctypes.c_uint8)]
        L.gbp_npairs_jackknife_xy_z.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, pd, i32, pd,
                                                i32, pd, i32, i32, pd]
        L.gbp_marked_npairs_xy_z.argtypes = [vp, vp, i64, vp, i64, vp, vp, i32, i32, pd, i32, pd,
                                             i32, pd, i32, i32, pd]
        L.gbp_weighted_npairs_s_mu.argtypes = [vp, vp, i64, vp, i64, vp, vp, pd, i32, pd, i32, pd,
                                               i32, i32, pi64, pd]
        L.gbp_measure_fp32_peak.argtypes = [vp, pd]
        L.gbp_npairs_3d_static.argtypes = [vp, i64, pd, i32, pd, i32, vp, vp]
        L.gbp_batched_npairs_3d.argtypes = [vp, vp, i32, pi64, i32, pd, i32, pd, i32, i32, pi64]
        L.gbp_plan_set_graph.argtypes = [vp, ctypes.c_int]
        L.gbp_weighted_adjoint_3d.argtypes = [vp, vp, i64, vp, pd, i32, pd, i32, i32, pd, vp]
        L.gbp_zheng07_weights.argtypes = [vp, vp, i64, pd, i32, vp]
        L.gbp_zheng07_vjp.argtypes = [vp, vp, i64, pd, vp, i32, pd]
        L.gbp_plan_set_autotune.argtypes = [vp, ctypes.c_int]
        L.gbp_plan_set_block.argtypes = [vp, ctypes.c_int]
        L.gbp_plan_set_limits.argtypes = [vp, i64, i64]
        L.gbp_grid_describe.argtypes = [pd, i32, pd, i64, i32, i32, i32, P(ctypes.c_int32)]
        L.gbp_npairs_3d_thresholds.argtypes = [pd, i32, pd, i32, i64, i32, i32,
                                               P(ctypes.c_float), P(ctypes.c_float), pd]
        pf = P(ctypes.c_float)
        L.gbp_npairs_xy_z_thresholds.argtypes = [pd, i32, pd, i32, pd, i32, i64, i32, i32,
                                                 pf, pf, pf, pf, pd]
        L.gbp_npairs_3d_lut.argtypes = [pd, i32, pd, i32, i64, i32, i32, pf,
                                        P(ctypes.c_int32), pf]
        L.gbp_stencil_describe.argtypes = [pd, i32, pd, i64, i32, i32, i32, i32,
                                           P(ctypes.c_int32), P(ctypes.c_int32)]
        L.gbp_npairs_s_mu_tables.argtypes = [pd, i32, pd, i32, pd, i32, i64, i32, i32, pf, pf, pf,
                                             pf, pf, pf, P(ctypes.c_int32), pf, pd]
        _lib = L
        return L


class Plan:
    """Owns one ``gbp_plan`` (stream + device workspace) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.gbp_plan_create(int(device), ctypes.byref(h))
        if rc == GBP_ERR_NODEVICE:
            raise GBPairsUnavailable("no CUDA device visible: the gbpairs engines need a GPU")
        if rc != GBP_OK:
            raise GBPairsError("gbp_plan_create failed with status %d" % rc)
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbp_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int):
        if rc == GBP_OK:
            return
        msg = self.lib.gbp_plan_last_error(self.handle).decode(errors="replace")
        if rc == GBP_ERR_RANGE:
            raise ValueError(msg)
        if rc == GBP_ERR_INVALID:
            raise ValueError(msg)
        raise GBPairsError("gbpairs failure %d: %s" % (rc, msg))

    def stats(self) -> dict:
        s = Stats()
        self.check(self.lib.gbp_plan_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def set_stream(self, stream_ptr):
        self.check(self.lib.gbp_plan_set_stream(self.handle, ctypes.c_void_p(stream_ptr)))

    def fp32_peak_tflops(self) -> float:
        v = ctypes.c_double()
        self.check(self.lib.gbp_measure_fp32_peak(self.handle, ctypes.byref(v)))
        return v.value

    def set_graph(self, enable: bool):
        self.check(self.lib.gbp_plan_set_graph(self.handle, int(bool(enable))))

    def set_autotune(self, enable: bool):
        self.check(self.lib.gbp_plan_set_autotune(self.handle, int(bool(enable))))

    def set_reach(self, reach: int):
        self.check(self.lib.gbp_plan_set_reach(self.handle, int(reach)))

    def set_limits(self, first_item_cap: int = 0, flush_after: int = 0):
        """Small capacities that make a small call take the item-overflow retry
        and the early histogram flush (0 = the defaults)."""
        self.check(self.lib.gbp_plan_set_limits(self.handle, int(first_item_cap),
                                                int(flush_after)))

    def set_block(self, block: int):
        """Fine cells per block edge of the two-level grid (1..4); 0 = automatic."""
        self.check(self.lib.gbp_plan_set_block(self.handle, int(block)))


_plans = {}


def default_plan(device: int = 0) -> Plan:
    with _lock:
        p = _plans.get(device)
    if p is None:
        p = Plan(device)
        with _lock:
            _plans[device] = p
    return p


def dptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def dptr_int(addr: int):
    return ctypes.c_void_p(int(addr))


def pd(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def pi64(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def pu32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def pu8(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def ref(obj):
    return ctypes.byref(obj)
