"""Batched pair counts: many mock realisations in one GPU launch.

The reference counts one sample per ``npairs_3d`` call (npairs_3d.py:20); an
analysis of many HOD realisations, or of many random-mark draws
(marked_tpcf.py:327-345), loops over calls.  ``npairs_3d_batched`` sorts all
mocks into one shared cell grid (cell key = mock * ncells + cell) and counts
every mock's auto-correlation in one persistent launch, with per-mock
histograms, optionally captured in a CUDA graph and with the stencil reach
picked by timing (autotune).  ``counts[m]`` is bit-identical to
``npairs_3d(mock_m, mock_m, rbins, period)``.
"""
from __future__ import annotations

import numpy as np

from . import _native
from .pair_counters import _bins, _nonneg, _period, _search_check

__all__ = ("npairs_3d_batched", "BatchedCounter")


def _pack(samples, offsets):
    if offsets is None:
        samples = [np.asarray(s) for s in samples]
        for s in samples:
            if s.ndim != 2 or s.shape[1] != 3:
                raise ValueError("every mock must be an (N, 3) array")
        f32 = all(s.dtype == np.float32 for s in samples)
        dt = np.float32 if f32 else np.float64
        offsets = np.zeros(len(samples) + 1, dtype=np.int64)
        offsets[1:] = np.cumsum([len(s) for s in samples])
        xyz = np.ascontiguousarray(np.concatenate(samples).astype(dt, copy=False)) if samples else \
            np.zeros((0, 3), dt)
    else:
        xyz = np.asarray(samples)
        if xyz.ndim != 2 or xyz.shape[1] != 3:
            raise ValueError("positions must be an (N, 3) array")
        f32 = xyz.dtype == np.float32
        xyz = np.ascontiguousarray(xyz, dtype=np.float32 if f32 else np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    return xyz, offsets, f32


class BatchedCounter:
    """A plan configured for repeated batched calls (graph capture, autotune)."""

    def __init__(self, device: int = 0, graph: bool = True, autotune: bool = True):
        self.plan = _native.Plan(device)
        self.plan.set_graph(graph)
        self.plan.set_autotune(autotune)

    def stats(self):
        return self.plan.stats()

    def __call__(self, samples, rbins, period, offsets=None):
        return npairs_3d_batched(samples, rbins, period, offsets=offsets, plan=self.plan)

    def count_device(self, xyz_dev, offsets, rbins, period, stream=None):
        """Positions already on the GPU: a contiguous (N, 3) float32/float64
        torch tensor on this plan's device; offsets is a host array."""
        rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with "
                             "at least two entries")
        _nonneg(rbins, "rbins")
        box = np.ascontiguousarray(_period(period), dtype=np.float64)
        _search_check([np.max(rbins)] * 3, box)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        if stream is not None:
            self.plan.set_stream(stream)
        f32 = str(xyz_dev.dtype) == "torch.float32"
        out = np.zeros((len(offsets) - 1, len(rbins)), dtype=np.int64)
        self.plan.check(self.plan.lib.gbp_batched_npairs_3d(
            self.plan.handle, _native.dptr_int(xyz_dev.data_ptr()), int(f32), _native.pi64(offsets),
            len(offsets) - 1, _native.pd(rbins), len(rbins), _native.pd(box), 1,
            _native.GBP_MEM_DEVICE, _native.pi64(out)))
        return out


def npairs_3d_batched(samples, rbins, period, offsets=None, plan=None):
    """Cumulative auto-correlation pair counts of each mock, shape (nmocks, len(rbins)).

    ``samples`` is a list of (N_m, 3) arrays, or one (N, 3) array with
    ``offsets`` (nmocks + 1 row offsets).  Periodic boxes only (``period``
    required), as for HOD mocks; float32 positions are upcast exactly on the
    GPU, as the reference's engine upcasts them (npairs_3d_engine.pyx:58-63).
    """
    if period is None:
        raise ValueError("npairs_3d_batched counts periodic mocks: pass period")
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    _nonneg(rbins, "rbins")
    box = np.ascontiguousarray(_period(period), dtype=np.float64)
    _search_check([np.max(rbins)] * 3, box)
    xyz, offsets, f32 = _pack(samples, offsets)
    nm = len(offsets) - 1
    plan = plan or _native.default_plan()
    out = np.zeros((nm, len(rbins)), dtype=np.int64)
    plan.check(plan.lib.gbp_batched_npairs_3d(
        plan.handle, _native.dptr(xyz), int(f32), _native.pi64(offsets), nm, _native.pd(rbins),
        len(rbins), _native.pd(box), 1, _native.GBP_MEM_HOST, _native.pi64(out)))
    return out
