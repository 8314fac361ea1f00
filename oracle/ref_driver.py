"""Driver of halotools' own compiled pair-counting engines, for machines that
have the compiled engines but not the halotools Python tree.

TEST INFRASTRUCTURE and the timed CPU reference of the benchmark: nothing on
the product path imports this module.  The engines themselves are the
reference's Cython (``cpairs/npairs_3d_engine.pyx``,
``cpairs/npairs_xy_z_engine.pyx``), compiled by ``oracle/build_ref.py`` into
``oracle/_ref``.  What a halotools front-end does around them is restated
here, because the front-end's Python files are not available where the
benchmark runs:

* the double mesh: ``sample1_cell_size`` and ``sample2_cell_sizes``
  (``pair_counters/rectangular_mesh.py:25-82``), ``RectangularMesh.__init__``
  (``:118-222``: cell counts, ``digitized_position`` ``:19-22``, the
  ``argsort`` of the cell ids and the ``searchsorted`` cell offsets) and the
  attributes of ``RectangularDoubleMesh`` the engines read (``:234-374``);
* the default cell sizes of ``npairs_3d.py:202-209`` and
  ``npairs_xy_z.py:226-233`` (the search lengths);
* the fan-out over cell1 ranges, ``_cell1_parallelization_indices``
  (``mesh_helpers.py:183-221``) with ``multiprocessing.Pool.map``
  (``npairs_3d.py:135-148``).

Periodic samples only (the benchmark workloads are periodic).  The counts do
not depend on the order of points within a cell, so the restated mesh gives
the reference's integer counts exactly; ``tests/test_ref_driver.py`` checks
that against the real front-ends where the halotools tree is present.

Two ways to run the engines:

* ``full_call`` -- the front-end's own structure: mesh, a ``functools.partial``
  holding the caller's arrays, a fresh ``Pool(num_threads)`` mapped over the
  cell1 ranges, partial counts summed;
* ``SlabCounter`` -- the same mesh built once, the points sorted once, and
  the engines run over contiguous slabs of cell1 ids (each slab split over
  the worker processes as the front-end splits the whole range), so that a
  bounded amount of work is timed per step and the slabs together count the
  whole workload exactly once.  The engines are given the pre-sorted arrays
  and an identity sort (a slice), which skips the per-call copies the
  front-end's engines make; this favours the CPU.
"""
from __future__ import annotations

import functools
import importlib
import math
import multiprocessing
import os
import sys
import sysconfig
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_ref")
PC = os.path.join("halotools", "mock_observables", "pair_counters")
BASE = "halotools.mock_observables.pair_counters"
MAX_CELLS = 50  # default_max_cells_per_dimension_cell1/2, rectangular_mesh.py:15-16


# ---------------------------------------------------------------------------
# the compiled engines
# ---------------------------------------------------------------------------

def engines_available() -> bool:
    """True when the reference's compiled engines for this platform are in
    ``oracle/_ref`` (or can be compiled there from its generated C++)."""
    from oracle import build_ref
    return build_ref.build_generated()


def _stub(name, path):
    if name in sys.modules:
        return sys.modules[name]
    mod = types.ModuleType(name)
    mod.__path__ = [path] if os.path.isdir(path) else []
    mod.__package__ = name
    sys.modules[name] = mod
    return mod


def load_engine(name: str):
    """The reference engine ``name`` (e.g. ``npairs_3d_engine``) from ``oracle/_ref``."""
    full = BASE + ".cpairs." + name
    if full in sys.modules:
        return getattr(sys.modules[full], name)
    if not engines_available():
        raise RuntimeError("the reference's compiled engines are not available here")
    _stub("halotools", os.path.join(BUILD, "halotools"))
    _stub("halotools.mock_observables", os.path.join(BUILD, "halotools", "mock_observables"))
    _stub(BASE, os.path.join(BUILD, PC))
    _stub(BASE + ".cpairs", os.path.join(BUILD, PC, "cpairs"))
    return getattr(importlib.import_module(full), name)


# ---------------------------------------------------------------------------
# the double mesh (restated)
# ---------------------------------------------------------------------------

def sample1_cell_size(period, search_length, approx_cell_size, max_cells=MAX_CELLS):
    """Cell size of mesh1 along one axis (rectangular_mesh.py:25-55)."""
    period = float(period)
    if search_length > period / 3.0:
        raise ValueError("Input ``search_length`` cannot exceed period/3")
    ndivs = max(int(math.floor(period / float(approx_cell_size))), 1)
    ndivs = min(max_cells, ndivs)
    nsearch = max(int(math.floor(period / float(search_length))), 1)
    ndivs = max(3, min(ndivs, nsearch))
    return period / float(ndivs)


def sample2_cell_sizes(period, cell1, approx_cell_size, max_cells=MAX_CELLS):
    """Cell size of mesh2 along one axis (rectangular_mesh.py:58-82)."""
    period = float(period)
    n1 = int(np.round(period / cell1))
    per1 = min(max_cells, max(1, int(np.round(cell1 / float(approx_cell_size)))))
    n2 = n1 * per1
    if n2 > max_cells:
        n2 = (max_cells // n1) * n1
    return period / float(n2)


class Mesh:
    """The attributes of ``RectangularMesh`` (rectangular_mesh.py:118-222)."""

    def __init__(self, x, y, z, periods, approx):
        self.npts = len(x)
        self.xperiod, self.yperiod, self.zperiod = (float(p) for p in periods)
        self.num_xdivs = max(int(np.round(self.xperiod / approx[0])), 1)
        self.num_ydivs = max(int(np.round(self.yperiod / approx[1])), 1)
        self.num_zdivs = max(int(np.round(self.zperiod / approx[2])), 1)
        self.ncells = self.num_xdivs * self.num_ydivs * self.num_zdivs
        self.xcell_size = self.xperiod / float(self.num_xdivs)
        self.ycell_size = self.yperiod / float(self.num_ydivs)
        self.zcell_size = self.zperiod / float(self.num_zdivs)

        def digit(p, size, n):  # digitized_position, rectangular_mesh.py:19-22
            ip = np.floor(p // size).astype(int)
            return np.where(ip >= n, n - 1, ip)
        ids = (digit(x, self.xcell_size, self.num_xdivs) * (self.num_ydivs * self.num_zdivs) +
               digit(y, self.ycell_size, self.num_ydivs) * self.num_zdivs +
               digit(z, self.zcell_size, self.num_zdivs))
        self.idx_sorted = np.ascontiguousarray(np.argsort(ids))
        first = np.searchsorted(ids, np.arange(self.ncells), sorter=self.idx_sorted)
        self.cell_id_indices = np.ascontiguousarray(np.append(first, self.npts))


class DoubleMesh:
    """The attributes of ``RectangularDoubleMesh`` that the engines read
    (rectangular_mesh.py:234-374), periodic."""

    def __init__(self, c1, c2, approx1, approx2, search, periods):
        self.xperiod, self.yperiod, self.zperiod = (float(p) for p in periods)
        self.search_xlength, self.search_ylength, self.search_zlength = (float(s) for s in search)
        self._PBCs = True
        for s, p in zip(search, periods):
            if s > p / 3.0:
                raise ValueError("cannot be larger than Lbox/3")
        a1 = [sample1_cell_size(p, s, a) for p, s, a in zip(periods, search, approx1)]
        self.mesh1 = Mesh(c1[0], c1[1], c1[2], periods, a1)
        cs1 = (self.mesh1.xcell_size, self.mesh1.ycell_size, self.mesh1.zcell_size)
        a2 = [sample2_cell_sizes(p, c, a) for p, c, a in zip(periods, cs1, approx2)]
        self.mesh2 = Mesh(c2[0], c2[1], c2[2], periods, a2)


class _Presorted:
    """A mesh view for pre-sorted columns: the same cells, an identity sort."""

    class _M:
        pass

    def __init__(self, dm: DoubleMesh):
        self.__dict__.update({k: v for k, v in dm.__dict__.items()
                              if k not in ("mesh1", "mesh2")})
        for nm in ("mesh1", "mesh2"):
            src, m = getattr(dm, nm), self._M()
            m.__dict__.update(src.__dict__)
            m.idx_sorted = slice(None)
            setattr(self, nm, m)


def cell1_ranges(first, last, nproc):
    """[first, last) split as ``_cell1_parallelization_indices`` splits [0, ncells)
    (mesh_helpers.py:183-221)."""
    cells = np.arange(first, last)
    if nproc <= 1 or len(cells) <= 1:
        return [(int(first), int(last))]
    parts = [a for a in np.array_split(cells, min(nproc, len(cells))) if len(a)]
    return [(int(a[0]), int(a[0] + len(a))) for a in parts]


def _geometry(kind, bins, bins2, period):
    periods = np.atleast_1d(np.asarray(period, dtype=np.float64))
    if len(periods) == 1:
        periods = np.repeat(periods, 3)
    rmax = float(np.max(bins))
    if kind == "3d":
        search = (rmax, rmax, rmax)
        args = (np.atleast_1d(bins).astype("f8"),)
        eng = "npairs_3d_engine"
    else:
        pmax = float(np.max(bins2))
        search = (rmax, rmax, pmax)
        args = (np.atleast_1d(bins).astype("f8"), np.atleast_1d(bins2).astype("f8"))
        eng = "npairs_xy_z_engine"
    return periods, search, args, eng


def _columns(s):
    s = np.asarray(s)
    return s[:, 0], s[:, 1], s[:, 2]


def full_call(kind, sample1, sample2, bins, bins2, period, num_threads):
    """One reference-structured call: mesh, partial over the caller's columns,
    a fresh Pool(num_threads) over the cell1 ranges (npairs_3d.py:117-148).
    Returns the cumulative counts (int64)."""
    periods, search, args, eng = _geometry(kind, bins, bins2, period)
    engine = load_engine(eng)
    c1, c2 = _columns(sample1), _columns(sample2)
    dm = DoubleMesh(c1, c2, search, search, search, periods)
    f = functools.partial(engine, dm, *c1, *c2, *args)
    tuples = cell1_ranges(0, dm.mesh1.ncells, num_threads)
    if len(tuples) > 1:
        _no_cuda_fork()
        with multiprocessing.get_context("fork").Pool(len(tuples)) as pool:
            res = pool.map(f, tuples)
        return np.sum(np.array(res), axis=0)
    return np.asarray(f(tuples[0]))


# worker state, inherited through fork by the SlabCounter's pool
_W = {}


def _slab_task(rng):
    return np.asarray(_W["f"](rng))


def _no_cuda_fork():
    t = sys.modules.get("torch")
    if t is not None and t.cuda.is_available() and t.cuda.is_initialized():
        raise RuntimeError("fork after CUDA initialisation; run the reference engines in a "
                           "process that has not touched the GPU")


class SlabCounter:
    """The workload cut into ``nslabs`` contiguous ranges of cell1 ids, each
    counted by the reference engine over ``nproc`` worker processes."""

    def __init__(self, kind, sample1, sample2, bins, bins2, period, nproc, nslabs):
        periods, search, args, eng = _geometry(kind, bins, bins2, period)
        engine = load_engine(eng)
        t0 = time.perf_counter()
        c1, c2 = _columns(sample1), _columns(sample2)
        dm = DoubleMesh(c1, c2, search, search, search, periods)
        s1 = [np.ascontiguousarray(c[dm.mesh1.idx_sorted], dtype=np.float64) for c in c1]
        s2 = [np.ascontiguousarray(c[dm.mesh2.idx_sorted], dtype=np.float64) for c in c2]
        self.setup_s = time.perf_counter() - t0  # mesh build and the sorted copies
        self.ncells = dm.mesh1.ncells
        self.nslabs = max(1, min(int(nslabs), self.ncells))
        self.nproc = nproc
        bounds = np.linspace(0, self.ncells, self.nslabs + 1).round().astype(int)
        self.slabs = [cell1_ranges(bounds[k], bounds[k + 1], nproc) for k in range(self.nslabs)]
        _no_cuda_fork()
        _W["f"] = functools.partial(engine, _Presorted(dm), *s1, *s2, *args)
        self.pool = multiprocessing.get_context("fork").Pool(nproc)

    def count(self, k):
        """Counts of slab ``k mod nslabs`` and the wall seconds they took."""
        t0 = time.perf_counter()
        res = self.pool.map(_slab_task, self.slabs[k % self.nslabs], chunksize=1)
        out = np.sum(np.array(res), axis=0)
        return out, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()
        _W.clear()


def platform_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX")
