"""Import the reference's own pair-counter front-ends with the engines built by
``oracle/build_ref.py``.

Test infrastructure only (golden-vector generation, oracle pinning).  Nothing
is copied: stub package objects point ``__path__`` at the read-only halotools
tree (for the ``.py`` front-ends) and at ``oracle/_ref`` (for the compiled
engines), so ``halotools/__init__.py`` and its astropy/h5py imports never run.
The one astropy symbol the front-ends import, ``NumpyRNGContext``
(halotools ``utils/array_utils.py:6``), is replaced by a small stand-in that
seeds and restores numpy's legacy global RNG.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_ref")
from oracle.build_ref import DEFAULT_SRC  # noqa: E402  (the one place the checkout path is set)


class NumpyRNGContext:
    """Seed numpy's legacy global RNG inside a ``with`` block, then restore it."""

    def __init__(self, seed):
        self.seed = seed

    def __enter__(self):
        self._state = np.random.get_state()
        np.random.seed(self.seed)

    def __exit__(self, *exc):
        np.random.set_state(self._state)


def _pkg(name: str, paths):
    mod = types.ModuleType(name)
    mod.__path__ = [p for p in paths if os.path.isdir(p)]
    mod.__package__ = name
    sys.modules[name] = mod
    return mod


def load(src_root: str = DEFAULT_SRC):
    """Return a namespace with the reference ``npairs_3d``, ``npairs_xy_z``,
    ``npairs_s_mu``, ``marked_npairs_3d`` and the brute-force ``pairs`` module."""
    if "halotools.mock_observables.pair_counters.npairs_3d" in sys.modules:
        return _namespace()
    from oracle import build_ref
    if not build_ref.build(src_root):
        raise RuntimeError("reference engines cannot be built here")

    if "astropy" not in sys.modules:
        astropy = types.ModuleType("astropy")
        utils = types.ModuleType("astropy.utils")
        misc = types.ModuleType("astropy.utils.misc")
        misc.NumpyRNGContext = NumpyRNGContext
        astropy.utils = utils
        utils.misc = misc
        sys.modules.update({"astropy": astropy, "astropy.utils": utils,
                            "astropy.utils.misc": misc})

    ht = os.path.join(src_root, "halotools")
    bt = os.path.join(BUILD, "halotools")
    pc = os.path.join("mock_observables", "pair_counters")
    _pkg("halotools", [ht])
    _pkg("halotools.utils", [os.path.join(ht, "utils")])
    _pkg("halotools.mock_observables", [os.path.join(ht, "mock_observables")])
    _pkg("halotools.mock_observables.pair_counters", [os.path.join(ht, pc)])
    cp = _pkg("halotools.mock_observables.pair_counters.cpairs",
              [os.path.join(ht, pc, "cpairs"), os.path.join(bt, pc, "cpairs")])
    mcp = _pkg("halotools.mock_observables.pair_counters.marked_cpairs",
               [os.path.join(ht, pc, "marked_cpairs"), os.path.join(bt, pc, "marked_cpairs")])
    base = "halotools.mock_observables.pair_counters"
    # the per-object engine imports halotools.utils.unsorting_indices, which
    # halotools/utils/__init__.py would bind from array_utils.py
    utils_mod = sys.modules["halotools.utils"]
    utils_mod.unsorting_indices = importlib.import_module(
        "halotools.utils.array_utils").unsorting_indices
    for name in ("npairs_3d_engine", "npairs_xy_z_engine", "npairs_s_mu_engine",
                 "npairs_projected_engine", "npairs_jackknife_3d_engine",
                 "npairs_per_object_3d_engine", "weighted_npairs_s_mu_engine",
                 "npairs_jackknife_xy_z_engine"):
        m = importlib.import_module(base + ".cpairs." + name)
        setattr(cp, name, getattr(m, name))
    m = importlib.import_module(base + ".marked_cpairs.marked_npairs_3d_engine")
    mcp.marked_npairs_3d_engine = m.marked_npairs_3d_engine
    m = importlib.import_module(base + ".marked_cpairs.marked_npairs_xy_z_engine")
    mcp.marked_npairs_xy_z_engine = m.marked_npairs_xy_z_engine
    # counts in cylinders and the isolation functions (engines bound on their packages)
    mo = os.path.join(ht, "mock_observables")
    mb = os.path.join(bt, "mock_observables")
    _pkg("halotools.mock_observables.counts_in_cells", [os.path.join(mo, "counts_in_cells")])
    ce = _pkg("halotools.mock_observables.counts_in_cells.engines",
              [os.path.join(mo, "counts_in_cells", "engines"),
               os.path.join(mb, "counts_in_cells", "engines")])
    _pkg("halotools.mock_observables.counts_in_cells.engines.conditions",
         [os.path.join(mo, "counts_in_cells", "engines", "conditions"),
          os.path.join(mb, "counts_in_cells", "engines", "conditions")])
    m = importlib.import_module("halotools.mock_observables.counts_in_cells.engines."
                                "counts_in_cylinders_engine")
    ce.counts_in_cylinders_engine = m.counts_in_cylinders_engine
    _pkg("halotools.mock_observables.isolation_functions", [os.path.join(mo, "isolation_functions")])
    ie = _pkg("halotools.mock_observables.isolation_functions.engines",
              [os.path.join(mo, "isolation_functions", "engines"),
               os.path.join(mb, "isolation_functions", "engines")])
    for name in ("spherical_isolation_engine", "cylindrical_isolation_engine",
                 "marked_spherical_isolation_engine", "marked_cylindrical_isolation_engine"):
        m = importlib.import_module("halotools.mock_observables.isolation_functions.engines." + name)
        setattr(ie, name, getattr(m, name))
    return _namespace()


def _namespace():
    base = "halotools.mock_observables.pair_counters"
    ns = types.SimpleNamespace()
    ns.npairs_3d = importlib.import_module(base + ".npairs_3d").npairs_3d
    ns.npairs_xy_z = importlib.import_module(base + ".npairs_xy_z").npairs_xy_z
    ns.npairs_s_mu = importlib.import_module(base + ".npairs_s_mu").npairs_s_mu
    ns.marked_npairs_3d = importlib.import_module(base + ".marked_npairs_3d").marked_npairs_3d
    ns.npairs_projected = importlib.import_module(base + ".npairs_projected").npairs_projected
    ns.npairs_jackknife_3d = importlib.import_module(
        base + ".npairs_jackknife_3d").npairs_jackknife_3d
    ns.npairs_per_object_3d = importlib.import_module(
        base + ".npairs_per_object_3d").npairs_per_object_3d
    ns.weighted_npairs_s_mu = importlib.import_module(
        base + ".weighted_npairs_s_mu").weighted_npairs_s_mu
    ns.marked_npairs_xy_z = importlib.import_module(
        base + ".marked_npairs_xy_z").marked_npairs_xy_z
    ns.npairs_jackknife_xy_z = importlib.import_module(
        base + ".npairs_jackknife_xy_z").npairs_jackknife_xy_z
    ns.counts_in_cylinders = importlib.import_module(
        "halotools.mock_observables.counts_in_cells.counts_in_cylinders").counts_in_cylinders
    iso = "halotools.mock_observables.isolation_functions."
    ns.spherical_isolation = importlib.import_module(iso + "spherical_isolation").spherical_isolation
    ns.cylindrical_isolation = importlib.import_module(
        iso + "cylindrical_isolation").cylindrical_isolation
    ns.conditional_spherical_isolation = importlib.import_module(
        iso + "conditional_spherical_isolation").conditional_spherical_isolation
    ns.conditional_cylindrical_isolation = importlib.import_module(
        iso + "conditional_cylindrical_isolation").conditional_cylindrical_isolation
    ns.pairs = importlib.import_module(base + ".pairs")
    ns.HalotoolsError = importlib.import_module("halotools.custom_exceptions").HalotoolsError
    return ns


def load_alignments(src_root: str = DEFAULT_SRC):
    """halotools' own intrinsic-alignment modules whose counters are the plain and
    marked ones (``ee_3d``, ``ee_projected``), over the reference's counters,
    loaded without ``ia_correlations/__init__.py`` (whose other modules need the
    positional marked engines).  Returns {name: module}."""
    ns = load(src_root)
    pc = sys.modules["halotools.mock_observables.pair_counters"]
    for name in ("npairs_3d", "npairs_xy_z", "marked_npairs_3d", "marked_npairs_xy_z"):
        setattr(pc, name, getattr(ns, name))
    name = "halotools.mock_observables.ia_correlations"
    _pkg(name, [os.path.join(src_root, "halotools", "mock_observables", "ia_correlations")])
    return {m: importlib.import_module(name + "." + m) for m in ("ee_3d", "ee_projected")}


def load_counter_users(src_root: str = DEFAULT_SRC):
    """The other halotools modules that bind a counter at import time and load
    without astropy: ``angular_tpcf`` and ``tpcf_one_two_halo_decomp`` (both over
    ``npairs_3d``; the latter also ``marked_npairs_3d``), the two large-scale
    density functions and ``underdensity_prob_func`` (over
    ``npairs_per_object_3d``).  Returns {name: module}."""
    load_estimators(src_root)
    mods = {}
    tpc = "halotools.mock_observables.two_point_clustering"
    for m in ("angular_tpcf", "tpcf_one_two_halo_decomp"):
        mods[m] = importlib.import_module(tpc + "." + m)
    for pkg, names in (("large_scale_density", ("large_scale_density_spherical_volume",
                                                "large_scale_density_spherical_annulus")),
                       ("void_statistics", ("underdensity_prob_func",))):
        name = "halotools.mock_observables." + pkg
        _pkg(name, [os.path.join(src_root, "halotools", "mock_observables", pkg)])
        for m in names:
            mods[m] = importlib.import_module(name + "." + m)
    return mods


def load_estimators(src_root: str = DEFAULT_SRC):
    """halotools' own estimator modules (``tpcf``, ``rp_pi_tpcf``, ``wp``,
    ``s_mu_tpcf``, ``marked_tpcf``) over the reference's counters, loaded
    without ``two_point_clustering/__init__.py`` (which reaches astropy through
    the jackknife helpers).  Returns {name: module}."""
    load(src_root)
    name = "halotools.mock_observables.two_point_clustering"
    _pkg(name, [os.path.join(src_root, "halotools", "mock_observables", "two_point_clustering")])
    return {m: importlib.import_module(name + "." + m)
            for m in ("tpcf", "rp_pi_tpcf", "wp", "s_mu_tpcf", "marked_tpcf")}
