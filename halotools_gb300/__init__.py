"""GB300-native pair-counting engines for halotools' mock observables.

``npairs_3d``, ``npairs_xy_z``, ``npairs_s_mu`` and ``marked_npairs_3d`` keep
the halotools signatures (mock_observables/pair_counters/__init__.py:3-18) and
run on hand-written sm_103a CUDA kernels through the C ABI declared in
``include/gbpairs.h``.  ``install_into_halotools()`` rebinds the names that
halotools' estimators bound at import time, so ``tpcf``, ``wp``,
``rp_pi_tpcf``, ``s_mu_tpcf`` and ``marked_tpcf`` pick them up as drop-ins.
"""
from .pair_counters import (HalotoolsError, marked_npairs_3d, marked_npairs_3d_channels,
                            marked_npairs_xy_z, npairs_3d, npairs_jackknife_3d,
                            npairs_jackknife_xy_z,
                            npairs_per_object_3d, npairs_projected, npairs_s_mu, npairs_xy_z,
                            weighted_npairs_s_mu)
from ._native import GBPairsError, GBPairsUnavailable, Plan, default_plan
from .neighbours import (conditional_cylindrical_isolation, conditional_spherical_isolation,
                         counts_in_cylinders, cylindrical_isolation, spherical_isolation)
from .batched import BatchedCounter, npairs_3d_batched
from . import estimators

__all__ = ("npairs_3d", "npairs_xy_z", "npairs_s_mu", "marked_npairs_3d",
           "marked_npairs_3d_channels", "npairs_projected", "npairs_jackknife_3d",
           "npairs_per_object_3d", "marked_npairs_xy_z", "weighted_npairs_s_mu",
           "npairs_jackknife_xy_z", "counts_in_cylinders", "spherical_isolation",
           "cylindrical_isolation", "conditional_spherical_isolation",
           "conditional_cylindrical_isolation",
           "HalotoolsError", "GBPairsError", "GBPairsUnavailable", "Plan", "default_plan",
           "npairs_3d_batched", "BatchedCounter", "install_into_halotools", "estimators")

# module attribute -> our function, for every place halotools binds a counter
_BINDINGS = tuple([
    ("halotools.mock_observables.pair_counters", "npairs_3d", npairs_3d),
    ("halotools.mock_observables.pair_counters", "npairs_xy_z", npairs_xy_z),
    ("halotools.mock_observables.pair_counters", "npairs_s_mu", npairs_s_mu),
    ("halotools.mock_observables.pair_counters", "marked_npairs_3d", marked_npairs_3d),
    ("halotools.mock_observables.pair_counters", "npairs_projected", npairs_projected),
    ("halotools.mock_observables", "npairs_projected", npairs_projected),
    ("halotools.mock_observables.pair_counters", "npairs_jackknife_3d", npairs_jackknife_3d),
    ("halotools.mock_observables.pair_counters", "npairs_per_object_3d", npairs_per_object_3d),
    ("halotools.mock_observables.two_point_clustering.tpcf_jackknife", "npairs_jackknife_3d",
     npairs_jackknife_3d),
    ("halotools.mock_observables.pair_counters", "marked_npairs_xy_z", marked_npairs_xy_z),
    ("halotools.mock_observables.pair_counters", "weighted_npairs_s_mu", weighted_npairs_s_mu),
    ("halotools.mock_observables.pair_counters", "npairs_jackknife_xy_z", npairs_jackknife_xy_z),
    ("halotools.mock_observables", "counts_in_cylinders", counts_in_cylinders),
    ("halotools.mock_observables.counts_in_cells", "counts_in_cylinders", counts_in_cylinders),
    ("halotools.mock_observables", "spherical_isolation", spherical_isolation),
    ("halotools.mock_observables", "cylindrical_isolation", cylindrical_isolation),
    ("halotools.mock_observables", "conditional_spherical_isolation",
     conditional_spherical_isolation),
    ("halotools.mock_observables", "conditional_cylindrical_isolation",
     conditional_cylindrical_isolation),
    ("halotools.mock_observables.isolation_functions", "spherical_isolation", spherical_isolation),
    ("halotools.mock_observables.isolation_functions", "cylindrical_isolation",
     cylindrical_isolation),
    ("halotools.mock_observables.isolation_functions", "conditional_spherical_isolation",
     conditional_spherical_isolation),
    ("halotools.mock_observables.isolation_functions", "conditional_cylindrical_isolation",
     conditional_cylindrical_isolation),
] + [
    # the intrinsic-alignment estimators bind their plain and marked counters at
    # import time (their positional marked counters have no GPU form here and
    # stay halotools' own); a name a module does not import is left alone
    ("halotools.mock_observables.ia_correlations." + m, attr, fn)
    for m in ("ee_projected", "ed_projected", "ii_plus_projected", "ii_minus_projected",
              "gi_plus_projected", "gi_minus_projected")
    for attr, fn in (("marked_npairs_xy_z", marked_npairs_xy_z), ("npairs_xy_z", npairs_xy_z))
] + [
    ("halotools.mock_observables.ia_correlations." + m, attr, fn)
    for m in ("ee_3d", "ed_3d", "ee_3d_one_two_halo_decomp", "ed_3d_one_two_halo_decomp",
              "ii_plus_3d", "ii_minus_3d", "gi_plus_3d", "gi_minus_3d")
    for attr, fn in (("marked_npairs_3d", marked_npairs_3d), ("npairs_3d", npairs_3d))
] + [
    ("halotools.mock_observables", "npairs_3d", npairs_3d),
    ("halotools.mock_observables", "npairs_xy_z", npairs_xy_z),
    ("halotools.mock_observables", "npairs_s_mu", npairs_s_mu),
    ("halotools.mock_observables", "marked_npairs_3d", marked_npairs_3d),
    ("halotools.mock_observables.two_point_clustering.tpcf", "npairs_3d", npairs_3d),
    ("halotools.mock_observables.two_point_clustering.rp_pi_tpcf", "npairs_xy_z", npairs_xy_z),
    ("halotools.mock_observables.two_point_clustering.s_mu_tpcf", "npairs_s_mu", npairs_s_mu),
    ("halotools.mock_observables.two_point_clustering.marked_tpcf", "marked_npairs_3d",
     marked_npairs_3d),
    ("halotools.mock_observables.two_point_clustering.marked_tpcf", "npairs_3d", npairs_3d),
    ("halotools.mock_observables.two_point_clustering.angular_tpcf", "npairs_3d", npairs_3d),
    ("halotools.mock_observables.two_point_clustering.tpcf_one_two_halo_decomp", "npairs_3d",
     npairs_3d),
    ("halotools.mock_observables.two_point_clustering.tpcf_one_two_halo_decomp",
     "marked_npairs_3d", marked_npairs_3d),
    ("halotools.mock_observables.two_point_clustering.wp_jackknife", "npairs_jackknife_xy_z",
     npairs_jackknife_xy_z),
    ("halotools.mock_observables.two_point_clustering.rp_pi_tpcf_jackknife",
     "npairs_jackknife_xy_z", npairs_jackknife_xy_z),
    ("halotools.mock_observables.large_scale_density.large_scale_density_spherical_volume",
     "npairs_per_object_3d", npairs_per_object_3d),
    ("halotools.mock_observables.large_scale_density.large_scale_density_spherical_annulus",
     "npairs_per_object_3d", npairs_per_object_3d),
    ("halotools.mock_observables.void_statistics.underdensity_prob_func",
     "npairs_per_object_3d", npairs_per_object_3d),
])


def install_into_halotools(strict=True):
    """Point halotools' estimators at the GB300 counters; returns the rebound names.

    Without halotools (``import halotools`` fails) nothing is rebound and the
    list is empty.  With halotools importable, every module of the binding
    table is imported and its name rebound; a module that fails to import is
    reported: ``strict=True`` raises ImportError naming each such module and
    its error (after rebinding the others), ``strict=False`` warns instead.
    """
    import importlib
    import warnings
    try:
        importlib.import_module("halotools")
    except ImportError:
        return []
    done, failed = [], {}
    for mod_name, attr, fn in _BINDINGS:
        try:
            mod = importlib.import_module(mod_name)
        except Exception as exc:  # reported below, never dropped
            failed.setdefault(mod_name, "%s: %s" % (type(exc).__name__, exc))
            continue
        if hasattr(mod, attr):
            setattr(mod, attr, fn)
            done.append("%s.%s" % (mod_name, attr))
    if failed:
        msg = ("halotools is importable, but these modules failed to import and keep their "
               "CPU counters: " + "; ".join("%s (%s)" % kv for kv in sorted(failed.items())))
        if strict:
            raise ImportError(msg)
        warnings.warn(msg)
    return done
