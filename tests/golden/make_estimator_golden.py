"""Golden vectors for the estimator layer, made by running halotools' own
``tpcf``, ``rp_pi_tpcf``, ``wp``, ``s_mu_tpcf`` and ``marked_tpcf``
(two_point_clustering/*.py) over its own pair counters (the Cython engines built by
``oracle/build_ref.py``, imported through ``oracle/ref_loader.py``).

Inputs are regenerated from their seeds by ``estimator_inputs`` (shared with the
tests); each ``.npz`` stores the outputs and a SHA-256 of the inputs.

Usage (needs Cython and the halotools tree; not needed on the GPU machine)::

    python tests/golden/make_estimator_golden.py [--src /path/to/halotools/checkout]
"""
from __future__ import annotations

import argparse
import hashlib
import importlib
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "estimators")
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
from oracle import build_ref  # noqa: E402
warnings.filterwarnings("ignore")

L = 100.0
RBINS = np.logspace(-0.5, 1.0, 9)
RP_BINS = np.logspace(-0.5, 1.0, 8)
PI_BINS = np.linspace(0.0, 12.0, 7)
S_BINS = np.logspace(-0.3, 1.0, 7)
MU_BINS = np.linspace(0.0, 1.0, 6)

# name: (function, sample2?, randoms?, periodic?, estimator, do_auto, do_cross, extra)
CASES = {
    "tpcf_auto_natural_pbc": ("tpcf", False, False, True, "Natural", True, True, {}),
    "tpcf_auto_ls_pbc": ("tpcf", False, False, True, "Landy-Szalay", True, True, {}),
    "tpcf_cross_natural_pbc": ("tpcf", True, False, True, "Natural", True, True, {}),
    "tpcf_cross_only_hamilton_pbc": ("tpcf", True, False, True, "Hamilton", False, True, {}),
    "tpcf_auto_ls_randoms_nopbc": ("tpcf", False, True, False, "Landy-Szalay", True, True, {}),
    "tpcf_cross_ls_randoms_nopbc": ("tpcf", True, True, False, "Landy-Szalay", True, True, {}),
    "tpcf_auto_dp_randoms_pbc": ("tpcf", False, True, True, "Davis-Peebles", True, True, {}),
    "tpcf_auto_hewett_randoms_pbc": ("tpcf", False, True, True, "Hewett", True, True, {}),
    "tpcf_auto_rr_precomputed": ("tpcf", False, True, True, "Landy-Szalay", True, True, {"rr": True}),
    "rp_pi_auto_natural_pbc": ("rp_pi_tpcf", False, False, True, "Natural", True, True, {}),
    "rp_pi_cross_ls_randoms_nopbc": ("rp_pi_tpcf", True, True, False, "Landy-Szalay", True, True, {}),
    "wp_auto_natural_pbc": ("wp", False, False, True, "Natural", True, True, {}),
    "wp_cross_natural_pbc": ("wp", True, False, True, "Natural", True, True, {}),
    "wp_auto_ls_randoms_nopbc": ("wp", False, True, False, "Landy-Szalay", True, True, {}),
    "s_mu_auto_natural_pbc": ("s_mu_tpcf", False, False, True, "Natural", True, True, {}),
    "s_mu_cross_ls_randoms_nopbc": ("s_mu_tpcf", True, True, False, "Landy-Szalay", True, True, {}),
    "marked_auto_random_marks": ("marked_tpcf", False, False, True, None, True, True,
                                 {"normalize_by": "random_marks", "iterations": 1, "seed": 3}),
    "marked_auto_random_marks_5it": ("marked_tpcf", False, False, True, None, True, True,
                                     {"normalize_by": "random_marks", "iterations": 5, "seed": 3}),
    "marked_cross_random_marks_3it": ("marked_tpcf", True, False, True, None, True, True,
                                      {"normalize_by": "random_marks", "iterations": 3, "seed": 5}),
    "marked_cross_number_counts": ("marked_tpcf", True, False, True, None, True, True,
                                   {"normalize_by": "number_counts"}),
    "marked_auto_sum_2it": ("marked_tpcf", False, False, True, None, True, True,
                            {"normalize_by": "random_marks", "iterations": 2, "seed": 9,
                             "weight_func_id": 2}),
    "jackknife_auto_natural_pbc": ("tpcf_jackknife", False, True, True, "Natural", True, True,
                                   {"Nsub": [3, 3, 3]}),
    "jackknife_cross_ls_pbc": ("tpcf_jackknife", True, True, True, "Landy-Szalay", True, True,
                               {"Nsub": [2, 3, 2]}),
    "jackknife_auto_ls_nopbc": ("tpcf_jackknife", False, True, False, "Landy-Szalay", True, True,
                                {"Nsub": 3}),
}


def estimator_inputs(seed=7):
    """Clustered sample1 (centres + tight satellites), uniform sample2 and randoms."""
    rng = np.random.default_rng(seed)
    cen = rng.uniform(0, L, (300, 3))
    sat = cen[rng.integers(0, 300, 2700)] + rng.normal(0, 1.5, (2700, 3))
    s1 = np.mod(np.concatenate([cen, sat]), L)
    s2 = rng.uniform(0, L, (2000, 3))
    ran = rng.uniform(0, L, (5000, 3))
    m1 = rng.lognormal(0.0, 0.5, len(s1))
    m2 = rng.uniform(0.0, 1.0, len(s2))
    return s1, s2, ran, m1, m2


def input_sha():
    h = hashlib.sha256()
    for a in estimator_inputs():
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run_case(mods, name):
    fn, use2, useran, pbc, est, da, dc, extra = CASES[name]
    s1, s2, ran, m1, m2 = estimator_inputs()
    if fn == "marked_tpcf":
        out = mods["marked_tpcf"].marked_tpcf(
            s1, RBINS, sample2=s2 if use2 else None, marks1=m1, marks2=m2 if use2 else None,
            period=L, do_auto=da, do_cross=dc, **extra)
        return out if isinstance(out, tuple) else (out,)
    kw = dict(sample2=s2 if use2 else None, randoms=ran if useran else None,
              period=L if pbc else None, do_auto=da, do_cross=dc, estimator=est)
    if fn == "tpcf_jackknife":
        out = mods["tpcf_jackknife"].tpcf_jackknife(
            s1, ran, RBINS, sample2=s2 if use2 else None, period=L if pbc else None,
            do_auto=da, do_cross=dc, estimator=est, **extra)
        return out if isinstance(out, tuple) else (out,)
    if fn == "s_mu_tpcf":
        out = mods["s_mu_tpcf"].s_mu_tpcf(s1, S_BINS, MU_BINS, **kw)
        return out if isinstance(out, tuple) else (out,)
    if fn == "tpcf":
        if extra.get("rr"):
            # RR precomputed for 5000 randoms, as tpcf.py's docstring suggests
            rr = np.diff(mods["pc"].npairs_3d(ran, ran, RBINS, period=L))
            kw.update(RR_precomputed=rr, NR_precomputed=len(ran))
        out = mods["tpcf"].tpcf(s1, RBINS, **kw)
    elif fn == "rp_pi_tpcf":
        out = mods["rp_pi_tpcf"].rp_pi_tpcf(s1, RP_BINS, PI_BINS, **kw)
    else:
        out = mods["wp"].wp(s1, RP_BINS, 12.0, **kw)
    return out if isinstance(out, tuple) else (out,)


def load_reference(src):
    from oracle import ref_loader
    ns = ref_loader.load(src)
    ht = os.path.join(src, "halotools")
    pc = sys.modules["halotools.mock_observables.pair_counters"]
    # the package's __init__ would bind the front-end functions (pair_counters/__init__.py:3-18)
    for n in ("npairs_3d", "npairs_xy_z", "npairs_s_mu", "marked_npairs_3d", "npairs_projected",
              "npairs_jackknife_3d", "npairs_per_object_3d"):
        setattr(pc, n, getattr(ns, n))
    # catalog_analysis_helpers (jackknife subvolume labels) imports two names from
    # modules that need astropy.table; the functions used here touch neither
    em = types.ModuleType("halotools.empirical_models")
    em.enforce_periodicity_of_box = None
    sm = types.ModuleType("halotools.sim_manager")
    sm.__path__ = []
    sd = types.ModuleType("halotools.sim_manager.sim_defaults")
    sd.default_cosmology, sd.default_redshift = None, 0.0
    sys.modules.update({"halotools.empirical_models": em, "halotools.sim_manager": sm,
                        "halotools.sim_manager.sim_defaults": sd})
    ref_loader._pkg("halotools.mock_observables.two_point_clustering",
                    [os.path.join(ht, "mock_observables", "two_point_clustering")])
    base = "halotools.mock_observables.two_point_clustering."
    return {"pc": pc, "tpcf": importlib.import_module(base + "tpcf"),
            "rp_pi_tpcf": importlib.import_module(base + "rp_pi_tpcf"),
            "wp": importlib.import_module(base + "wp"),
            "s_mu_tpcf": importlib.import_module(base + "s_mu_tpcf"),
            "marked_tpcf": importlib.import_module(base + "marked_tpcf"),
            "tpcf_jackknife": importlib.import_module(base + "tpcf_jackknife")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=build_ref.DEFAULT_SRC)
    args = ap.parse_args()
    mods = load_reference(args.src)
    sha = input_sha()
    for name in CASES:
        outs = run_case(mods, name)
        os.makedirs(OUT, exist_ok=True)
        np.savez_compressed(os.path.join(OUT, "est_" + name + ".npz"), sha=sha,
                            n=len(outs), **{"out%d" % k: np.asarray(o) for k, o in enumerate(outs)})
        print(name, [np.asarray(o).shape for o in outs])


if __name__ == "__main__":
    main()
