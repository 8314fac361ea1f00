"""Golden vectors for the sibling counters (npairs_projected, npairs_jackknife_3d,
npairs_per_object_3d, marked_npairs_xy_z, weighted_npairs_s_mu,
npairs_jackknife_xy_z, counts_in_cylinders and the isolation functions), made by running
halotools' own front-ends and Cython engines (built by ``oracle/build_ref.py``,
imported by ``oracle/ref_loader.py``).

Inputs are regenerated from their seeds by ``sibling_inputs`` (shared with the
tests); each ``.npz`` stores the output and a SHA-256 of the inputs.

Usage (needs Cython and the halotools tree; not needed on the GPU machine)::

    python tests/golden/make_sibling_golden.py [--src /path/to/halotools/checkout]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "siblings")
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
from oracle import build_ref  # noqa: E402
warnings.filterwarnings("ignore")

L = 120.0
RBINS = np.logspace(-0.7, 1.1, 10)


def sibling_inputs(seed=11):
    """Clustered sample1, uniform sample2, jackknife tags by x-slab (5 slabs)."""
    rng = np.random.default_rng(seed)
    cen = rng.uniform(0, L, (250, 3))
    sat = cen[rng.integers(0, 250, 2250)] + rng.normal(0, 1.2, (2250, 3))
    s1 = np.mod(np.concatenate([cen, sat]), L)
    s2 = rng.uniform(0, L, (1800, 3))
    t1 = 1 + np.minimum((s1[:, 0] / (L / 5)).astype(int), 4)
    t2 = 1 + np.minimum((s2[:, 0] / (L / 5)).astype(int), 4)
    return s1, s2, t1, t2


def sibling_weights(seed=12):
    """One float mark per point (lognormal for sample1, uniform for sample2) and a
    two-column mark (uniform in [0, 3) and [0, 1)) for the two-weight functions."""
    s1, s2, _, _ = sibling_inputs()
    rng = np.random.default_rng(seed)
    w1 = rng.lognormal(0.0, 0.5, len(s1))
    w2 = rng.uniform(0.0, 1.0, len(s2))
    W1 = np.stack([rng.uniform(0, 3, len(s1)), rng.uniform(0, 1, len(s1))], axis=1)
    W2 = np.stack([rng.uniform(0, 3, len(s2)), rng.uniform(0, 1, len(s2))], axis=1)
    return w1, w2, W1, W2


def neigh_inputs(seed=13):
    """Per-point radii (sphere r, cylinder rp and pi), masses and two-column marks."""
    s1, s2, _, _ = sibling_inputs()
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.5, 5.0, len(s1))
    rp = rng.uniform(0.5, 4.0, len(s1))
    pi = rng.uniform(1.0, 8.0, len(s1))
    # (arithmetic only: a libm power may round differently on another platform,
    # which would change the inputs' hash)
    m1 = rng.uniform(1.0, 1.0e4, len(s1))
    m2 = rng.uniform(1.0, 1.0e4, len(s2))
    k1 = rng.uniform(0, 3, (len(s1), 2))
    k2 = rng.uniform(0, 3, (len(s2), 2))
    return r, rp, pi, m1, m2, k1, k2


def input_sha():
    h = hashlib.sha256()
    for a in sibling_inputs() + sibling_weights() + neigh_inputs():
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


RP = np.logspace(-0.7, 1.1, 10)
PI = np.linspace(0.0, 12.0, 7)
SB = np.logspace(-0.5, 1.1, 9)
MU = np.linspace(0.0, 1.0, 11)


def _wt():
    return sibling_weights()


def _nb():
    return neigh_inputs()


def _sorted_pairs(r):
    """(counts, pair list): the pairs as an (n, 2) uint32 array sorted by (i1, i2)."""
    counts, idx = r
    idx = np.sort(np.asarray(idx), order=["i1", "i2"])
    return np.asarray(counts), np.stack([idx["i1"], idx["i2"]], axis=1).astype(np.uint32)


# name -> (front-end, call); calls take the module (halotools' or this package's)
CASES = {
    "projected_auto_pbc": ("npairs_projected", lambda m, s1, s2, t1, t2: m.npairs_projected(
        s1, s1, RBINS, 8.0, period=L)),
    "projected_cross_nopbc": ("npairs_projected", lambda m, s1, s2, t1, t2: m.npairs_projected(
        s1, s2, RBINS, 6.5)),
    "jackknife_auto_pbc": ("npairs_jackknife_3d", lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s1, RBINS, t1, t1, 5, period=L)),
    "jackknife_cross_pbc": ("npairs_jackknife_3d", lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s2, RBINS, t1, t2, 5, period=L)),
    "jackknife_auto_nopbc": ("npairs_jackknife_3d", lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s1, RBINS, t1, t1, 5)),
    "per_object_cross_pbc": ("npairs_per_object_3d", lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s1[:700], s2, RBINS, period=L)),
    "per_object_auto_pbc": ("npairs_per_object_3d", lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s1, s1, RBINS, period=L)),
    "per_object_cross_nopbc": ("npairs_per_object_3d", lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s2[:500], s1, RBINS)),
    "marked_xy_z_id1_auto_pbc": ("marked_npairs_xy_z", lambda m, s1, s2, t1, t2: m.marked_npairs_xy_z(
        s1, s1, RP, PI, weights1=_wt()[0], weights2=_wt()[0], weight_func_id=1, period=L)),
    "marked_xy_z_id5_cross_nopbc": ("marked_npairs_xy_z", lambda m, s1, s2, t1, t2: m.marked_npairs_xy_z(
        s1, s2, RP, PI, weights1=_wt()[2], weights2=_wt()[3], weight_func_id=5)),
    "marked_xy_z_id9_auto_pbc": ("marked_npairs_xy_z", lambda m, s1, s2, t1, t2: m.marked_npairs_xy_z(
        s1, s1, RP, PI, weights1=_wt()[2], weights2=_wt()[2], weight_func_id=9, period=L)),
    "marked_xy_z_id2_cross_pbc": ("marked_npairs_xy_z", lambda m, s1, s2, t1, t2: m.marked_npairs_xy_z(
        s1, s2, RP, PI, weights1=_wt()[0], weights2=_wt()[1], weight_func_id=2, period=L)),
    "marked_xy_z_threes_auto_pbc": ("marked_npairs_xy_z", lambda m, s1, s2, t1, t2: m.marked_npairs_xy_z(
        s1, s1, RP, PI, weights1=np.full(len(s1), 3.0), weights2=np.full(len(s1), 3.0),
        weight_func_id=1, period=L)),
    "jackknife_w_auto_pbc": ("npairs_jackknife_3d", lambda m, s1, s2, t1, t2:
                             m.npairs_jackknife_3d(s1, s1, RBINS, t1, t1, 5, period=L,
                                                   weights1=_wt()[2][:, 0],
                                                   weights2=_wt()[2][:, 0])),
    "jackknife_w_cross_nopbc": ("npairs_jackknife_3d", lambda m, s1, s2, t1, t2:
                                m.npairs_jackknife_3d(s1, s2, RBINS, t1, t2, 5,
                                                      weights1=_wt()[2][:, 0],
                                                      weights2=_wt()[3][:, 0])),
    "jackknife_xy_z_w_auto_pbc": ("npairs_jackknife_xy_z", lambda m, s1, s2, t1, t2:
                                  m.npairs_jackknife_xy_z(s1, s1, RP, PI, t1, t1, 5, period=L,
                                                          weights1=_wt()[2][:, 1],
                                                          weights2=_wt()[2][:, 1])),
    "jackknife_xy_z_auto_pbc": ("npairs_jackknife_xy_z", lambda m, s1, s2, t1, t2:
                                m.npairs_jackknife_xy_z(s1, s1, RP, PI, t1, t1, 5, period=L)),
    "jackknife_xy_z_cross_pbc": ("npairs_jackknife_xy_z", lambda m, s1, s2, t1, t2:
                                 m.npairs_jackknife_xy_z(s1, s2, RP, PI, t1, t2, 5, period=L)),
    "jackknife_xy_z_auto_nopbc": ("npairs_jackknife_xy_z", lambda m, s1, s2, t1, t2:
                                  m.npairs_jackknife_xy_z(s1, s1, RP, PI, t1, t1, 5)),
    "cic_auto_pbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2: m.counts_in_cylinders(
        s1, None, _nb()[1], _nb()[2], period=L)),
    "cic_cross_pbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2: m.counts_in_cylinders(
        s1, s2, _nb()[1], _nb()[2], period=L)),
    "cic_cross_scalar_nopbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2:
                               m.counts_in_cylinders(s1, s2, 2.5, 6.0)),
    "cic_mass_frac_pbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2: m.counts_in_cylinders(
        s1, s2, _nb()[1], _nb()[2], period=L, condition="mass_frac",
        condition_args=(_nb()[3], _nb()[4], (0.1, 2.0), True, False))),
    "cic_indexes_auto_pbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2: _sorted_pairs(
        m.counts_in_cylinders(s1, None, _nb()[1], _nb()[2], period=L, return_indexes=True))),
    "cic_indexes_cross_nopbc": ("counts_in_cylinders", lambda m, s1, s2, t1, t2: _sorted_pairs(
        m.counts_in_cylinders(s2, s1, 1.5, 4.0, return_indexes=True))),
    "iso_sph_cross_pbc": ("spherical_isolation", lambda m, s1, s2, t1, t2: m.spherical_isolation(
        s1, s2, _nb()[0], period=L)),
    "iso_sph_auto_pbc": ("spherical_isolation", lambda m, s1, s2, t1, t2: m.spherical_isolation(
        s1, s1, _nb()[0], period=L)),
    "iso_sph_cross_nopbc": ("spherical_isolation", lambda m, s1, s2, t1, t2: m.spherical_isolation(
        s1, s2, _nb()[0])),
    "iso_cyl_cross_pbc": ("cylindrical_isolation", lambda m, s1, s2, t1, t2:
                          m.cylindrical_isolation(s1, s2, _nb()[1], _nb()[2], period=L)),
    "iso_cyl_auto_pbc": ("cylindrical_isolation", lambda m, s1, s2, t1, t2:
                         m.cylindrical_isolation(s1, s1, _nb()[1], _nb()[2], period=L)),
    "iso_csph_f1_pbc": ("conditional_spherical_isolation", lambda m, s1, s2, t1, t2:
                        m.conditional_spherical_isolation(s1, s2, _nb()[0], _nb()[5][:, 0],
                                                          _nb()[6][:, 0], 1, period=L)),
    "iso_csph_f6_auto_pbc": ("conditional_spherical_isolation", lambda m, s1, s2, t1, t2:
                             m.conditional_spherical_isolation(s1, s1, _nb()[0], _nb()[5],
                                                               _nb()[5], 6, period=L)),
    "iso_ccyl_f2_pbc": ("conditional_cylindrical_isolation", lambda m, s1, s2, t1, t2:
                        m.conditional_cylindrical_isolation(s1, s2, _nb()[1], _nb()[2],
                                                            _nb()[5][:, 0], _nb()[6][:, 0], 2,
                                                            period=L)),
    "iso_ccyl_f5_nopbc": ("conditional_cylindrical_isolation", lambda m, s1, s2, t1, t2:
                          m.conditional_cylindrical_isolation(s1, s2, _nb()[1], _nb()[2],
                                                              _nb()[5], _nb()[6], 5)),
    "weighted_s_mu_auto_pbc": ("weighted_npairs_s_mu", lambda m, s1, s2, t1, t2: m.weighted_npairs_s_mu(
        s1, s1, _wt()[0], _wt()[0], SB, MU, period=L)),
    "weighted_s_mu_cross_nopbc": ("weighted_npairs_s_mu", lambda m, s1, s2, t1, t2: m.weighted_npairs_s_mu(
        s1, s2, _wt()[0], _wt()[1], SB, MU)),
    "weighted_s_mu_ones_cross_pbc": ("weighted_npairs_s_mu", lambda m, s1, s2, t1, t2: m.weighted_npairs_s_mu(
        s2, s1, np.ones(len(s2)), np.ones(len(s1)), SB, MU, period=L)),
}

# float results: within this relative tolerance of halotools' FP64 sums
# (integer-valued marks are exact); the counts are exact
RTOL_WEIGHTED = 1e-6


def run_case(mod, name):
    """The case's output: one array, or (counts, weighted counts) for weighted_npairs_s_mu."""
    r = CASES[name][1](mod, *sibling_inputs())
    if isinstance(r, tuple):
        return tuple(np.asarray(a) for a in r)
    return np.asarray(r)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=build_ref.DEFAULT_SRC)
    args = ap.parse_args()
    from oracle import ref_loader
    ns = ref_loader.load(args.src)
    sha = input_sha()
    os.makedirs(OUT, exist_ok=True)
    for name in CASES:
        out = run_case(ns, name)
        if isinstance(out, tuple):
            np.savez_compressed(os.path.join(OUT, name + ".npz"), sha=sha, out=out[0],
                                out_w=out[1])
            print(name, out[0].shape, out[0].dtype, out[1].dtype)
        else:
            np.savez_compressed(os.path.join(OUT, name + ".npz"), sha=sha, out=out)
            print(name, out.shape, out.dtype)


if __name__ == "__main__":
    main()
