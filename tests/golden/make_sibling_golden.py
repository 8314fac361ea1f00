"""Golden vectors for the sibling counters (npairs_projected, npairs_jackknife_3d,
npairs_per_object_3d), made by running halotools' own front-ends and Cython
engines (built by ``oracle/build_ref.py``, imported by ``oracle/ref_loader.py``).

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


def input_sha():
    h = hashlib.sha256()
    for a in sibling_inputs():
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


CASES = {
    "projected_auto_pbc": lambda m, s1, s2, t1, t2: m.npairs_projected(s1, s1, RBINS, 8.0,
                                                                        period=L),
    "projected_cross_nopbc": lambda m, s1, s2, t1, t2: m.npairs_projected(s1, s2, RBINS, 6.5),
    "jackknife_auto_pbc": lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s1, RBINS, t1, t1, 5, period=L),
    "jackknife_cross_pbc": lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s2, RBINS, t1, t2, 5, period=L),
    "jackknife_auto_nopbc": lambda m, s1, s2, t1, t2: m.npairs_jackknife_3d(
        s1, s1, RBINS, t1, t1, 5),
    "per_object_cross_pbc": lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s1[:700], s2, RBINS, period=L),
    "per_object_auto_pbc": lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s1, s1, RBINS, period=L),
    "per_object_cross_nopbc": lambda m, s1, s2, t1, t2: m.npairs_per_object_3d(
        s2[:500], s1, RBINS),
}


def run_case(mod, name):
    return np.asarray(CASES[name](mod, *sibling_inputs()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default="/root/reference")
    args = ap.parse_args()
    from oracle import ref_loader
    ns = ref_loader.load(args.src)
    sha = input_sha()
    os.makedirs(OUT, exist_ok=True)
    for name in CASES:
        out = run_case(ns, name)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), sha=sha, out=out)
        print(name, out.shape, out.dtype)


if __name__ == "__main__":
    main()
