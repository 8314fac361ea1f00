"""Generate the golden vectors in this directory by running the reference.

Runs halotools' own pair-counter front-ends and Cython engines (built from a
halotools source tree by ``oracle/build_ref.py`` and imported by
``oracle/ref_loader.py``) on small, seeded inputs and stores inputs and
outputs as ``.npz`` files.  The inputs follow the shapes of the reference's
own tests (tight loci and a regular mesh as in test_npairs_3d.py:32-197, a
point inside a ring of points as in test_npairs_s_mu.py:161-192, a non-cubic
box as in test_non_cubic_volumes.py:17-68, marking-function ids 1-17 as in
test_marked_npairs_3d.py) plus seeded uniform samples and pairs placed exactly
on a bin edge, which pin the FP64 operation order of the squared distance.

Usage (needs Cython and the halotools tree; not needed on the GPU machine)::

    python tests/golden/make_golden.py [--src /path/to/halotools/checkout]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
from oracle import build_ref  # noqa: E402

warnings.filterwarnings("ignore", category=SyntaxWarning)


def locus(rng, n, c, eps=0.001):
    return np.vstack([rng.uniform(ci - eps / 2, ci + eps / 2, n) for ci in c]).T


def regular_mesh(npts):
    g = np.linspace(0, 1, npts + 1)
    d = np.diff(g)[0] / 2.0
    x, y, z = np.array(np.meshgrid(g[:-1], g[:-1], g[:-1]))
    return np.vstack([x.flatten() + d, y.flatten() + d, z.flatten() + d]).T


def tie_pairs_3d(rng, L, npts, lo, hi):
    """One centre and npts partners whose left-to-right FP64 dsq is an exact
    edge, chosen where the other association orders give different values."""
    c = np.array([rng.uniform(0, 2.0), rng.uniform(0, 2.0), rng.uniform(L - 2.0, L)])
    pts, edges = [], []
    tries = 0
    while len(pts) < npts and tries < 200000:
        tries += 1
        r = rng.uniform(lo, hi)
        d = rng.normal(size=3)
        d *= r / np.linalg.norm(d)
        p = (c + d) % L
        dx = []
        for k in range(3):
            cands = [c[k] - p[k], (c[k] - L) - p[k], (c[k] + L) - p[k]]
            dx.append(min(cands, key=abs))
        dx, dy, dz = dx
        ltr = (dx * dx + dy * dy) + dz * dz
        alt = dx * dx + (dy * dy + dz * dz)
        if ltr == alt:
            continue
        r0 = np.sqrt(ltr)
        e = None
        for cand in (r0, np.nextafter(r0, 0), np.nextafter(r0, np.inf)):
            if cand * cand == ltr:
                e = cand
        if e is None or any(abs(e - q) < 1e-9 for q in edges):
            continue
        pts.append(p)
        edges.append(e)
    order = np.argsort(edges)
    return c[None, :], np.array(pts)[order], np.array(edges)[order]


def tie_pairs_xy(rng, L, npts, lo, hi):
    c = np.array([rng.uniform(0, 2.0), rng.uniform(L - 2.0, L), rng.uniform(0, L)])
    pts, edges = [], []
    tries = 0
    while len(pts) < npts and tries < 200000:
        tries += 1
        r = rng.uniform(lo, hi)
        t = rng.uniform(0, 2 * np.pi)
        p = np.array([(c[0] + r * np.cos(t)) % L, (c[1] + r * np.sin(t)) % L,
                      (c[2] + rng.uniform(-0.5, 0.5)) % L])
        dd = []
        for k in range(2):
            cands = [c[k] - p[k], (c[k] - L) - p[k], (c[k] + L) - p[k]]
            dd.append(min(cands, key=abs))
        v = dd[0] * dd[0] + dd[1] * dd[1]
        r0 = np.sqrt(v)
        e = None
        for cand in (r0, np.nextafter(r0, 0), np.nextafter(r0, np.inf)):
            if cand * cand == v:
                e = cand
        if e is None or any(abs(e - q) < 1e-9 for q in edges):
            continue
        pts.append(p)
        edges.append(e)
    order = np.argsort(edges)
    return c[None, :], np.array(pts)[order], np.array(edges)[order]


def main(src):
    from oracle import ref_loader
    ref = ref_loader.load(src)
    cases = {}

    def save(name, **kw):
        cases[name] = kw

    rng = np.random.default_rng(20240611)
    # ---- npairs_3d ----
    for i, (c1, c2, period) in enumerate([((0.1, 0.1, 0.1), (0.1, 0.1, 0.2), 1.0),
                                          ((0.1, 0.1, 0.05), (0.1, 0.1, 0.95), 1.0),
                                          ((0.05, 0.05, 0.05), (0.95, 0.95, 0.95), 1.0),
                                          ((0.05, 0.05, 0.05), (0.95, 0.95, 0.95), None)]):
        s1, s2 = locus(rng, 100, c1), locus(rng, 100, c2)
        rb = np.array((0.05, 0.15, 0.3))
        save("3d_locus%d" % i, kind="3d", s1=s1, s2=s2, bins=rb, period=period,
             out=ref.npairs_3d(s1, s2, rb, period=period))
    m = regular_mesh(10)
    sp = 0.1
    rb = np.array([sp / 100.0, sp + 1e-4, sp * np.sqrt(2) + 1e-4, sp * np.sqrt(3) + 1e-4])
    save("3d_regular_mesh", kind="3d", s1=m, s2=m.copy(), bins=rb, period=1.0,
         out=ref.npairs_3d(m, m.copy(), rb, period=1.0, approx_cell1_size=0.1))
    L = 250.0
    rb = np.logspace(-1, np.log10(20), 15)
    s1, s2 = rng.uniform(0, L, (3000, 3)), rng.uniform(0, L, (2500, 3))
    save("3d_cross_pbc", kind="3d", s1=s1, s2=s2, bins=rb, period=L,
         out=ref.npairs_3d(s1, s2, rb, period=L))
    save("3d_cross_nopbc", kind="3d", s1=s1, s2=s2, bins=rb, period=None,
         out=ref.npairs_3d(s1, s2, rb))
    s = rng.uniform(0, L, (4000, 3))
    save("3d_auto_pbc", kind="3d", s1=s, s2=None, bins=rb, period=L, out=ref.npairs_3d(s, s, rb, period=L))
    save("3d_auto_nopbc", kind="3d", s1=s, s2=None, bins=rb, period=None, out=ref.npairs_3d(s, s, rb))
    s32 = rng.uniform(0, L, (3000, 3)).astype(np.float32)
    save("3d_float32_auto", kind="3d", s1=s32, s2=None, bins=rb, period=L,
         out=ref.npairs_3d(s32, s32, rb, period=L))
    save("3d_two_edges_decreasing", kind="3d", s1=s1, s2=s2, bins=np.array([15.0, 5.0]),
         period=L, out=ref.npairs_3d(s1, s2, np.array([15.0, 5.0]), period=L))
    save("3d_zero_edge_auto", kind="3d", s1=s, s2=None, bins=np.array([0.0, 3.0, 10.0]),
         period=L, out=ref.npairs_3d(s, s, np.array([0.0, 3.0, 10.0]), period=L))
    pc = np.array([1.0, 2.0, 3.0])
    s1n = rng.uniform(0, 1, (300, 3)) * pc
    s2n = rng.uniform(0, 1, (280, 3)) * pc
    rb = np.arange(0.05, 0.31, 0.05)
    save("3d_noncubic_pbc", kind="3d", s1=s1n, s2=s2n, bins=rb, period=pc,
         out=ref.npairs_3d(s1n, s2n, rb, period=pc))
    for i in range(3):
        c, p, e = tie_pairs_3d(rng, 100.0, 40, 2.0, 30.0)
        save("3d_ties%d" % i, kind="3d", s1=c, s2=p, bins=e, period=100.0,
             out=ref.npairs_3d(c, p, e, period=100.0))
    # config-1 workload: inputs regenerated from the seed, checked by hash
    x = np.random.default_rng(0).uniform(0, 250, (100000, 3))
    rb = np.logspace(-1, np.log10(20), 15)
    save("3d_config1", kind="3d", s1=None, s2=None, bins=rb, period=250.0,
         gen="default_rng(0).uniform(0,250,(100000,3))",
         sha=hashlib.sha256(x.tobytes()).hexdigest(), out=ref.npairs_3d(x, x, rb, period=250.0))

    # ---- npairs_xy_z ----
    L = 250.0
    rp = np.logspace(-1, np.log10(30), 20)
    pi = np.linspace(0, 40, 40)
    s1, s2 = rng.uniform(0, L, (3000, 3)), rng.uniform(0, L, (2500, 3))
    save("xyz_cross_pbc", kind="xyz", s1=s1, s2=s2, bins=rp, bins2=pi, period=L,
         out=ref.npairs_xy_z(s1, s2, rp, pi, period=L))
    save("xyz_cross_nopbc", kind="xyz", s1=s1, s2=s2, bins=rp, bins2=pi, period=None,
         out=ref.npairs_xy_z(s1, s2, rp, pi))
    s = rng.uniform(0, L, (4000, 3))
    save("xyz_auto_pbc", kind="xyz", s1=s, s2=None, bins=rp, bins2=pi, period=L,
         out=ref.npairs_xy_z(s, s, rp, pi, period=L))
    rpn = np.arange(0, 0.31, 0.1)
    s1n = rng.uniform(0, 1, (100, 3)) * pc
    s2n = rng.uniform(0, 1, (90, 3)) * pc
    save("xyz_noncubic_pbc", kind="xyz", s1=s1n, s2=s2n, bins=rpn, bins2=rpn, period=pc,
         out=ref.npairs_xy_z(s1n, s2n, rpn, rpn, period=pc))
    save("xyz_noncubic_nopbc", kind="xyz", s1=s1n, s2=s2n, bins=rpn, bins2=rpn, period=None,
         out=ref.npairs_xy_z(s1n, s2n, rpn, rpn))
    for i in range(2):
        c, p, e = tie_pairs_xy(rng, 100.0, 40, 2.0, 30.0)
        pib = np.array([0.25, 0.5, 1.0])
        save("xyz_ties%d" % i, kind="xyz", s1=c, s2=p, bins=e, bins2=pib, period=100.0,
             out=ref.npairs_xy_z(c, p, e, pib, period=100.0))

    # ---- npairs_s_mu ----
    sb = np.logspace(np.log10(0.5), np.log10(30), 25)
    mu = np.linspace(0, 1, 20)
    save("smu_cross_pbc", kind="smu", s1=s1, s2=s2, bins=sb, bins2=mu, period=L,
         out=ref.npairs_s_mu(s1, s2, sb, mu, period=L))
    save("smu_cross_nopbc", kind="smu", s1=s1, s2=s2, bins=sb, bins2=mu, period=None,
         out=ref.npairs_s_mu(s1, s2, sb, mu))
    save("smu_auto_pbc", kind="smu", s1=s, s2=None, bins=sb, bins2=mu, period=L,
         out=ref.npairs_s_mu(s, s, sb, mu, period=L))
    theta = np.linspace(0, 2 * np.pi - 2 * np.pi / 360, 360) + (2.0 * np.pi) / (360 * 2)
    ring = np.vstack((1.5 * np.cos(theta), np.zeros(360), 1.5 * np.sin(theta))).T
    origin = np.array([[0.0, 0.0, 0.0]])
    mub = np.sort(np.cos(np.linspace(0.0, np.pi / 2.0, 91)))
    sbr = np.array([0.0, 1.0, 2.0])
    save("smu_ring", kind="smu", s1=origin, s2=ring, bins=sbr, bins2=mub, period=None,
         out=ref.npairs_s_mu(origin, ring, sbr, mub))

    # ---- marked_npairs_3d ----
    nw = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 2, 11: 2,
          12: 4, 13: 4, 14: 3, 15: 3, 16: 5, 17: 5}
    L = 100.0
    rb = np.array([0.0, 2.0, 5.0, 10.0, 20.0])
    s1, s2 = rng.uniform(0, L, (1500, 3)), rng.uniform(0, L, (1200, 3))
    for wid, k in nw.items():
        w1 = rng.uniform(0, 1, (1500, k))
        w2 = rng.uniform(0, 1, (1200, k))
        if wid in (3, 4, 16, 17):  # equality tests on integer tags
            col = 0 if wid in (3, 4) else 4
            w1[:, col] = rng.integers(0, 3, 1500)
            w2[:, col] = rng.integers(0, 3, 1200)
        save("marked_id%d" % wid, kind="marked", s1=s1, s2=s2, bins=rb, period=L, wid=wid,
             w1=w1, w2=w2, out=ref.marked_npairs_3d(s1, s2, rb, wid, period=L, weights1=w1,
                                                    weights2=w2))
    w = rng.lognormal(0, 0.5, 2000)
    sa = rng.uniform(0, L, (2000, 3))
    save("marked_auto_id1", kind="marked", s1=sa, s2=None, bins=rb, period=L, wid=1, w1=w,
         w2=None, out=ref.marked_npairs_3d(sa, sa, rb, 1, period=L, weights1=w, weights2=w))
    save("marked_nopbc_id1", kind="marked", s1=sa, s2=None, bins=rb, period=None, wid=1, w1=w,
         w2=None, out=ref.marked_npairs_3d(sa, sa, rb, 1, weights1=w, weights2=w))

    for name, kw in cases.items():
        arrs = {}
        for k, v in kw.items():
            if v is None:
                arrs[k] = np.array([])
                arrs[k + "_none"] = np.array(True)
            elif isinstance(v, str):
                arrs[k] = np.array(v)
            else:
                arrs[k] = np.asarray(v)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    print("wrote %d golden cases" % len(cases))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=build_ref.DEFAULT_SRC)
    main(ap.parse_args().src)
