"""Stencil coverage, checked on the host (no GPU).

The reference visits every cell pair within the search length
(npairs_3d_engine.pyx:117-123), so it sees each in-range pair.  The GPU grid
prunes its stencil: a neighbour block's fine cells farther than the search
from the item's block are dropped.  These tests put pairs at up to the full
search length (a pair at exactly the search length still counts,
npairs_3d_engine.pyx:178) and within a few ulps of cell faces, digitise both
points as the kernel does, and check that the j point's (block offset, fine
cell) lies in a run of the stencil (gbp_stencil_describe); for an
auto-correlation, which lists each unordered block pair once, that either
order does.  Spheres for the 3-D and (s, mu') counts, cylinders for (rp, pi)."""
import ctypes

import numpy as np
import pytest

from halotools_gb300 import _native as N


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def stencil(L, search, n2, kind, reach=0, block=0, autocorr=True, pbc=1):
    lib = N.load()
    per = np.array([L] * 3)
    s = np.ascontiguousarray(search, dtype=np.float64)
    out = (ctypes.c_int32 * 7)()
    assert lib.gbp_grid_describe(_p(per, ctypes.c_double), pbc, _p(s, ctypes.c_double), n2, kind,
                                 reach, block, out) == 0
    runs = np.zeros((729, 5), np.int32)
    nr = np.zeros(1, np.int32)
    assert lib.gbp_stencil_describe(_p(per, ctypes.c_double), pbc, _p(s, ctypes.c_double), n2,
                                    kind, reach, block, int(autocorr), _p(runs, ctypes.c_int32),
                                    _p(nr, ctypes.c_int32)) == 0
    g = {"reach": out[0], "bf": out[1], "n3": [out[2], out[3], out[4]], "nruns": out[5]}
    if autocorr:  # gbp_grid_describe counts the auto-correlation's runs
        assert nr[0] == g["nruns"]
    return g, runs[:nr[0]]


def cell_of(x, L, n, bf):
    c = L / n
    k = np.clip(np.floor(x * (1.0 / c)).astype(np.int64), 0, n - 1)
    return k // bf, k % bf


def covered(runs, o, l):
    """Whether (block offset o, fine cell l) lies in some run."""
    ok = np.zeros(len(l), bool)
    for ox, oy, oz, l0, span in runs:
        ok |= (o[:, 0] == ox) & (o[:, 1] == oy) & (o[:, 2] == oz) & (l >= l0) & (l < l0 + span)
    return ok


def pairs(rng, L, search, kind, n):
    """Pairs at up to the search length, many at exactly it, some on cell faces."""
    xi = rng.uniform(0, L, (n, 3))
    if kind == 2:
        rp, pim = search[0], search[2]
        r = rp * np.sqrt(rng.uniform(0, 1, n))
        r[: n // 3] = rp
        phi = rng.uniform(0, 2 * np.pi, n)
        z = rng.uniform(-pim, pim, n)
        z[n // 3: 2 * n // 3] = pim * rng.choice([-1.0, 1.0], n // 3)
        d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    else:
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        r = search[0] * rng.uniform(0, 1, n) ** (1 / 3)
        r[: n // 2] = search[0]
        d *= r[:, None]
    xj = xi + d
    return xi, xj


GEOMETRIES = [
    # (box, search, points of sample 2, kind, reach hint, block hint)
    (2000.0, [50.0] * 3, 10_000_000, 0, 0, 0),     # the 10M-point headline: reach 4, blocks of 2
    (2000.0, [50.0] * 3, 10_000_000, 1, 0, 0),     # (s, mu') on the same points
    (250.0, [20.0] * 3, 100_000, 0, 0, 0),         # config 1: reach 1
    (1000.0, [30.0, 30.0, 40.0], 2_000_000, 2, 0, 0),  # xyz2m: cylinders
    (1000.0, [30.0] * 3, 10_000, 0, 0, 0),         # sparse: blocks of 4
    (300.0, [25.0] * 3, 40_000, 0, 3, 2),          # forced reach 3 in blocks of 2
    (420.0, [20.0] * 3, 30_000, 0, 2, 3),          # forced reach 2 in blocks of 3
]


@pytest.mark.parametrize("L,search,n2,kind,reach,block", GEOMETRIES)
@pytest.mark.parametrize("autocorr", [True, False])
def test_stencil_covers_every_pair_in_range(L, search, n2, kind, reach, block, autocorr):
    g, runs = stencil(L, search, n2, kind, reach, block, autocorr)
    bf = g["bf"]
    rng = np.random.default_rng(int(L) + kind + 10 * reach + block)
    xi, xj = pairs(rng, L, search, kind, 60_000)
    xj = np.mod(xj, L)
    # a third of the j points nudged onto the faces of their fine cells (a few
    # ulps either side); only pairs still within the search length are tested
    for d in range(3):
        c = L / g["n3"][d]
        m = rng.uniform(size=len(xj)) < 0.3
        face = np.round(xj[m, d] / c) * c
        xj[m, d] = np.mod(face + rng.choice([-1, 0, 1], m.sum()) * np.spacing(face + 1.0), L)
    d = np.mod(xj - xi + L / 2, L) - L / 2
    if kind == 2:
        keep = (d[:, 0] ** 2 + d[:, 1] ** 2 <= search[0] ** 2) & (np.abs(d[:, 2]) <= search[2])
    else:
        keep = (d ** 2).sum(axis=1) <= search[0] ** 2
    xi, xj = xi[keep], xj[keep]
    assert len(xi) > 30_000
    bi, li, bj, lj = [], [], [], []
    for d in range(3):
        n = g["n3"][d]
        a, la = cell_of(xi[:, d], L, n, bf)
        b, lb = cell_of(xj[:, d], L, n, bf)
        bi.append(a), li.append(la), bj.append(b), lj.append(lb)
    nbk = np.array(g["n3"]) // bf
    o = np.stack([bj[d] - bi[d] for d in range(3)], axis=1)
    o = np.where(o > nbk // 2, o - nbk, np.where(o < -(nbk // 2), o + nbk, o))
    lfi = (li[0] * bf + li[1]) * bf + li[2]
    lfj = (lj[0] * bf + lj[1]) * bf + lj[2]
    ok = covered(runs, o, lfj)
    if autocorr:
        ok |= covered(runs, -o, lfi)
    assert np.all(ok), (g, np.flatnonzero(~ok)[:5])


def test_pruning_drops_cells():
    # the 10M-point headline keeps 84 of the 125 x 8 fine-cell slots of its
    # half stencil in runs; the blocks beyond the search corners are dropped
    g, runs = stencil(2000.0, [50.0] * 3, 10_000_000, 0)
    assert (g["reach"], g["bf"]) == (4, 2)
    kept = int(runs[:, 4].sum())
    assert kept < 63 * 8, kept


@pytest.mark.parametrize("L,search,n2,kind,reach,block", [GEOMETRIES[i] for i in (0, 2, 3, 4)])
def test_stencil_covers_every_pair_in_range_without_wrap(L, search, n2, kind, reach, block):
    # non-periodic: the box [0, L] without wrap, pairs whose points both lie in it
    g, runs = stencil(L, search, n2, kind, reach, block, autocorr=False, pbc=0)
    bf = g["bf"]
    rng = np.random.default_rng(7 + int(L) + kind)
    xi, xj = pairs(rng, L, search, kind, 60_000)
    inside = np.all((xj >= 0) & (xj <= L), axis=1)
    xi, xj = xi[inside], xj[inside]
    o, lj = [], []
    for d in range(3):
        n = g["n3"][d]
        a, _ = cell_of(xi[:, d], L, n, bf)
        b, lb = cell_of(xj[:, d], L, n, bf)
        o.append(b - a)
        lj.append(lb)
    o = np.stack(o, axis=1)
    lfj = (lj[0] * bf + lj[1]) * bf + lj[2]
    assert np.all(covered(runs, o, lfj))
