"""The FP32 guard band of the count kernels, checked on the host (no GPU).

A pair is counted in bin k iff its FP64 squared separation, formed as
npairs_3d_engine.pyx:167-176 does ((x1 - shift) - x2 per coordinate, squared
and summed left to right), is <= fl(rbins[k]^2).  The count kernel decides that
from an FP32 value instead and sends only pairs between two FP32 thresholds to
an FP64 recheck: v32 <= lo[k] must prove v64 <= E[k] and v32 > hi[k] must
prove v64 > E[k].  These tests form v32 exactly as the kernel does (each
coordinate as an FP32 offset from its block corner, the neighbour block's FP32
offset added to the j point, the differences squared with fused multiply-adds)
for adversarial pairs within a few parts per million of every edge, on the
grids the library chooses, and check both implications against the thresholds
the library computes (gbp_npairs_3d_thresholds)."""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

from halotools_gb300 import _native as N

LD = np.longdouble
pytestmark = pytest.mark.skipif(np.finfo(LD).nmant < 60,
                                reason="needs an extended long double to emulate FMA")


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def grid_and_thresholds(L, rbins, n2, reach=0, block=0):
    lib = N.load()
    per = np.array([L] * 3)
    rb = np.ascontiguousarray(rbins, dtype=np.float64)
    out = (ctypes.c_int32 * 7)()
    search = np.array([rb.max()] * 3)
    assert lib.gbp_grid_describe(_p(per, ctypes.c_double), 1, _p(search, ctypes.c_double), n2,
                                 0, reach, block, out) == 0
    hi = np.zeros(len(rb), np.float32)
    lo = np.zeros(len(rb), np.float32)
    c = np.zeros(3)
    assert lib.gbp_npairs_3d_thresholds(_p(per, ctypes.c_double), 1, _p(rb, ctypes.c_double),
                                        len(rb), n2, reach, block, _p(hi, ctypes.c_float),
                                        _p(lo, ctypes.c_float), _p(c, ctypes.c_double)) == 0
    return {"reach": out[0], "bf": out[1], "n": out[2], "DB": out[6], "c": c[0],
            "n3": [out[2], out[3], out[4]], "c3": list(c)}, hi, lo


def grid_and_thresholds_xy_z(L, rp, pi, n2, reach=0, block=0):
    lib = N.load()
    per = np.array([L] * 3)
    rp = np.ascontiguousarray(rp, dtype=np.float64)
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    out = (ctypes.c_int32 * 7)()
    search = np.array([rp.max(), rp.max(), pi.max()])
    assert lib.gbp_grid_describe(_p(per, ctypes.c_double), 1, _p(search, ctypes.c_double), n2,
                                 2, reach, block, out) == 0
    t = [np.zeros(len(a), np.float32) for a in (rp, rp, pi, pi)]
    c = np.zeros(3)
    fp = ctypes.c_float
    assert lib.gbp_npairs_xy_z_thresholds(_p(per, ctypes.c_double), 1, _p(rp, ctypes.c_double),
                                          len(rp), _p(pi, ctypes.c_double), len(pi), n2, reach,
                                          block, _p(t[0], fp), _p(t[1], fp), _p(t[2], fp),
                                          _p(t[3], fp), _p(c, ctypes.c_double)) == 0
    g = {"reach": out[0], "bf": out[1], "DB": out[6], "n3": [out[2], out[3], out[4]],
         "c3": list(c)}
    return g, t


def fma32(a, b, c):
    """fmaf(a, b, c) for float32 arrays: one rounding of a*b + c to float32."""
    p = a.astype(LD) * b.astype(LD)          # exact: 24 + 24 bits
    cl = c.astype(LD)
    s = p + cl
    z = s - p
    e = (p - (s - z)) + (cl - z)             # s + e == a*b + c exactly
    r = s.astype(np.float32)
    # s exactly halfway between two floats with a nonzero remainder: the
    # remainder's sign decides (a rare case, settled exactly)
    d = s - r.astype(LD)
    half = np.spacing(np.abs(r)).astype(LD) / 2
    tie = (np.abs(d) == half) & (e != 0)
    for i in np.flatnonzero(tie):
        q = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        cand = [r[i], np.nextafter(r[i], np.float32(np.inf)), np.nextafter(r[i], np.float32(-np.inf))]
        r[i] = min(cand, key=lambda f: abs(Fraction(float(f)) - q))
    return r


def deltas32(xi, xj, g, f32_input):
    """The kernel's FP32 coordinate differences of i-point xi and j-point xj."""
    bf, DB = g["bf"], g["DB"]
    dv = []
    for d in range(3):
        c, n = g["c3"][d], g["n3"][d]
        nbk = n // bf

        def rel(x):
            k = np.clip(np.floor(x * (1.0 / c)).astype(np.int64), 0, n - 1)
            ib = k // bf
            C = (ib * bf) * c
            if f32_input:
                chi = C.astype(np.float32)
                clo = (C - chi.astype(np.float64)).astype(np.float32)
                return ((x.astype(np.float32) - chi) - clo).astype(np.float32), ib
            return (x - C).astype(np.float32), ib
        ui, bi = rel(xi[:, d])
        uj, bj = rel(xj[:, d])
        ox = bj - bi
        ox = np.where(ox > nbk // 2, ox - nbk, np.where(ox < -(nbk // 2), ox + nbk, ox))
        assert np.all(np.abs(ox) <= DB)
        D = (ox * bf * c).astype(np.float32)
        t = (uj + D).astype(np.float32)
        dv.append((ui - t).astype(np.float32))
    return dv


def v32_of(xi, xj, g, L, f32_input):
    """The 3-D count's FP32 squared separation: fma(dz, dz, fma(dy, dy, dx * dx))."""
    dx, dy, dz = deltas32(xi, xj, g, f32_input)
    return fma32(dz, dz, fma32(dy, dy, (dx * dx).astype(np.float32)))


def deltas64(xi, xj, L):
    """npairs_*_engine.pyx: (x1 - shift) - x2 with the shift in {-L, 0, L} of the visit."""
    out = []
    for d in range(3):
        best = None
        for shift in (0.0, L, -L):
            dd = (xi[:, d] - shift) - xj[:, d]
            best = dd if best is None else np.where(np.abs(dd) < np.abs(best), dd, best)
        out.append(best)
    return out


def v64_of(xi, xj, L):
    """npairs_3d_engine.pyx:167-176: the differences squared and summed left to right."""
    dx, dy, dz = deltas64(xi, xj, L)
    return (dx * dx + dy * dy) + dz * dz


def adversarial_pairs(rng, L, rbins, npairs, rel, f32_input):
    """Pairs whose separation lies within `rel` (relative) of a random edge."""
    k = rng.integers(0, len(rbins), npairs)
    r = rbins[k] * (1.0 + rng.uniform(-rel, rel, npairs))
    d = rng.normal(size=(npairs, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    xi = rng.uniform(0, L, (npairs, 3))
    xj = np.mod(xi + r[:, None] * d, L)
    if f32_input:  # the engines upcast float32 exactly
        xi = xi.astype(np.float32).astype(np.float64)
        xj = np.minimum(xj.astype(np.float32).astype(np.float64), np.nextafter(L, 0))
    return xi, xj


CASES = [
    # (box, rbins, points of sample 2, reach hint, block hint, float32 input)
    (2000.0, np.logspace(np.log10(0.5), np.log10(50), 30), 10_000_000, 0, 0, False),
    (250.0, np.logspace(-1, np.log10(20), 15), 100_000, 0, 0, False),
    (1000.0, np.logspace(-1, np.log10(30), 20), 10_000, 0, 0, False),
    (1000.0, np.logspace(-1, np.log10(20), 15), 2_000_000, 3, 2, True),
    (420.0, np.logspace(-1, np.log10(20), 15), 30_000, 2, 1, False),
]


@pytest.mark.parametrize("L,rbins,n2,reach,block,f32", CASES)
def test_fp32_thresholds_bracket_the_fp64_edges(L, rbins, n2, reach, block, f32):
    g, hi, lo = grid_and_thresholds(L, rbins, n2, reach, block)
    E = rbins * rbins
    rng = np.random.default_rng(int(L) + n2 % 1000 + reach)
    decided = 0
    for rel in (3e-5, 3e-6, 4e-7):
        xi, xj = adversarial_pairs(rng, L, rbins, 100_000, rel, f32)
        for a, b in ((xi, xj), (xj, xi)):  # both orders, as the kernel's symmetric walk
            v32 = v32_of(a, b, g, L, f32)
            v64 = v64_of(a, b, L)
            for k in range(len(E)):
                inside = v32 <= lo[k]
                outside = v32 > hi[k]
                assert np.all(v64[inside] <= E[k]), (k, "inside")
                assert np.all(v64[outside] > E[k]), (k, "outside")
                decided += int(np.count_nonzero(inside | outside))
    assert decided > 0


def test_headline_grid_is_the_blocked_one():
    g, hi, lo = grid_and_thresholds(2000.0, np.logspace(np.log10(0.5), np.log10(50), 30),
                                    10_000_000)
    assert (g["reach"], g["bf"], g["n"]) == (4, 2, 160)
    E = np.logspace(np.log10(0.5), np.log10(50), 30) ** 2
    assert np.all(lo <= E) and np.all(E <= hi)
    # the band is narrow at the outer edges, where most pairs lie: a few parts
    # per million (at the inner edges the offsets' absolute error dominates)
    assert np.all(((hi - lo) / E)[-5:] < 1e-5)


@pytest.mark.parametrize("f32", [False, True])
def test_fp32_thresholds_bracket_the_fp64_edges_xy_z(f32):
    # the xyz2m geometry: rp 20 log edges 0.1-30, pi 40 linear edges 0-40
    L = 1000.0
    rp = np.logspace(-1, np.log10(30), 20)
    pi = np.linspace(0.0, 40.0, 40)
    g, (hr, lr, hp, lp) = grid_and_thresholds_xy_z(L, rp, pi, 2_000_000)
    E0, E1 = rp * rp, pi * pi
    rng = np.random.default_rng(21 + f32)
    for rel in (3e-5, 3e-6, 4e-7):
        n = 100_000
        # half the pairs near an rp edge, half near a pi edge
        k = rng.integers(0, len(rp), n)
        q = rng.integers(1, len(pi), n)
        near_rp = np.arange(n) < n // 2
        r = np.where(near_rp, rp[k] * (1 + rng.uniform(-rel, rel, n)), rng.uniform(0, 30.0, n))
        z = np.where(near_rp, rng.uniform(-40.0, 40.0, n),
                     pi[q] * (1 + rng.uniform(-rel, rel, n)) * rng.choice([-1.0, 1.0], n))
        phi = rng.uniform(0, 2 * np.pi, n)
        xi = rng.uniform(0, L, (n, 3))
        xj = np.mod(xi + np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1), L)
        if f32:
            xi = xi.astype(np.float32).astype(np.float64)
            xj = np.minimum(xj.astype(np.float32).astype(np.float64), np.nextafter(L, 0))
        for a, b in ((xi, xj), (xj, xi)):
            dx, dy, dz = deltas32(a, b, g, f32)
            v0 = fma32(dy, dy, (dx * dx).astype(np.float32))
            v1 = (dz * dz).astype(np.float32)
            ex, ey, ez = deltas64(a, b, L)
            w0, w1 = ex * ex + ey * ey, ez * ez
            for kk in range(len(E0)):
                assert np.all(w0[v0 <= lr[kk]] <= E0[kk]) and np.all(w0[v0 > hr[kk]] > E0[kk]), kk
            for kk in range(len(E1)):
                assert np.all(w1[v1 <= lp[kk]] <= E1[kk]) and np.all(w1[v1 > hp[kk]] > E1[kk]), kk


def lut_of(L, rbins, n2, reach=0, block=0):
    lib = N.load()
    per = np.array([L] * 3)
    rb = np.ascontiguousarray(rbins, dtype=np.float64)
    lut = np.zeros((1024, 4), np.float32)
    info = np.zeros(3, np.int32)
    vr = np.zeros(2, np.float32)
    assert lib.gbp_npairs_3d_lut(_p(per, ctypes.c_double), 1, _p(rb, ctypes.c_double), len(rb),
                                 n2, reach, block, _p(lut, ctypes.c_float),
                                 _p(info, ctypes.c_int32), _p(vr, ctypes.c_float)) == 0
    T, S, B = (int(v) for v in info)
    return lut[:T], S, B, vr


@pytest.mark.parametrize("L,rbins,n2", [c[:3] for c in CASES])
def test_bin_table_agrees_with_the_thresholds(L, rbins, n2):
    # the kernel bins v by one table slot: b0 + (v > upper), rechecked when
    # lower < v <= upper.  Where that does not ask for a recheck, the bin must be
    # the one the per-edge thresholds prove: every edge below it provably
    # exceeded (v > hi), its own edge provably not (v <= lo), or past the top
    lut, S, B, (vlo, vhi) = lut_of(L, rbins, n2)
    _, hi, lo = grid_and_thresholds(L, rbins, n2)
    rng = np.random.default_rng(int(L))
    # values log-uniform over the table's range and beyond, plus every threshold
    # and its float neighbours
    v = np.exp(rng.uniform(np.log(vlo) - 2, np.log(vhi) + 2, 400_000)).astype(np.float32)
    th = np.concatenate([hi, lo, [vlo, vhi, 0.0]]).astype(np.float32)
    v = np.concatenate([v, th, np.nextafter(th, np.float32(np.inf)),
                        np.nextafter(th, np.float32(-np.inf)), [np.float32(0.0)]])
    v = v[np.isfinite(v) & (v >= 0)]
    vc = np.clip(v, vlo, vhi)
    slot = (vc.view(np.uint32) >> np.uint32(S)).astype(np.int64) - B
    assert np.all((slot >= 0) & (slot < len(lut)))
    e = lut[slot]
    b0 = e[:, 0].view(np.int32)
    up, low = e[:, 1], e[:, 2]
    b = b0 + (v > up)
    walk = (v > low) & ~(v > up)
    nb = len(hi)
    for i in np.flatnonzero(~walk):
        k = b[i]
        assert np.all(v[i] > hi[:k]), (v[i], k)
        assert k == nb or v[i] <= lo[k], (v[i], k)


def smu_tables(L, sb, mup, n2):
    lib = N.load()
    per = np.array([L] * 3)
    sb = np.ascontiguousarray(sb, dtype=np.float64)
    mup = np.ascontiguousarray(mup, dtype=np.float64)
    fp = ctypes.c_float
    s_lut = np.zeros((1024, 4), np.float32)
    q_lut = np.zeros((1024, 4), np.float32)
    s_hi, s_lo = np.zeros(len(sb), np.float32), np.zeros(len(sb), np.float32)
    q_hi, q_lo = np.zeros(len(mup), np.float32), np.zeros(len(mup), np.float32)
    info = np.zeros(6, np.int32)
    vr = np.zeros(4, np.float32)
    c = np.zeros(3)
    assert lib.gbp_npairs_s_mu_tables(
        _p(per, ctypes.c_double), 1, _p(sb, ctypes.c_double), len(sb), _p(mup, ctypes.c_double),
        len(mup), n2, 0, 0, _p(s_lut, fp), _p(s_hi, fp), _p(s_lo, fp), _p(q_lut, fp),
        _p(q_hi, fp), _p(q_lo, fp), _p(info, ctypes.c_int32), _p(vr, fp),
        _p(c, ctypes.c_double)) == 0
    T0, S0, B0, T1, S1, B1 = (int(v) for v in info)
    out = (ctypes.c_int32 * 7)()
    search = np.array([sb.max()] * 3)
    assert lib.gbp_grid_describe(_p(per, ctypes.c_double), 1, _p(search, ctypes.c_double), n2, 1,
                                 0, 0, out) == 0
    g = {"bf": out[1], "DB": out[6], "n3": [out[2], out[3], out[4]], "c3": list(c)}
    return g, dict(s_lut=s_lut[:T0], S0=S0, B0=B0, s_hi=s_hi, s_lo=s_lo, q_lut=q_lut[:T1], S1=S1,
                   B1=B1, q_hi=q_hi, q_lo=q_lo, vr=vr)


def slot_of(v, vlo, vhi, S, B):
    return (np.clip(v, vlo, vhi).view(np.uint32) >> np.uint32(S)).astype(np.int64) - B


def smu_kernel_bins(v0, v1, q, t):
    """The (s, mu') kernel's binning of FP32 s^2 = v0, dxy = v1 and quotient q:
    (s bin, mu' bin, settled).  A pair not settled goes to the FP64 recheck."""
    ns, nq = len(t["s_hi"]), len(t["q_hi"])
    e0 = t["s_lut"][slot_of(v0, t["vr"][0], t["vr"][1], t["S0"], t["B0"])]
    b0 = e0[:, 0].view(np.int32)
    bs = b0 + (v0 > e0[:, 1])
    amb = (v0 > e0[:, 2]) & ~(v0 > e0[:, 1])
    qb = e0[:, 3]
    # the q thresholds as the kernel lays them out: {thr, lo, hi below, lo above}
    hq = np.zeros((nq + 2, 4), np.float32)
    for k in range(nq):
        hq[k] = (t["q_hi"][k], t["q_lo"][k], t["q_hi"][k - 1] if k > 0 else -3.0e38,
                 t["q_lo"][k + 1] if k + 1 < nq else 3.0e38)
    hq[nq] = (np.inf, 3.0e38, t["q_hi"][nq - 1], 3.0e38)
    hq[nq + 1] = (np.inf, -np.inf, -3.0e38, 3.0e38)
    e1 = t["q_lut"][slot_of(q, t["vr"][2], t["vr"][3], t["S1"], t["B1"])]
    bq0 = e1[:, 0].view(np.int32)
    h = np.where((bq0 < nq) & (e1[:, 2] == -np.inf), nq + 1, bq0)
    th = hq[h]
    up = q > th[:, 0]
    bq = bq0 + up
    below = np.where(up, th[:, 0], th[:, 2])
    above = np.where(up, th[:, 3], th[:, 1])
    walk = th[:, 1] < -3.0e38
    amb |= ~(q - below > qb) | ~(above - q > qb) | walk
    return bs, bq, ~amb


@pytest.mark.parametrize("f32", [False, True])
def test_s_mu_bins_settled_in_fp32_are_the_fp64_bins(f32):
    # config 5's (s, mu') geometry: 30 log s bins 0.5-50, 21 linear mu edges 0-1
    L = 2000.0
    sb = np.logspace(np.log10(0.5), np.log10(50), 30)
    mu = np.linspace(0.0, 1.0, 21)
    mup = np.sort(np.sin(np.arccos(mu)))
    g, t = smu_tables(L, sb, mup, 10_000_000)
    Es, Eq = sb * sb, mup * mup
    rng = np.random.default_rng(31 + f32)
    settled = 0
    for rel in (3e-5, 3e-6, 4e-7):
        n = 100_000
        # half near an s edge (random direction), half near a mu' edge (random s)
        k = rng.integers(0, len(sb), n)
        qk = rng.integers(0, len(mup), n)
        s = np.where(np.arange(n) < n // 2, sb[k] * (1 + rng.uniform(-rel, rel, n)),
                     sb[-1] * rng.uniform(0.02, 1.0, n) ** (1 / 3))
        qq = np.where(np.arange(n) < n // 2, rng.uniform(0, 1, n),
                      np.clip(Eq[qk] * (1 + rng.uniform(-rel, rel, n)), 0, 1))
        phi = rng.uniform(0, 2 * np.pi, n)
        rxy = s * np.sqrt(qq)
        dz = s * np.sqrt(1 - qq) * rng.choice([-1.0, 1.0], n)
        xi = rng.uniform(0, L, (n, 3))
        xj = np.mod(xi + np.stack([rxy * np.cos(phi), rxy * np.sin(phi), dz], axis=1), L)
        if f32:
            xi = xi.astype(np.float32).astype(np.float64)
            xj = np.minimum(xj.astype(np.float32).astype(np.float64), np.nextafter(L, 0))
        for a, b in ((xi, xj), (xj, xi)):
            dx, dy, dzz = deltas32(a, b, g, f32)
            v1 = fma32(dy, dy, (dx * dx).astype(np.float32))
            v0 = fma32(dzz, dzz, v1)
            ex, ey, ez = deltas64(a, b, L)
            dxy = ex * ex + ey * ey
            s2 = ez * ez + dxy
            mu2 = np.where(s2 > 0, dxy / np.where(s2 > 0, s2, 1.0), 0.0)
            ms = np.searchsorted(Es, s2, side="left")
            mq = np.searchsorted(Eq, mu2, side="left")
            ok = v0 > 0
            qrn = np.zeros_like(v0)
            qrn[ok] = v1[ok] / v0[ok]
            # the FP32 quotient is within 2 ulp of the exact one: every float
            # within 2 ulp of the rounded quotient
            for step in (-2, -1, 0, 1, 2):
                q = qrn.copy()
                for _ in range(abs(step)):
                    q = np.nextafter(q, np.float32(np.inf if step > 0 else -np.inf))
                bs, bq, settled_k = smu_kernel_bins(v0, v1, q, t)
                sel = ok & settled_k & (bs < len(sb))
                # a settled pair lands in the reference's (s, mu') bin, or both
                # leave it out beyond the top mu' edge
                assert np.all(ms[sel] == bs[sel]), "s bin"
                cnt = sel & (bq < len(mup))
                assert np.all(mq[cnt] == bq[cnt]), "mu bin"
                drop = sel & (bq >= len(mup))
                assert np.all(mq[drop] >= len(mup)), "mu gate"
                # s beyond the top edge, settled in FP32: the reference skips it too
                gate = ok & (bs >= len(sb))
                assert np.all(ms[gate] >= len(sb)), "s gate"
                settled += int(np.count_nonzero(sel))
    assert settled > 0
