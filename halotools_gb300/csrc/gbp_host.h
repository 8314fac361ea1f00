// Host-side planning shared by the plan API (gbp_api.cu) and the
// allocation-free entry point (gbp_static.cu): the reference's bin-edge
// semantics, FP32 thresholds with a rigorous error band, float-bit lookup
// tables, grid choice and the cell stencil.  Everything works on fixed-size
// storage supplied by the caller; nothing here allocates.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

#include "gbp_internal.cuh"

#define GBP_STEN_CAP 729  // (2*4+1)^3 cells for reach <= 4; runs of blocked grids fit too

namespace gbp {

const double INF = std::numeric_limits<double>::infinity();
const float FINF = std::numeric_limits<float>::infinity();

// Walk-from-the-top semantics of npairs_3d / npairs_xy_z / marked engines
// (npairs_3d_engine.pyx:178-182): counts[k] is incremented iff v <= r[m]^2 for
// every m >= k; a NaN edge stops the walk.  E'[k] = min(r[k..]^2), -inf once a
// NaN was met, so bin(v) = smallest k with v <= E'[k].
inline void edges_top_walk(const double *r, int n, double *E) {
    double m = INF;
    bool dead = false;
    for (int k = n - 1; k >= 0; k--) {
        double e = r[k] * r[k];
        if (std::isnan(e)) dead = true;
        if (dead) {
            E[k] = -INF;
        } else {
            m = std::min(m, e);
            E[k] = m;
        }
    }
}

// npairs_s_mu_engine.pyx:198-226 semantics for squared edges Ein: a value is
// skipped when it exceeds max(Ein) (a NaN max never skips); otherwise its index
// is 1 + the first k (walking down from n-2) with v > Ein[k].  Writes
// non-decreasing E' with bin(v) = smallest m such that v <= E'[m].
inline void edges_smu(const double *Ein, int n, double *Ep) {
    double gate = -INF;
    bool nan = false;
    for (int k = 0; k < n; k++) {
        if (std::isnan(Ein[k])) nan = true;
        else gate = std::max(gate, Ein[k]);
    }
    Ep[n - 1] = nan ? INF : gate;
    double m = INF;
    for (int k = n - 2; k >= 0; k--) {
        if (!std::isnan(Ein[k])) m = std::min(m, Ein[k]);
        Ep[k] = m;
    }
    for (int k = n - 2; k >= 0; k--) Ep[k] = std::min(Ep[k], Ep[k + 1]);
}

inline float f_down(double x) {
    if (std::isnan(x)) return -FINF;
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -FINF);
    return f;
}

inline float f_up(double x) {
    if (std::isnan(x)) return FINF;
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, FINF);
    return f;
}

inline float bitsf(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Error model.  Coordinates are FP32 offsets from a block corner, |u| <= c
// (c = block size here), each rounded at most twice (float32 input forms
// (x - hi) - lo in FP32), the stencil offset o*c (|o| <= K blocks) is rounded
// to FP32 and added, and dx is formed in FP32:
// |dx32 - dx| <= delta = 2^-24 (2c + 2c + K c + (K+1) c + |dx|) plus the
// corner's representation and the reference's own dx rounding (~2^-46 L).
struct ErrModel {
    double cmax = 0, K = 1, Lmax = 0;
    double delta(double Ebound) const {
        double dxmax = std::sqrt(std::max(Ebound, 0.0));
        return std::ldexp(1.0, -24) * (4 * cmax + K * cmax + (K + 1) * cmax + dxmax) * 1.02 +
               std::ldexp(1.0, -46) * Lmax;
    }
    // bound on |v32 - v64| for v a sum of m squares near E
    double band(double E, int m) const {
        double E1 = E * (1.0 + std::ldexp(1.0, -10)) + 1e-300;
        double d = delta(E1);
        return 2.0 * d * std::sqrt((double)m) * std::sqrt(E1) + m * d * d +
               (m + 1) * std::ldexp(1.0, -24) * E1 + m * std::ldexp(1.0, -50) * E1;
    }
};

// FP32 thresholds: v32 <= lo[k] proves v64 <= E[k]; v32 > hi[k] proves
// v64 > E[k] (twice the error bound on each side).  em == nullptr gives the
// tight FP32 bracket of E (used for the mu' axis, whose band is per pair).
inline void thresholds(int nb, const double *E, const ErrModel *em, int m, float *hi, float *lo) {
    for (int k = 0; k < nb; k++) {
        double e = E[k];
        if (std::isinf(e)) {
            hi[k] = lo[k] = (float)e;
            continue;
        }
        double b = em ? 2.0 * em->band(e, m) : 0.0;
        lo[k] = f_down(e - b);
        hi[k] = f_up(e + b);
    }
    for (int k = 1; k < nb; k++) hi[k] = std::max(hi[k], hi[k - 1]);
}

struct LutInfo {
    int T = 0, S = 0, B = 0;
    float vlo = 0, vhi = 0;
};

// Float-bit lookup table: slot s covers the FP32 values whose bits, shifted
// right by S, equal B + s; values below/above the covered octaves clamp into
// the first/last slot.  Each slot stores the first bin not provably exceeded
// by every value of the slot (b0) and, if at most one edge can be crossed in
// the slot, that edge's thresholds; otherwise (thr, lo) = (+inf, -inf), which
// sends the pair to the per-edge walk.  qband(a) goes to .w.  The octaves run
// from just below the smallest positive lower threshold (an edge at 0 lives in
// slot 0) to just above the largest finite upper threshold.
template <class QB>
LutInfo build_lut(int nb, const float *hi, const float *lo, QB qband, float4 *lut) {
    LutInfo L;
    double hmax = 0, pmin = INF;
    for (int k = 0; k < nb; k++) {
        if (std::isfinite(hi[k]) && hi[k] > 0) hmax = std::max(hmax, (double)hi[k]);
        if (std::isfinite(lo[k]) && lo[k] > 0) pmin = std::min(pmin, (double)lo[k]);
    }
    int emax = hmax > 0 ? std::ilogb(hmax) + 1 : 0;
    emax = std::min(emax, 126);
    int emin = std::isfinite(pmin) ? std::ilogb(pmin) - 1 : emax - 1;
    emin = std::min(emin, emax - 1);
    emin = std::max(emin, std::max(emax - 40, -126));
    int O = emax - emin + 1;
    int m = 0;
    while (m < 10 && (O << (m + 1)) <= GBP_LUT_MAX) m++;
    L.S = 23 - m;
    L.T = O << m;
    L.B = (emin + 127) << m;
    L.vlo = std::ldexp(1.0f, emin);
    L.vhi = std::nextafter(std::ldexp(1.0f, emax + 1), 0.0f);
    for (int s = 0; s < L.T; s++) {
        float a = s == 0 ? 0.0f : bitsf((uint32_t)(L.B + s) << L.S);
        float bnext = s == L.T - 1 ? FINF : bitsf((uint32_t)(L.B + s + 1) << L.S);
        float pred = std::nextafter(bnext, 0.0f);
        int b0 = 0;
        while (b0 < nb && hi[b0] < a) b0++;
        float4 e;
        std::memcpy(&e.x, &b0, 4);
        if (b0 == nb) {
            e.y = FINF;
            e.z = FINF;
        } else {
            bool simple = (b0 + 1 == nb) || (pred <= lo[b0 + 1]);
            e.y = simple ? hi[b0] : FINF;
            e.z = simple ? lo[b0] : -FINF;
        }
        e.w = qband(a);
        lut[s] = e;
    }
    return L;
}

inline float no_qband(float) { return 0.0f; }

// bin of an exactly known FP64 value (self-pairs: every separation is 0)
inline int host_bin(int nb, const double *E, double v) {
    int k = 0;
    while (k < nb && !(v <= E[k])) k++;
    return k;
}

// ---------------- grid & stencil ----------------
// Two-level grid: fine cells of size c (K c >= search) grouped into blocks of
// bf^3 fine cells.  Points are sorted block-major (key = block * bf^3 + fine
// cell within the block), so a block's points are contiguous and form the
// i-side of a work item; the j-side is the list of fine cells within the search
// of the block's box.  bf = 1 is the plain cell list.
struct Geometry {
    int n[3];       // fine cells per dimension (n = nb * bf)
    int nb[3];      // blocks per dimension
    int bf = 1;     // fine cells per block edge
    double c[3], L[3];
    int K;          // fine reach
    int DB = 1;     // block reach of the stencil
    int pbc;
    int64_t ncells;   // fine cells
    int64_t nblocks;
    int nsten;
    int nself;
    int sten[GBP_STEN_CAP];
    float4 stenD[GBP_STEN_CAP];
};

const int64_t MAX_CELLS_PER_DIM = 256;
// Mean points per reach-K cell from which choose_grid takes reach K >= 2.  The
// unweighted 3-D and (s, mu') counts, whose cost is mostly per binned pair,
// take finer cells earlier than the marked and (rp, pi) ones: on 10M clustered
// points (19.5 per reach-2 cell) reach 2 cut the 3-D count 22.2 -> 20.8 ms and
// the (s, mu') count 32.6 -> 30.4 ms, while the 2-channel marked count went
// 48.2 -> 85.9 ms and the (rp, pi) count on 2M points (9 per cell) 3.6 -> 3.9 ms.
const double GBP_DENSE_REACH2 = 16.0;

// Cells per dimension for reach K: as many as keep K*c >= search, capped;
// with periodic wrap every offset in [-K, K] must reach a distinct cell.
inline bool grid_for_reach(int K, const double L[3], const double search[3], int pbc,
                           int64_t n[3], int64_t cap) {
    for (int d = 0; d < 3; d++) {
        int64_t m = (int64_t)std::floor(L[d] * K / search[d]);
        m = std::min<int64_t>(std::max<int64_t>(m, 1), cap);
        // search <= L/3, so three cells of size L/3 always cover it for K = 1
        if (pbc && K == 1) m = std::max<int64_t>(m, 3);
        if (pbc && m < 2 * K + 1) return false;
        n[d] = m;
    }
    return true;
}

// Reach K in 1..4 (hint > 0 forces it when feasible); the automatic choice
// keeps about 28+ points of sample 2 per cell: finer cells prune more of the
// cube stencil, but each work item then streams fewer points per i-point.
// Sparse samples (fewer than ~12 points per reach-1 cell): by default reach-1
// fine cells grouped into blocks of about 32 points (bf = round(cbrt(32 /
// occupancy)), at most 4), so that an item's i-points come from a block while
// its j-cells hug the block's search region; with ppc > 0, single cells larger
// than the search holding about ppc points instead.  ppc < 0 disables both.
// bf_hint > 0 forces the block factor (when the grid allows it).  With split,
// an automatic choice of reach 2 becomes reach 4 in blocks of 2^3 cells: the
// items' i-points come from the same reach-2-sized blocks, while the j side is
// pruned at half the cell size (on 10M clustered points 12.7e9 -> 11.1e9
// candidates, the 3-D count 20.30 -> 19.47 ms and the (s, mu') count 30.1 ->
// 29.0 ms; reach 3 in blocks of 2, 20.25 ms; reach 4 in blocks of 4, 20.21 ms).
inline void choose_grid(Geometry &g, const double L[3], const double search[3], int pbc,
                        int64_t n2, int reach_hint, int64_t cap_per_dim, double ppc = 0.0,
                        int bf_hint = 0, double dense = 28.0, bool split = false) {
    for (int d = 0; d < 3; d++) g.L[d] = L[d];
    g.pbc = pbc;
    double vol = L[0] * L[1] * L[2];
    double rho = vol > 0 ? (double)n2 / vol : 0;
    int best = 1;
    for (int K = 2; K <= 4; K++) {
        int64_t n[3];
        if (!grid_for_reach(K, L, search, pbc, n, cap_per_dim)) break;
        double cvol = (L[0] / n[0]) * (L[1] / n[1]) * (L[2] / n[2]);
        if (reach_hint > 0) {
            if (K <= reach_hint) best = K;
            continue;
        }
        if (rho * cvol >= dense) best = K;
    }
    bool split4 = false;
    if (split && reach_hint <= 0 && bf_hint <= 0 && best == 2) {
        // reach 4 in blocks of 2: feasible when the blocks tile the grid, the
        // stencil's block offsets (DB = 2) reach distinct blocks and its runs fit
        int64_t n4[3];
        split4 = grid_for_reach(4, L, search, pbc, n4, cap_per_dim) &&
                 5 * 5 * 5 * 2 * 2 <= GBP_STEN_CAP;
        for (int d = 0; d < 3 && split4; d++)
            if (n4[d] / 2 < 1 || (pbc && n4[d] / 2 < 5)) split4 = false;
        if (split4) best = 4;
    }
    int64_t n[3];
    grid_for_reach(best, L, search, pbc, n, cap_per_dim);
    int bf = 1;
    if (best == 1 && ppc >= 0.0 && rho > 0) {
        double cvol = (L[0] / n[0]) * (L[1] / n[1]) * (L[2] / n[2]);
        if (ppc > 0.0) {
            double ct = std::cbrt(ppc / rho);
            for (int d = 0; d < 3; d++) {
                int64_t m = (int64_t)std::floor(L[d] / ct);
                m = std::max<int64_t>(m, pbc ? 3 : 1);
                n[d] = std::min(n[d], m);  // never finer than the reach-1 grid
            }
        } else if (bf_hint > 0) {
            bf = bf_hint;
        } else if (bf_hint == 0 && rho * cvol < 12.0) {
            bf = (int)std::lround(std::cbrt(32.0 / std::max(rho * cvol, 1e-6)));
        }
    } else if (bf_hint > 0) {
        bf = bf_hint;
    } else if (split4) {
        bf = 2;
    }
    bf = std::max(1, std::min(bf, 4));
    // blocks must tile the grid and, with periodic wrap, every block offset of
    // the stencil must reach a distinct block
    for (; bf > 1; bf--) {
        const int DB = (best + bf - 1) / bf;
        // at most bf^2 runs per neighbour block
        bool ok = (2 * DB + 1) * (2 * DB + 1) * (2 * DB + 1) * bf * bf <= GBP_STEN_CAP;
        for (int d = 0; d < 3; d++) {
            const int64_t nbk = n[d] / bf;
            if (nbk < 1 || (pbc && nbk < 2 * DB + 1)) ok = false;
        }
        if (ok) break;
    }
    g.K = best;
    g.bf = bf;
    g.DB = (best + bf - 1) / bf;
    g.ncells = 1;
    g.nblocks = 1;
    for (int d = 0; d < 3; d++) {
        g.nb[d] = (int)(n[d] / bf);
        g.n[d] = g.nb[d] * bf;
        g.c[d] = L[d] / (double)g.n[d];
        g.ncells *= g.n[d];
        g.nblocks *= g.nb[d];
    }
}

// kind 0: sphere of radius search[0]; kind 1: cylinder (rp = search[0], pi = search[2]).
// An entry is a run of consecutive fine-cell keys of one neighbour block:
// sten = block offset (8 bits each, biased by 64) | first fine cell << 24, and
// stenD = (block offset * block size, run length).  Fine cells whose box is
// farther than the search from the item block's box are dropped.  The own
// block comes first as one run of bf^3 cells; in auto mode only the
// lexicographically positive half of the other block offsets follows (each
// unordered block pair once).
inline void build_stencil(Geometry &g, const double search[3], int kind, bool autocorr) {
    const int bf = g.bf, bf3 = bf * bf * bf;
    const int DB = (g.K + bf - 1) / bf;
    g.DB = DB;
    g.nsten = 0;
    auto push = [&](int ox, int oy, int oz, int l0, int span) {
        g.sten[g.nsten] = (ox + 64) | ((oy + 64) << 8) | ((oz + 64) << 16) | (l0 << 24);
        float sp;
        std::memcpy(&sp, &span, 4);
        g.stenD[g.nsten] = make_float4((float)(ox * bf * g.c[0]), (float)(oy * bf * g.c[1]),
                                       (float)(oz * bf * g.c[2]), sp);
        g.nsten++;
    };
    // gap along d between fine cell f (block-relative) and the block [0, bf),
    // less the few-ulp distance a point may lie outside its cell (the digitiser
    // picks the cell with a rounded reciprocal, in FP32 for float32 input)
    const double slop = std::ldexp(std::max(g.L[0], std::max(g.L[1], g.L[2])), -19);
    auto gap = [&](int f, int d) {
        return std::max(0.0, g.c[d] * std::max(0, std::max(f - bf, -f - 1)) - slop);
    };
    auto keep = [&](int fx, int fy, int fz) {
        double gx = gap(fx, 0), gy = gap(fy, 1), gz = gap(fz, 2);
        const double slack = 1.0 + 1e-9;
        if (kind == 0) return gx * gx + gy * gy + gz * gz <= search[0] * search[0] * slack;
        return gx * gx + gy * gy <= search[0] * search[0] * slack && gz <= search[2] * slack;
    };
    int Dx = std::min(DB, g.pbc ? DB : g.nb[0] - 1);
    int Dy = std::min(DB, g.pbc ? DB : g.nb[1] - 1);
    int Dz = std::min(DB, g.pbc ? DB : g.nb[2] - 1);
    push(0, 0, 0, 0, bf3);
    for (int ox = -Dx; ox <= Dx; ox++)
        for (int oy = -Dy; oy <= Dy; oy++)
            for (int oz = -Dz; oz <= Dz; oz++) {
                if (ox == 0 && oy == 0 && oz == 0) continue;
                if (autocorr) {
                    bool pos = ox > 0 || (ox == 0 && (oy > 0 || (oy == 0 && oz > 0)));
                    if (!pos) continue;
                }
                int run = -1;
                for (int l = 0; l <= bf3; l++) {
                    bool k = false;
                    if (l < bf3) {
                        const int lx = l / (bf * bf), ly = (l / bf) % bf, lz = l % bf;
                        k = keep(ox * bf + lx, oy * bf + ly, oz * bf + lz);
                    }
                    if (k && run < 0) run = l;
                    if (!k && run >= 0) {
                        push(ox, oy, oz, run, l - run);
                        run = -1;
                    }
                }
            }
    g.nself = autocorr ? 1 : 0;
}

// Coordinates are FP32 offsets from the point's block corner, |u| <= bf c, and
// stencil offsets are block offsets of at most DB blocks.
inline ErrModel err_model(const Geometry &g) {
    ErrModel em;
    em.cmax = g.bf * std::max(g.c[0], std::max(g.c[1], g.c[2]));
    em.K = g.DB;
    em.Lmax = std::max(g.L[0], std::max(g.L[1], g.L[2]));
    return em;
}

inline double max_nan(const double *r, int n) {
    double m = r[0];
    for (int k = 0; k < n; k++) {
        if (std::isnan(r[k]) || std::isnan(m)) m = NAN;
        else m = std::max(m, r[k]);
    }
    return m;
}

}  // namespace gbp
