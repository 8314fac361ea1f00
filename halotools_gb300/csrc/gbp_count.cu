// Pair-count kernels (sm_103a).  Replace the cell walks of
// npairs_3d_engine.pyx:103-182, npairs_xy_z_engine.pyx:143-194,
// npairs_s_mu_engine.pyx:150-229 and marked_npairs_3d_engine.pyx:150-216.
//
// Work decomposition: a persistent grid pulls work items (cell, first i,
// i count <= 256) from an atomic cursor.  Each thread holds one i-point (FP32,
// relative to its cell) in registers; the points of the item's stencil cells
// are staged through shared memory with the cell offset o*c already added.
// When the i count is small the CTA's warps split the staged j range into
// groups instead of idling.
//
// Two stages per warp.  Stage 1 (every candidate): a broadcast LDS.128, three
// FSUB, the squared quantities and one compare against the outermost edge;
// in-range pairs are compacted with a ballot into a 64-entry per-warp queue
// {v0, v1, i, j | symmetric-flag}.  Stage 2 (every 32 queued pairs, all lanes
// busy): float-bit table lookup of the bin, the guard-band test, and the
// histogram update.  Most candidates of a cube stencil are out of range, so
// the binning work is paid only for the ~15-40% that count.
//
// Exactness: the FP32 value is compared with FP32 thresholds that bracket each
// FP64 edge by a rigorous error bound (built on the host).  A pair whose FP32
// value falls inside a bracket is re-evaluated in FP64 with the reference's
// operation order, ((x1 - shift) - x2) squared and summed left to right,
// unfused (npairs_3d_engine.pyx:167-176), so integer counts equal the
// reference's.
//
// Histograms: 1-D counts go to lane-private u32 bins in shared memory (no
// atomics, no bank conflicts: bin-major, lane-minor); 2-D counts go to shared
// u32 copies updated with shared atomics; marked sums go to lane-private FP32
// (sum, compensation) pairs (Kahan).  All are flushed to global u64 / FP64
// histograms at the end (integer copies also early, before a u32 could wrap).
#include "gbp_internal.cuh"

#include "gbp_device.cuh"

#define SYM_BIT 0x80000000u

// One in-range pair for stage 2: its FP32 value(s), the i-slot and j-slot it
// came from (indices are looked up only when the pair needs the FP64 recheck)
// and whether it stands for both orders.
struct PairV {
    float v0, v1;
    int iu, jj;
    bool sym;
    float w;  // weighted modes: the pair's weight
    int tg;   // weighted jackknife: tag_i | tag_j << 16
};
struct Ix {
    const float4 *u;  // i-slots {x, y, z, sorted index bits}
    const int *jw;    // sorted index of each j-slot
    __device__ __forceinline__ int ui(int s) const { return __float_as_int(u[s].w); }
};

// ---------------- stage 2: 1-D (3-D separation) ----------------
// Bins of a pair whose FP32 value may straddle an edge.  Returns 0 with k[0]
// the bin when FP32 decides it after all; else re-evaluates in FP64 and
// returns the number of orders (1, or 2 for a symmetric pair) written to k[].
__device__ __noinline__ int slow_3d(float v, int b0, int is, int js, bool sym, int *k,
                                    const AxisSm &A, const CountArgs &a) {
    int kk = walk_bin(v, b0, A);
    if (kk >= 0) {
        k[0] = kk;
        return 0;
    }
    if (is < 0 || js < 0) {  // never a real pair (idle lane or padding)
        k[0] = A.nb;
        return 0;
    }
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, is, p);
    ref_pos(a, 1, js, q);
    k[0] = exact_bin(exact_pair(p, q, a).s2, b0, A);
    if (!sym) return 1;
    k[1] = exact_bin(exact_pair(q, p, a).s2, b0, A);
    return 2;
}

template <bool LANE, class HT>
__device__ __forceinline__ void bin_3d(const PairV &p, HT *h, const AxisSm &A, const Ix &ix,
                                       const CountArgs &a) {
    const float v = p.v0;
    const bool sym = p.sym;
    const unsigned w = sym ? 2u : 1u;
    float4 t = lut_entry_c<false>(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        int n = slow_3d(v, __float_as_int(t.x), ix.ui(p.iu), ix.jw[p.jj], sym, k, A, a);
        if (n == 0) {
            b = k[0];
        } else {
            for (int q = 0; q < n; q++) {
                if (LANE) h[k[q] * 32] += 1u;
                else if (k[q] < A.nb) atomicAdd(&h[k[q]], (HT)1);
            }
            return;
        }
    }
    if (LANE) h[b * 32] += w;
    else if (b < A.nb) atomicAdd(&h[b], (HT)w);
}

// ---------------- stage 2: jackknife (counts + pair ends by tag) ----------------
// Each ordered pair in bin k adds 1 to the counts and 1 to (tag_i, k) and to
// (tag_j, k) of the CTA's table; with N_k(s) = sum of those ends, the count
// without subsample s is C_k - N_k(s) / 2 (npairs_jackknife_3d_engine.pyx:238-289).
__device__ __forceinline__ void bin_jack(const PairV &p, int ti, int tj, unsigned *h,
                                         unsigned long long *tab, const AxisSm &A, const Ix &ix,
                                         const CountArgs &a) {
    const float v = p.v0;
    const int ts = A.nb + 1;
    float4 t = lut_entry_c<false>(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        const int n = slow_3d(v, __float_as_int(t.x), ix.ui(p.iu), ix.jw[p.jj], p.sym, k, A, a);
        if (n == 0) {
            b = k[0];
        } else {
            for (int q = 0; q < n; q++) {
                h[k[q] * 32] += 1u;
                atomicAdd(&tab[ti * ts + k[q]], 1ull);
                atomicAdd(&tab[tj * ts + k[q]], 1ull);
            }
            return;
        }
    }
    const unsigned w = p.sym ? 2u : 1u;
    h[b * 32] += w;
    atomicAdd(&tab[ti * ts + b], (unsigned long long)w);
    atomicAdd(&tab[tj * ts + b], (unsigned long long)w);
}

// ---------------- stage 2: marked (Kahan in lane-private FP32 pairs) ----------------
__device__ __forceinline__ void kahan_add(float *hs, float *hc, int b, float x) {
    float s = hs[b * 32], c = hc[b * 32];
    float y = x - c;
    float t = s + y;
    hc[b * 32] = (t - s) - y;
    hs[b * 32] = t;
}

__device__ __forceinline__ void bin_mark(const PairV &p, float *hs, float *hc, const AxisSm &A,
                                         const Ix &ix, const CountArgs &a) {
    const float v = p.v0, wt = p.v1;
    const bool sym = p.sym;
    float4 t = lut_entry_c<false>(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        int n = slow_3d(v, __float_as_int(t.x), ix.ui(p.iu), ix.jw[p.jj], sym, k, A, a);
        if (n == 0) {
            b = k[0];
        } else {
            for (int q = 0; q < n; q++)
                if (k[q] < A.nb) kahan_add(hs, hc, k[q], wt);
            return;
        }
    }
    if (b < A.nb) kahan_add(hs, hc, b, sym ? 2.0f * wt : wt);
}

// ---------------- weighted 2-D sums (marked xy_z, weighted s_mu) ----------------
// hi takes each weight by atomic add; the add's exact rounding error (TwoSum on
// the value the atomic returned, the sum it stored being that value plus x
// rounded to nearest) goes to lo, so hi + lo carries the sum to about 2^-48.
struct WSink {
    float *hi, *lo;
    unsigned long long *tab;  // jackknife (rp, pi): the global (tag, bin) table of pair ends
    int tstride;              // its row length (bins per tag)
};

__device__ __forceinline__ void w2_add(const WSink &s, int b, float x) {
    const float old = atomicAdd(&s.hi[b], x);
    const float t = old + x;
    const float bp = t - old;
    const float err = (old - (t - bp)) + (x - bp);
    if (err != 0.0f) atomicAdd(&s.lo[b], err);
}

// What a binned pair adds besides its count: X_W its weight w (times the
// multiplicity m), X_TAG one pair end per tag (w holds tag_i | tag_j << 16),
// X_TAGW its weight to the sums and to both ends' rows of the FP64 table (tg
// holds the tags)
#define X_NONE 0
#define X_W 1
#define X_TAG 2
#define X_TAGW 3
template <int X>
__device__ __forceinline__ void sink_add(const WSink &s, int b, int m, float w, int tg = 0) {
    if (X == X_W) w2_add(s, b, m == 2 ? 2.0f * w : w);
    if (X == X_TAG) {
        const int t = __float_as_int(w);
        atomicAdd(&s.tab[(t & 0xffff) * s.tstride + b], (unsigned long long)m);
        atomicAdd(&s.tab[(t >> 16) * s.tstride + b], (unsigned long long)m);
    }
    if (X == X_TAGW) {
        const float x = m == 2 ? 2.0f * w : w;
        w2_add(s, b, x);
        double *t = reinterpret_cast<double *>(s.tab);
        atomicAdd(&t[(tg & 0xffff) * s.tstride + b], (double)x);
        atomicAdd(&t[(tg >> 16) * s.tstride + b], (double)x);
    }
}

// ---------------- stage 2: weighted jackknife, 3-D ----------------
// w_i w_j to the sums and to both ends' table rows, per ordered pair
// (npairs_jackknife_3d_engine.pyx: jweight with weights)
__device__ __forceinline__ void bin_3dw(const PairV &p, const WSink &ws, const AxisSm &A,
                                        const Ix &ix, const CountArgs &a) {
    const float v = p.v0;
    const float4 t = lut_entry_c<false>(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        const int n = slow_3d(v, __float_as_int(t.x), ix.ui(p.iu), ix.jw[p.jj], p.sym, k, A, a);
        if (n == 0) {
            b = k[0];
        } else {
            for (int q = 0; q < n; q++)
                if (k[q] < A.nb) sink_add<X_TAGW>(ws, k[q], 1, p.w, p.tg);
            return;
        }
    }
    if (b < A.nb) sink_add<X_TAGW>(ws, b, p.sym ? 2 : 1, p.w, p.tg);
}

// ---------------- deferred FP64 rechecks (s, mu') ----------------
// A pair whose bins FP32 cannot settle joins the warp's ring as {i, j, walk
// starts and flags, weight}; the warp re-evaluates 32 at once, every lane busy,
// which costs one FP64 warp instruction where a lone lane's recheck costs the
// same.  A pair that finds the ring full is re-evaluated at once by its lane.
#define RQ_SYM 1
#define RQ_KNOWN_A 2
struct RQ {
    int4 *ring;      // GBP_RQCAP entries of this warp
    unsigned *tail;  // slots taken so far
    unsigned head;   // warp-uniform: slots re-evaluated so far
};

__device__ __forceinline__ bool rq_push(const RQ &q, int4 e) {
    const unsigned t = atomicAdd(q.tail, 1u);
    if (t - q.head >= GBP_RQCAP) return false;
    q.ring[t % GBP_RQCAP] = e;
    return true;
}

// ---------------- stage 2: (rp, pi) ----------------
// (rechecks are rare here, about 1e-4 of the pairs: each lane re-evaluates its
// own).  CNT: integer counts into hw; X: what else the pair adds (sink_add).
template <class HT, bool CNT, int X>
__device__ __noinline__ void slow_xyz(float v0, float v1, int b0a, int b0b, int is, int js,
                                      bool sym, float wt, int tg, HT *hw, const WSink ws,
                                      int stride, const AxisSm &A, const AxisSm &Bx,
                                      const CountArgs &a) {
    int ka = walk_bin(v0, b0a, A);
    int kb = walk_bin(v1, b0b, Bx);
    if (ka >= 0 && kb >= 0) {
        if (ka < A.nb && kb < Bx.nb) {
            if (CNT) atomicAdd(&hw[ka * stride + kb], (HT)(sym ? 2 : 1));
            sink_add<X>(ws, ka * stride + kb, sym ? 2 : 1, wt, tg);
        }
        return;
    }
    // a settled bin beyond the last edge leaves the pair out in both orders
    if (ka >= A.nb || kb >= Bx.nb) return;
    if (is < 0 || js < 0) return;  // never a real pair (idle lane or padding)
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, is, p);
    ref_pos(a, 1, js, q);
    for (int o = 0; o < (sym ? 2 : 1); o++) {
        const Exact3 r = o == 0 ? exact_pair(p, q, a) : exact_pair(q, p, a);
        const int ea = ka >= 0 ? ka : exact_bin(r.dxy, b0a, A);
        const int eb = kb >= 0 ? kb : exact_bin(r.dz2, b0b, Bx);
        if (ea < A.nb && eb < Bx.nb) {
            if (CNT) atomicAdd(&hw[ea * stride + eb], (HT)1);
            sink_add<X>(ws, ea * stride + eb, 1, wt, tg);
        }
    }
}

template <class HT, bool CNT, int X>
__device__ __forceinline__ void bin_xyz(const PairV &p, HT *hw, const WSink &ws, int stride,
                                        const AxisSm &A, const AxisSm &Bx, const Ix &ix,
                                        const CountArgs &a) {
    const float v0 = p.v0, v1 = p.v1;
    const bool sym = p.sym;
    float4 e0 = lut_entry_c<false>(v0, A);
    float4 e1 = lut_entry_c<false>(v1, Bx);
    int ba = __float_as_int(e0.x) + (v0 > e0.y ? 1 : 0);
    int bb = __float_as_int(e1.x) + (v1 > e1.y ? 1 : 0);
    bool amb = ((v0 > e0.z) & !(v0 > e0.y)) | ((v1 > e1.z) & !(v1 > e1.y));
    if (amb) {
        slow_xyz<HT, CNT, X>(v0, v1, __float_as_int(e0.x), __float_as_int(e1.x), ix.ui(p.iu),
                              ix.jw[p.jj], sym, p.w, p.tg, hw, ws, stride, A, Bx, a);
        return;
    }
    if ((ba < A.nb) & (bb < Bx.nb)) {
        if (CNT) atomicAdd(&hw[ba * stride + bb], (HT)(sym ? 2 : 1));
        sink_add<X>(ws, ba * stride + bb, sym ? 2 : 1, p.w, p.tg);
    }
}

// ---------------- stage 2: (s, mu') ----------------
// v = s^2 on axis 0; q = dxy / s^2 on axis 1, whose FP32 error depends on s:
// the s table's 4th field holds the q error bound for the slot's smallest s.
// A queued pair: {i, j, s walk start | mu' walk start << 11 | flags << 22, weight}.
template <class HT, bool CNT, int X>
__device__ __forceinline__ void exact_smu(const int4 &e, HT *hw, const WSink &ws, int stride,
                                          const AxisSm &A, const AxisSm &Q, const CountArgs &a);

template <class HT, bool CNT, int X>
__device__ __noinline__ void slow_smu(float v, float q, float qb, int b0s, int is, int js,
                                      bool sym, float wt, HT *hw, const WSink ws, int stride,
                                      const AxisSm &A, const AxisSm &Q, const RQ &rq,
                                      const CountArgs &a) {
    int ks = walk_bin(v, b0s, A);
    int kq = -1, gq = 0;
    if (ks >= 0 && ks < A.nb && v > 0.0f) {
        int g = 0;
        while (g < Q.nb && q > Q.hi[g] + qb) g++;
        if (!(g < Q.nb && q > Q.lo[g] - qb)) kq = g;
        gq = g > 0 ? g - 1 : 0;  // mu'^2 of both orders lies above edge g - 2
    }
    if (ks >= A.nb) return;  // beyond the s gate: never counted
    if (ks >= 0 && kq >= 0) {
        if (kq < Q.nb) {
            if (CNT) atomicAdd(&hw[ks * stride + kq], (HT)(sym ? 2 : 1));
            sink_add<X>(ws, ks * stride + kq, sym ? 2 : 1, wt);
        }
        return;
    }
    if (is < 0 || js < 0) return;  // never a real pair (idle lane or padding)
    const int ss = ks >= 0 ? ks : -1 - ks;
    const int4 e = make_int4(is, js,
                             ss | (gq << 11) | (((sym ? RQ_SYM : 0) | (ks >= 0 ? RQ_KNOWN_A : 0)) << 22),
                             __float_as_int(wt));
    if (rq_push(rq, e)) return;
    atomicAdd(a.nrecheck, 1ull);
    exact_smu<HT, CNT, X>(e, hw, ws, stride, A, Q, a);
}

// FP64 (s, mu') bins of a queued pair: sqr_mu = dxy / s^2 as an FP64 quotient,
// 0 at s = 0 (npairs_s_mu_engine.pyx:200-226)
template <class HT, bool CNT, int X>
__device__ __forceinline__ void exact_smu(const int4 &e, HT *hw, const WSink &ws, int stride,
                                          const AxisSm &A, const AxisSm &Q, const CountArgs &a) {
    double p[3], qq[3];
    ref_pos(a, 0, e.x, p);
    ref_pos(a, 1, e.y, qq);
    const int ss = e.z & 0x7ff, sq = (e.z >> 11) & 0x7ff, fl = e.z >> 22;
    const float wt = __int_as_float(e.w);
    for (int o = 0; o < ((fl & RQ_SYM) ? 2 : 1); o++) {
        const Exact3 r = o == 0 ? exact_pair(p, qq, a) : exact_pair(qq, p, a);
        const int es = (fl & RQ_KNOWN_A) ? ss : exact_bin(r.s2, ss, A);
        if (es >= A.nb) continue;
        const double mu2 = (r.s2 > 0.0) ? __ddiv_rn(r.dxy, r.s2) : 0.0;
        const int eq = exact_bin(mu2, sq, Q);
        if (eq >= Q.nb) continue;
        if (CNT) atomicAdd(&hw[es * stride + eq], (HT)1);
        sink_add<X>(ws, es * stride + eq, 1, wt);
    }
}

template <class HT, bool CNT, int X>
__device__ __forceinline__ void bin_smu(const PairV &p, HT *hw, const WSink &ws, int stride,
                                        const AxisSm &A, const AxisSm &Q, const Ix &ix,
                                        const RQ &rq, const CountArgs &a) {
    const float v = p.v0, dxy = p.v1;
    const bool sym = p.sym;
    float4 e0 = lut_entry_c<true>(v, A);
    int bs = __float_as_int(e0.x) + (v > e0.y ? 1 : 0);
    if (bs >= A.nb) return;  // beyond the s gate
    float q = __fdividef(dxy, v);
    float qb = e0.w;
    // nearest edges around q must be farther than qb
    const QBin e1 = lut_q(q, Q);
    const int bq = e1.b;
    bool amb = ((v > e0.z) & !(v > e0.y)) | !(q - e1.below > qb) | !(e1.above - q > qb) |
               e1.walk;
    if (amb) {
        slow_smu<HT, CNT, X>(v, q, qb, __float_as_int(e0.x), ix.ui(p.iu), ix.jw[p.jj], sym, p.w,
                              hw, ws, stride, A, Q, rq, a);
        return;
    }
    if (bq < Q.nb) {
        if (CNT) atomicAdd(&hw[bs * stride + bq], (HT)(sym ? 2 : 1));
        sink_add<X>(ws, bs * stride + bq, sym ? 2 : 1, p.w);
    }
}

// ---------------- marking functions (marking_functions.pyx:21-218) ----------------
// WF 1 and 2 evaluate in FP32 (product, sum).  WF 0 evaluates any id 1-17 in
// FP64 from the FP64 weights, exactly as the reference does (comparisons
// included), and rounds the result to FP32 for accumulation.
__device__ __forceinline__ double wfunc64(int id, const double *A, const double *B) {
    switch (id) {
    case 1: return A[0] * B[0];
    case 2: return A[0] + B[0];
    case 3: return (A[0] == B[0]) ? A[1] * B[1] : 0.0;
    case 4: return (A[0] != B[0]) ? A[1] * B[1] : 0.0;
    case 5: return (B[0] > A[0]) ? A[1] * B[1] : 0.0;
    case 6: return (B[0] < A[0]) ? A[1] * B[1] : 0.0;
    case 7: return (B[0] > (A[0] + A[1])) ? B[1] : 0.0;
    case 8: return (B[0] < (A[0] + A[1])) ? B[1] : 0.0;
    case 9: return (fabs(A[0] - B[0]) < A[1]) ? B[1] : 0.0;
    case 10: return (fabs(A[0] - B[0]) > A[1]) ? B[1] : 0.0;
    case 11: return (B[0] > A[0] * A[1]) ? B[1] : 0.0;
    case 12: return A[0] * B[0] * (A[1] * B[1] + A[2] * B[2] + A[3] * B[3]);
    case 13: {
        double d = A[1] * B[1] + A[2] * B[2] + A[3] * B[3];
        return A[0] * B[0] * d * d;
    }
    case 14: return A[0] * B[0] * (A[1] * B[1] + A[2] * B[2]);
    case 15: {
        double d = A[1] * B[1] + A[2] * B[2];
        return A[0] * B[0] * d * d;
    }
    case 16:
        if (A[4] == B[4]) {
            double d = A[1] * B[1] + A[2] * B[2] + A[3] * B[3];
            return A[0] * B[0] * d * d;
        }
        return 0.0;
    case 17:
        if (A[4] != B[4]) {
            double d = A[1] * B[1] + A[2] * B[2] + A[3] * B[3];
            return A[0] * B[0] * d * d;
        }
        return 0.0;
    default: return 0.0;
    }
}

// Stage-1 range test folded into one FP32 value per pair: R0 - dx^2 - dy^2 - dz^2
// (3-D, s_mu) or (R0 - dx^2 - dy^2) | (R1 - dz^2) bits (xy_z).  Its sign bit is
// set exactly when the pair lies beyond the thresholds.
template <int MODE>
__device__ __forceinline__ unsigned out_bits(const float4 &u, const float4 &t, float R0, float R1) {
    const float dx = u.x - t.x, dy = u.y - t.y, dz = u.z - t.z;
    if (gbp_mode_xyz(MODE)) {
        const float a = fmaf(-dy, dy, fmaf(-dx, dx, R0));
        const float b = fmaf(-dz, dz, R1);
        return __float_as_uint(a) | __float_as_uint(b);
    }
    return __float_as_uint(fmaf(-dz, dz, fmaf(-dy, dy, fmaf(-dx, dx, R0))));
}

// ---------------- kernel ----------------
// Warp-centric: every warp independently pulls items, loads the i-points of
// its item (two per lane), walks the item's stencil group 32 j-points at a
// time through a per-warp buffer and feeds its own queue.  There is no CTA
// barrier in the main loop; the CTA only shares the read-only tables.
template <int MODE, int WF>
__global__ void __launch_bounds__(GBP_BLOCK, 2) k_count(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr bool JACK2 = (MODE == MODE_JACKXYZ);  // jackknife (rp, pi): w1 / w2 hold tags
    constexpr bool XYZF = gbp_mode_xyz(MODE);  // (rp, pi) geometry
    constexpr bool SMUF = gbp_mode_smu(MODE);  // (s, mu') geometry
    constexpr bool TWO = XYZF || SMUF;
    // weighted 2-D: a marking function's value per pair into the CTA's (hi, lo)
    // sums; weighted s_mu also counts
    // weighted jackknife (3-D, (rp, pi)): rows {w, tag} per point, w_i w_j to the
    // sums and to both ends' FP64 table rows
    constexpr bool JW = (MODE == MODE_JACKW || MODE == MODE_JACKXYZW);
    constexpr bool W2 = (MODE == MODE_XYZW || MODE == MODE_SMUW || JW);
    constexpr bool MW2 = (MODE == MODE_XYZW || MODE == MODE_SMUW);  // marking-function sums
    constexpr bool CNT2 = (MODE != MODE_XYZW && !JW);
    constexpr bool MARK = (MODE == MODE_MARK);
    constexpr bool MW = MARK || MW2;  // per-pair marking function of staged weights
    // what 2-D bins add besides counts
    constexpr int XS = JW ? X_TAGW : W2 ? X_W : JACK2 ? X_TAG : X_NONE;
    constexpr bool MARKC = (MODE == MODE_MARKC);  // nw = channels of product marks
    constexpr bool COLS = MARKC || JW;  // nw FP32 columns staged per point
    // prefetch of the next j batch's slot: the modes whose registers hold it
    // without spilling (measured: 2-3 % on the (rp, pi) and marked counts)
    constexpr bool PREF = MODE == MODE_3D || MODE == MODE_3DS || MODE == MODE_XYZ ||
                          MODE == MODE_MARK || MODE == MODE_MARKC || MODE == MODE_JACK ||
                          MODE == MODE_JACKW;
    constexpr unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, nb1 = TWO ? a.ax[1].nb : 0;
    const int T0 = a.ax[0].T, T1 = TWO ? a.ax[1].T : 0;
    const int copies = a.hist_copies;  // 2-D / wide: GBP_WARPS (one per warp) or 0 (global)
    constexpr bool JACK = (MODE == MODE_JACK);    // w1 / w2 hold the subsample tags
    const int nw = (MW || COLS || JACK || JACK2) ? a.nw : 0;
    // MARKC: channel pairs and the staged column count (sorted form: zero columns
    // pad to 2 mP, a power of two)
    const int mP = MARKC ? gbp_markc_pairs(nw) : 1;
    const int ncol = MARKC ? gbp_markc_cols(nw) : nw;
    const bool cpow2 = ncol > 0 && (ncol & (ncol - 1)) == 0;
    const int lcol = 31 - __clz(ncol > 0 ? ncol : 1);
    const bool msort = MARKC && gbp_markc_sorted(nw);
    // staged element t of a column table: its row
    auto col_row = [&](int t) { return cpow2 ? t >> lcol : t / ncol; };
    const int jwb = MW ? (WF == 0 ? 8 * nw : 4) : COLS ? 4 * ncol : (JACK || JACK2) ? 4 : 0;
    const SmemLayout L = gbp_smem_layout(MODE, T0, T1, nb0, nb1, a.nsten, copies, jwb, a.ntag);
    if (gbp_smem_too_small(L.total, a.err)) return;
    unsigned *s_l0 = (unsigned *)(smem + L.off_lut0);
    unsigned *s_l1 = (unsigned *)(smem + L.off_lut1);
    float2 *s_hl0 = (float2 *)(smem + L.off_hl0);
    float2 *s_hl1 = (float2 *)(smem + L.off_hl1);
    float4 *s_hq = SMUF ? (float4 *)(smem + L.off_hl1) : nullptr;
    // this warp's 32 staged j-points: x, y, z (cell offset added) and sorted index
    float *jx = (float *)(smem + L.off_j) + warp * 128;
    float *jy = jx + 32, *jz = jx + 64;
    int *jix = (int *)(jx + 96);
    // the same j-points with each coordinate twice, for the packed stage 1
    ulonglong2 *jxy = (ulonglong2 *)(smem + L.off_j2) + warp * 32;
    unsigned long long *jzz = (unsigned long long *)(smem + L.off_j2 + GBP_JCAP * 16) + warp * 32;
    float *jw = (float *)(smem + L.off_jw) + warp * 32 * (COLS ? ncol : 1);
    double *jw64 = (double *)(smem + L.off_jw) + warp * 32 * (nw > 0 ? nw : 1);
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    double *s_E1 = (double *)(smem + L.off_E1);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    float *s_hi1 = (float *)(smem + L.off_hi1);
    float *s_lo1 = (float *)(smem + L.off_lo1);
    int *s_off = (int *)(smem + L.off_off);
    unsigned *s_hist = (unsigned *)(smem + L.off_hist);
    // this warp's 64 i-points (and their weights) for stage 2, at slots gbp_uslot(iu)
    // this warp's i-slots {x, y, z, sorted index bits}: one 16-byte load per pair end
    float4 *u4 = (float4 *)(smem + L.off_q) + warp * GBP_USLOTS;
    float *s_uw = (float *)(smem + L.off_q + GBP_WARPS * GBP_USLOTS * 16) +
                  warp * GBP_USLOTS * (COLS ? ncol : 1);
    // MARKC per-round form (up to 4 or over 16 channels): this warp's binned pairs
    // of one round {bin | multiplicity << 16, second bin, i, j}
    int4 *s_rec = (int4 *)(smem + L.off_rec) + warp * 32;
    // MARKC sorted, per warp and code batch: each code's bin, the codes sorted by
    // bin, and per bin its count and (after the scatter) its end
    unsigned char *s_bin = (unsigned char *)(smem + L.off_rec) + warp * gbp_markc_sort_bytes(nb0);
    unsigned short *s_rec2 = (unsigned short *)(s_bin + GBP_MARKC_CODES);
    int *s_cnt = (int *)(s_bin + 3 * GBP_MARKC_CODES), *s_cur = s_cnt + (nb0 + 1);
    // (s, mu'): this warp's ring of deferred FP64 rechecks and its tail
    constexpr bool RQM = SMUF;
    RQ rq{(int4 *)(smem + L.off_rq) + warp * GBP_RQCAP,
          (unsigned *)(smem + L.off_rq + GBP_WARPS * GBP_RQCAP * 16) + warp, 0u};
    double *s_uw64 = (double *)(smem + L.off_q + GBP_WARPS * GBP_USLOTS * 16) +
                     warp * GBP_USLOTS * (nw > 0 ? nw : 1);
    const Ix ix{u4, jix};
    // this warp's pair codes of one 32-point j batch: at most 64 x 32 (marked
    // modes other than the sorted channel form: one i-point at a time, 32 x 32)
    unsigned short *s_code =
        (unsigned short *)(smem + L.off_code) +
        warp * ((MARK || (MARKC && !msort)) ? 1024 : msort ? GBP_MARKC_CODES : 2048);

    // 3-D: each slot's threshold pair beside its word, so that the two loads of
    // a lookup are independent (the shared pair of the compact form is read
    // through the word: 20.49 -> 20.30 ms on the 10M-point count)
    float2 *s_t0 = (float2 *)(smem + L.off_lut0 + gbp_align(T0 * 4, 16));
    if (MODE == MODE_3D)
        for (int i = tid; i < T0; i += GBP_BLOCK) {
            const float4 e = a.ax[0].lut[i];
            s_t0[i] = make_float2(e.y, e.z);
        }
    lut_compact(a.ax[0].lut, T0, a.ax[0].hi, a.ax[0].lo, nb0, s_l0, s_hl0, SMUF, nullptr, tid,
                GBP_BLOCK);
    if (TWO) lut_compact(a.ax[1].lut, T1, a.ax[1].hi, a.ax[1].lo, nb1, s_l1, s_hl1, false, s_hq,
                         tid, GBP_BLOCK);
    for (int i = tid; i < nb0; i += GBP_BLOCK) {
        s_E0[i] = a.ax[0].E[i];
        s_hi0[i] = a.ax[0].hi[i];
        s_lo0[i] = a.ax[0].lo[i];
    }
    for (int i = tid; i < nb1; i += GBP_BLOCK) {
        s_E1[i] = a.ax[1].E[i];
        s_hi1[i] = a.ax[1].hi[i];
        s_lo1[i] = a.ax[1].lo[i];
    }
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    const int nbin = (nb0 + 1) * (TWO ? nb1 + 1 : 1);
    // this warp's histogram words: lane-private (3-D, marked) or its own copy
    const int warp_words = (MODE == MODE_3D || JACK) ? (nb0 + 1) * 32
                           : (MARK || (MARKC && !msort)) ? (nb0 + 1) * 32 * 2
                           : MARKC ? (nb0 + 1) * mP * 4
                           : (copies ? nbin : 0);
    unsigned *wh = s_hist + warp * warp_words;
    for (int i = lane; i < warp_words; i += 32) wh[i] = 0u;
    if (msort)
        for (int i = lane; i <= nb0; i += 32) s_cnt[i] = 0;
    if (RQM && lane == 0) *rq.tail = 0u;
    // jackknife: the CTA's (tag, bin) table of pair ends, after the warps' counts
    unsigned long long *s_tab =
        (unsigned long long *)(smem + L.off_hist + gbp_align(GBP_WARPS * (nb0 + 1) * 32 * 4, 16));
    if (JACK)
        for (int i = tid; i < a.ntag * (nb0 + 1); i += GBP_BLOCK) s_tab[i] = 0ull;
    // weighted 2-D: the CTA's (hi, lo) FP32 sums and FP64 totals, after the copies
    float *s_whi = (float *)(smem + L.off_hist + gbp_align(copies * nbin * 4, 16));
    float *s_wlo = s_whi + gbp_align(nbin * 4, 16) / 4;
    double *s_wacc = (double *)(s_wlo + gbp_align(nbin * 4, 16) / 4);
    const WSink wsink{s_whi, s_wlo, a.htag, nbin};
    if (W2)
        for (int i = tid; i < nbin; i += GBP_BLOCK) {
            s_whi[i] = 0.f;
            s_wlo[i] = 0.f;
            s_wacc[i] = 0.0;
        }
    unsigned w2_binned = 0;  // pairs this warp binned since it last moved (hi, lo) to FP64
    AxisSm A0{nullptr, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi,
              s_l0, s_hl0, nullptr};
    AxisSm A1{nullptr, s_hi1, s_lo1, s_E1, nb1, TWO ? a.ax[1].S : 0, TWO ? a.ax[1].B : 0,
              TWO ? a.ax[1].vlo : 0.f, TWO ? a.ax[1].vhi : 0.f, s_l1, s_hl1, s_hq};
    const int stride2 = nb1 + 1;
    unsigned *hl = wh + lane;                       // 1-D: lane-private column
    float *hs = (float *)wh + lane;                 // marked: sums
    float *hc = hs + (nb0 + 1) * 32;                // marked: compensations
    // MARKC: (bin, channel pair) packed sums and negated compensations
    unsigned long long *hs2 = (unsigned long long *)wh, *hc2 = hs2 + (nb0 + 1) * mP;
    const int nitems = *a.nitems;
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    // stage-1 thresholds: top * (1 + 2^-18) + 1e-30 covers the rounding of the
    // folded R - v against the stage-2 value v (three roundings of 2^-24 each)
    const float R0 = fmaf(a.top0, 0x1p-18f, a.top0) + 1.0e-30f;
    const float R1 = fmaf(a.top1, 0x1p-18f, a.top1) + 1.0e-30f;
    const unsigned long long RR0 = pk2(R0, R0), RR1 = pk2(R1, R1);
    unsigned long long drained = 0, cand = 0;
    int cur_mock = -1;   // mock whose histogram this warp is filling
    __syncthreads();

    // 2-D / wide histograms go to this warp's u32 copy, or (too many bins for
    // shared memory) straight to the mock's u64 global histogram
    auto bin_entry = [&](const PairV &e, int mk) {
        unsigned long long *gh = a.hist + (size_t)mk * a.hist_stride;
        if (MODE == MODE_3D) bin_3d<true>(e, hl, A0, ix, a);
        else if (JACK) bin_jack(e, (int)s_uw[e.iu], (int)jw[e.jj], hl, s_tab, A0, ix, a);
        else if (MODE == MODE_3DS) {
            if (copies) bin_3d<false>(e, wh, A0, ix, a); else bin_3d<false>(e, gh, A0, ix, a);
        } else if (XYZF) {
            if (copies) bin_xyz<unsigned, CNT2, XS>(e, wh, wsink, stride2, A0, A1, ix, a);
            else bin_xyz<unsigned long long, CNT2, XS>(e, gh, wsink, stride2, A0, A1, ix, a);
        } else if (SMUF) {
            if (copies) bin_smu<unsigned, CNT2, XS>(e, wh, wsink, stride2, A0, A1, ix, rq, a);
            else bin_smu<unsigned long long, CNT2, XS>(e, gh, wsink, stride2, A0, A1, ix, rq, a);
        } else if (MARK) bin_mark(e, hs, hc, A0, ix, a);
        else if (MODE == MODE_JACKW) bin_3dw(e, wsink, A0, ix, a);
    };
    // Bin the rest of the queue, add this warp's histogram to mock mk and clear it.
    // Re-evaluate queued rechecks in FP64, 32 at a time, until fewer than
    // `keep` wait (keep = 1: all of them); they go to mock mk's histogram.
    // Slots past a full ring were re-evaluated by their lanes: the tail
    // drops back to the last stored slot.
    auto rq_drain = [&](int mk, unsigned keep) {
        __syncwarp();
        const unsigned t = *(volatile unsigned *)rq.tail;
        const unsigned end = rq.head + min(t - rq.head, (unsigned)GBP_RQCAP);
        unsigned long long *gh = a.hist + (size_t)mk * a.hist_stride;
        while (end - rq.head >= keep && end != rq.head) {
            const unsigned n = min(end - rq.head, 32u);
            if ((unsigned)lane < n) {
                const int4 e = rq.ring[(rq.head + lane) % GBP_RQCAP];
                if (copies) exact_smu<unsigned, CNT2, XS>(e, wh, wsink, stride2, A0, A1, a);
                else exact_smu<unsigned long long, CNT2, XS>(e, gh, wsink, stride2, A0, A1, a);
            }
            if (lane == 0) atomicAdd(a.nrecheck, (unsigned long long)n);
            rq.head += n;
        }
        __syncwarp();
        if (lane == 0 && end != t) *rq.tail = end;
        __syncwarp();
    };
    // weighted 2-D: move the CTA's (hi, lo) FP32 sums into its FP64 totals (any
    // warp may, at any time: exchanging each word keeps every add counted once)
    auto w2_move = [&]() {
        for (int b = lane; b < nbin; b += 32) {
            const float h = atomicExch(&s_whi[b], 0.f);
            const float l = atomicExch(&s_wlo[b], 0.f);
            if (h != 0.f || l != 0.f) atomicAdd(&s_wacc[b], (double)h + (double)l);
        }
        w2_binned = 0;
    };
    auto warp_flush = [&](int mk) {
        if (RQM) {
            // the ring empties here, so its counters restart from 0
            rq_drain(mk, 1u);
            if (lane == 0) *rq.tail = 0u;
            rq.head = 0;
        }
        __syncwarp();
        unsigned long long *gh = a.hist + (size_t)mk * a.hist_stride;
        if (MODE == MODE_3D || JACK) {
            for (int b = 0; b <= nb0; b++) {
                unsigned long long v = hl[b * 32];
                hl[b * 32] = 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if (lane == 0 && v) atomicAdd(&gh[b], v);
            }
        } else if (MARKC && !msort) {
            // lane = (pair group g, channel c): channel c sums lanes c, c + nw, ...
            double *gd = a.histd + (size_t)mk * a.hist_stride;
            const int G = 32 / nw, c = lane % nw;
            for (int b = 0; b < nb0; b++) {
                const double v = (double)hs[b * 32] - (double)hc[b * 32];
                hs[b * 32] = 0.f;
                hc[b * 32] = 0.f;
                double tot = 0.0;
                for (int g = 0; g < G; g++) tot += __shfl_sync(FULL, v, g * nw + c);
                if (lane < nw && tot != 0.0) atomicAdd(&gd[lane * (nb0 + 1) + b], tot);
            }
        } else if (MARKC) {
            // one (bin, channel pair) per lane: its two channels' sums in FP64
            double *gd = a.histd + (size_t)mk * a.hist_stride;
            for (int i = lane; i < nb0 * mP; i += 32) {
                const int b = i / mP, c = 2 * (i - b * mP);
                const unsigned long long sv = hs2[i], cv = hc2[i];
                hs2[i] = 0ull;
                hc2[i] = 0ull;
                const double v0 = (double)__uint_as_float((unsigned)sv) +
                                  (double)__uint_as_float((unsigned)cv);
                const double v1 = (double)__uint_as_float((unsigned)(sv >> 32)) +
                                  (double)__uint_as_float((unsigned)(cv >> 32));
                if (c < nw && v0 != 0.0) atomicAdd(&gd[c * (nb0 + 1) + b], v0);
                if (c + 1 < nw && v1 != 0.0) atomicAdd(&gd[(c + 1) * (nb0 + 1) + b], v1);
            }
        } else if (MARK) {
            double *gd = a.histd + (size_t)mk * a.hist_stride;
            for (int b = 0; b < nb0; b++) {
                double v = (double)hs[b * 32] - (double)hc[b * 32];
                hs[b * 32] = 0.f;
                hc[b * 32] = 0.f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if (lane == 0 && v != 0.0) atomicAdd(&gd[b], v);
            }
        } else if (copies) {
            for (int b = lane; b < nbin; b += 32) {
                unsigned v = wh[b];
                wh[b] = 0u;
                if (v) atomicAdd(&gh[b], (unsigned long long)v);
            }
        }
        __syncwarp();
        drained = 0;
    };

    while (true) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.counter, 1);
        it = __shfl_sync(FULL, it, 0);
        if (it >= nitems) break;
        const int4 item = a.items[it];
        const int mock = item.x / a.ncells_mock;
        const int cell = item.x - mock * a.ncells_mock, ifirst = item.y;
        const int icnt = item.z & 127, s0 = (item.z >> 7) & 1023, s1 = (item.z >> 17) & 1023;
        if (mock != cur_mock) {
            // batched mocks: this warp's histogram changes owner here
            if (cur_mock >= 0) warp_flush(cur_mock);
            cur_mock = mock;
        }
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
        const int keybase = mock * a.ncells_mock;
        // two i-points per lane
        float4 u0 = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(-1));
        float4 u1 = u0;
        if (lane < icnt) u0 = a.pos1[ifirst + lane];
        if (lane + 32 < icnt) u1 = a.pos1[ifirst + 32 + lane];
        const int is0 = __float_as_int(u0.w), is1 = __float_as_int(u1.w);
        const unsigned long long UX = pk2(u0.x, u1.x), UY = pk2(u0.y, u1.y), UZ = pk2(u0.z, u1.z);
        u4[lane] = u0;
        u4[lane + 48] = u1;
        float w0 = 0.f, w1 = 0.f;
        double wa[5] = {0, 0, 0, 0, 0}, wb[5] = {0, 0, 0, 0, 0};
        if (JACK || JACK2) {
            s_uw[lane] = lane < icnt ? a.w1[ifirst + lane] : 0.f;
            s_uw[lane + 48] = lane + 32 < icnt ? a.w1[ifirst + 32 + lane] : 0.f;
        }
        if (MW) {
            if (WF == 0) {
                for (int k = 0; k < nw; k++) {
                    if (lane < icnt) wa[k] = a.w64_1[(int64_t)(ifirst + lane) * nw + k];
                    if (lane + 32 < icnt) wb[k] = a.w64_1[(int64_t)(ifirst + 32 + lane) * nw + k];
                }
            } else {
                if (lane < icnt) w0 = a.w1[ifirst + lane];
                if (lane + 32 < icnt) w1 = a.w1[ifirst + 32 + lane];
            }
            if (WF == 0) {
                for (int k = 0; k < nw; k++) {
                    s_uw64[lane * nw + k] = wa[k];
                    s_uw64[(lane + 48) * nw + k] = wb[k];
                }
            } else {
                s_uw[lane] = w0;
                s_uw[lane + 48] = w1;
            }
        }
        if (COLS) {
            // lanes over (point, column): whole rows read, contiguous stores; the
            // read-only loads of a batch are all issued before its stores
            for (int t0 = 0; t0 < 64 * ncol; t0 += 256) {
                float v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int t = t0 + 32 * u + lane, sp = col_row(t), q = t - sp * ncol;
                    v[u] = (t < 64 * ncol && sp < icnt && q < nw)
                               ? __ldg(&a.w1[(int64_t)(ifirst + sp) * nw + q]) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int t = t0 + 32 * u + lane, sp = col_row(t), q = t - sp * ncol;
                    if (t < 64 * ncol) s_uw[gbp_uslot(sp) * ncol + q] = v[u];
                }
            }
        }
        __syncwarp();
        for (int sb = s0; sb < s1; sb += 32) {
            // one stencil entry per lane: its j range and FP32 cell offset
            const int s = sb + lane;
            int st = 0, cn = 0;
            float4 D = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s < s1) {
                D = s_D[s];
                const int key = gbp_run_key(s_off[s], cx, cy, cz, a.n, a.pbc, keybase, a.bf3);
                if (key >= 0) {
                    st = a.start2[key];
                    cn = a.start2[key + __float_as_int(D.w)] - st;
                }
            }
            int incl = cn;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            const int T = __shfl_sync(FULL, incl, 31);
            // own-cell j-slots (auto mode, stencil entry 0): ordered pairs, i == j excluded
            const int selfT = (sb == 0 && a.nself) ? __shfl_sync(FULL, cn, 0) : 0;
            cand += (unsigned long long)icnt * (unsigned long long)T;
            // lane l stages j-slot f0 + l of each batch: the stencil entry k holding
            // it is the smallest k with incl[k] > f (5-step search over the lanes).
            // Where registers allow (PREF), the next batch's slot (its entry, sorted
            // index and position) is fetched before the current batch is tested and
            // binned, so the global load's latency overlaps that work; the other
            // modes fetch each batch's slot when they stage it.
            int jgN = -1;
            float4 pN = make_float4(0.f, 0.f, 0.f, 0.f), DN = pN;
            auto fetch = [&](int f) {
                int k = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(FULL, incl, k + step - 1);
                    if (v <= f) k += step;
                }
                k &= 31;
                const int stk = __shfl_sync(FULL, st, k);
                const int exk = __shfl_sync(FULL, incl - cn, k);
                DN = make_float4(__shfl_sync(FULL, D.x, k), __shfl_sync(FULL, D.y, k),
                                 __shfl_sync(FULL, D.z, k), 0.f);
                jgN = -1;
                if (f < T) {
                    jgN = stk + (f - exk);
                    pN = a.pos2[jgN];
                }
            };
            if (PREF && T > 0) fetch(lane);
            for (int f0 = 0; f0 < T; f0 += 32) {
                const int f = f0 + lane;
                if (!PREF) fetch(f);
                const int j = jgN;  // this batch's slot (-1: padding)
                const float4 p = pN;
                const float Dx = DN.x, Dy = DN.y, Dz = DN.z;
                if (PREF && f0 + 32 < T) fetch(f0 + 32 + lane);
                // this lane's j-slot in registers too (the transposed stage 1)
                float jtx = -GBP_FAR, jty = -GBP_FAR, jtz = -GBP_FAR;
                int jg = -1;  // the slot's sorted j index (-1: padding)
                if (f < T) {
                    jg = j;
                    const float tx = p.x + Dx, ty = p.y + Dy, tz = p.z + Dz;
                    jtx = tx; jty = ty; jtz = tz;
                    jx[lane] = tx; jy[lane] = ty; jz[lane] = tz; jix[lane] = __float_as_int(p.w);
                    jxy[lane] = make_ulonglong2(pk2(tx, tx), pk2(ty, ty));
                    jzz[lane] = pk2(tz, tz);
                    if (MW) {
                        if (WF == 0) {
                            for (int q = 0; q < nw; q++) jw64[lane * nw + q] = a.w64_2[(int64_t)j * nw + q];
                        } else {
                            jw[lane] = a.w2[j];
                        }
                    }
                    if (JACK || JACK2) jw[lane] = a.w2[j];
                } else {
                    // padding slot: at -FAR, so it is 2*FAR from an idle i-lane (+FAR)
                    // and farther still from every real point; its bits are also masked
                    jx[lane] = -GBP_FAR; jy[lane] = -GBP_FAR; jz[lane] = -GBP_FAR; jix[lane] = -2;
                    jxy[lane] = make_ulonglong2(pk2(-GBP_FAR, -GBP_FAR), pk2(-GBP_FAR, -GBP_FAR));
                    jzz[lane] = pk2(-GBP_FAR, -GBP_FAR);
                }
                if (COLS) {
                    // lanes over (slot, column): whole rows read, contiguous stores;
                    // a batch's read-only loads are all issued before its stores
                    for (int t0 = 0; t0 < 32 * ncol; t0 += 256) {
                        float v[8];
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            const int t = t0 + 32 * u + lane, r = col_row(t), q = t - r * ncol;
                            const int js = __shfl_sync(FULL, jg, r & 31);
                            v[u] = (t < 32 * ncol && js >= 0 && q < nw)
                                       ? __ldg(&a.w2[(int64_t)js * nw + q]) : 0.f;
                        }
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            if (t0 + 32 * u < 32 * ncol) jw[t0 + 32 * u + lane] = v[u];
                    }
                }
                __syncwarp();
                const int nj = min(32, T - f0);
                const int ns = min(max(selfT - f0, 0), nj);
                // stage 1: the sign bit of R - v is 1 exactly when the pair is out
                // of range; a funnel shift appends it to the lane's out-mask, so
                // slot jj lands in bit 31 - jj.  Items of at most 32 points take
                // the one-point loop, items of at most GBP_TRANSPOSE points the
                // transposed one.
                unsigned o0 = 0u, o1 = 0u;
                if (icnt <= GBP_TRANSPOSE) {
                    // few i-points: each lane tests its own j-slot against every
                    // i-point of the item, and a ballot hands i-point i (lane i) its
                    // in-range bits, slot jj at bit jj
                    const float4 tj = make_float4(jtx, jty, jtz, 0.f);
                    unsigned mine = 0u;
                    for (int i = 0; i < icnt; i++) {
                        const float4 ui = u4[i];
                        const unsigned in = __ballot_sync(FULL, (int)out_bits<MODE>(ui, tj, R0, R1) >= 0);
                        if (lane == i) mine = in;
                    }
                    o0 = __brev(~mine);
                    o1 = 0xffffffffu;
                } else if (icnt > 32) {
                    // both i-points in packed f32x2 arithmetic: v exactly as stage 2
                    // forms it, then R - v
#pragma unroll 8
                    for (int jj = 0; jj < 32; jj++) {
                        const ulonglong2 txy = jxy[jj];
                        const unsigned long long tzz = jzz[jj];
                        const unsigned long long dX = f2_sub(UX, txy.x), dY = f2_sub(UY, txy.y),
                                                 dZ = f2_sub(UZ, tzz);
                        unsigned long long d;
                        if (XYZF) {
                            d = f2_sub(RR0, f2_fma(dY, dY, f2_mul(dX, dX))) |
                                f2_sub(RR1, f2_mul(dZ, dZ));
                        } else {
                            d = f2_sub(RR0, f2_fma(dZ, dZ, f2_fma(dY, dY, f2_mul(dX, dX))));
                        }
                        o0 = __funnelshift_l((unsigned)d, o0, 1);
                        o1 = __funnelshift_l((unsigned)(d >> 32), o1, 1);
                    }
                } else {
#pragma unroll 8
                    for (int jj = 0; jj < 32; jj++) {
                        const ulonglong2 txy = jxy[jj];
                        const float4 t = make_float4(__uint_as_float((unsigned)txy.x),
                                                     __uint_as_float((unsigned)txy.y),
                                                     __uint_as_float((unsigned)jzz[jj]), 0.f);
                        o0 = __funnelshift_l(out_bits<MODE>(u0, t, R0, R1), o0, 1);
                    }
                    o1 = 0xffffffffu;
                }
                const unsigned valid = nj >= 32 ? 0xffffffffu : ((1u << nj) - 1u);
                unsigned m0 = __brev(~o0) & valid;
                unsigned m1 = __brev(~o1) & valid;
                if (ns > 0 && !MARKC) {
                    // own cell: (i, i) has separation exactly 0 and is handled apart
                    // (MARKC bins it like any pair: v = 0 exactly)
                    for (int jj = 0; jj < ns; jj++) {
                        const int jt = jix[jj];
                        if (jt == is0) {
                            m0 &= ~(1u << jj);
                            if (MARK && a.self_bin < nb0) {
                                const float ws = WF == 1 ? w0 * jw[jj] : WF == 2 ? w0 + jw[jj]
                                                 : (float)wfunc64(a.wfunc, wa, jw64 + jj * nw);
                                kahan_add(hs, hc, a.self_bin, ws);
                            }
                            if (MW2 && a.self_bin >= 0) {
                                const float ws = WF == 1 ? w0 * jw[jj] : WF == 2 ? w0 + jw[jj]
                                                 : (float)wfunc64(a.wfunc, wa, jw64 + jj * nw);
                                w2_add(wsink, a.self_bin, ws);
                            }
                            if (JW && a.self_bin >= 0) {
                                const int t = (int)jw[jj * 2 + 1];
                                sink_add<X_TAGW>(wsink, a.self_bin, 1, jw[jj * 2] * jw[jj * 2],
                                                 t | (t << 16));
                            }
                        }
                        if (jt == is1) {
                            m1 &= ~(1u << jj);
                            if (MARK && a.self_bin < nb0) {
                                const float ws = WF == 1 ? w1 * jw[jj] : WF == 2 ? w1 + jw[jj]
                                                 : (float)wfunc64(a.wfunc, wb, jw64 + jj * nw);
                                kahan_add(hs, hc, a.self_bin, ws);
                            }
                            if (MW2 && a.self_bin >= 0) {
                                const float ws = WF == 1 ? w1 * jw[jj] : WF == 2 ? w1 + jw[jj]
                                                 : (float)wfunc64(a.wfunc, wb, jw64 + jj * nw);
                                w2_add(wsink, a.self_bin, ws);
                            }
                            if (JW && a.self_bin >= 0) {
                                const int t = (int)jw[jj * 2 + 1];
                                sink_add<X_TAGW>(wsink, a.self_bin, 1, jw[jj * 2] * jw[jj * 2],
                                                 t | (t << 16));
                            }
                        }
                    }
                }
                // stage 2: the warp's in-range pairs are numbered lane by lane
                // (prefix sum of the bit counts), written as codes, then binned
                const unsigned own_bits = ns >= 32 ? 0xffffffffu : ((1u << ns) - 1u);
                const unsigned sym_bits = a.nself ? ~own_bits : 0u;
                // (marked modes bin the two i-points' codes in two phases: half the
                // code buffer, which keeps two CTAs per SM beside the Kahan columns)
                auto stage2 = [&](const unsigned mA, const unsigned mB) {
                    const int cl = __popc(mA) + __popc(mB);
                    int pre = cl;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int t = __shfl_up_sync(FULL, pre, o);
                        if (lane >= o) pre += t;
                    }
                    const int C = __shfl_sync(FULL, pre, 31);
                    pre -= cl;  // exclusive
                    // each lane writes a 16-bit code (i-slot, j-slot) per in-range pair
                    // at its prefix offset; the warp then bins 64 codes per round, two
                    // per lane, every lane busy
                    {
                        int k = pre;
                        unsigned m = mA;
                        while (m) {
                            const int jj = __ffs(m) - 1;
                            m &= m - 1u;
                            s_code[k++] = (unsigned short)(lane | (jj << 7));
                        }
                        m = mB;
                        while (m) {
                            const int jj = __ffs(m) - 1;
                            m &= m - 1u;
                            s_code[k++] = (unsigned short)((lane + 48) | (jj << 7));
                        }
                    }
                    __syncwarp();
                    auto entry = [&](int code) {
                        const int iu = code & 127, jj = code >> 7;
                        const float4 ui = u4[iu];
                        const float dx = ui.x - jx[jj], dy = ui.y - jy[jj], dz = ui.z - jz[jj];
                        float v0, v1 = 0.f, wt = 0.f;
                        if (XYZF) {
                            v0 = fmaf(dy, dy, dx * dx);
                            v1 = dz * dz;
                        } else if (SMUF) {
                            v1 = fmaf(dy, dy, dx * dx);
                            v0 = fmaf(dz, dz, v1);
                        } else {
                            v0 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                        }
                        if (MW) {
                            if (WF == 0) {
                                wt = (float)wfunc64(a.wfunc, s_uw64 + iu * nw, jw64 + jj * nw);
                            } else {
                                const float wi = s_uw[iu];
                                wt = WF == 1 ? wi * jw[jj] : wi + jw[jj];
                            }
                            if (MARK) v1 = wt;
                        }
                        // jackknife (rp, pi): both ends' tags (exact small integers)
                        if (JACK2) wt = __int_as_float((int)s_uw[iu] | ((int)jw[jj] << 16));
                        int tg = 0;
                        if (JW) {
                            wt = s_uw[iu * 2] * jw[jj * 2];
                            tg = (int)s_uw[iu * 2 + 1] | ((int)jw[jj * 2 + 1] << 16);
                        }
                        return PairV{v0, v1, iu, jj, ((sym_bits >> jj) & 1u) != 0u, wt, tg};
                    };
                    if (MARKC && !msort) {
                        // each lane bins one pair per round; then lane (g, c) adds channel
                        // c's product for pairs g, g + G, ... of the round to its own
                        // Kahan column, so no two lanes touch one column
                        const int G = 32 / nw, g = lane / nw, ch = lane - g * nw;
                        for (int r0 = 0; r0 < C; r0 += 32) {
                            const int sa = r0 + lane;
                            int b0 = nb0, b1 = nb0, mult = 1, iu = 0, jj = 0;
                            if (sa < C) {
                                const PairV e = entry(s_code[sa]);
                                iu = e.iu;
                                jj = e.jj;
                                mult = e.sym ? 2 : 1;
                                const float4 t = lut_entry_c<false>(e.v0, A0);
                                b0 = __float_as_int(t.x) + (e.v0 > t.y ? 1 : 0);
                                if ((e.v0 > t.z) & !(e.v0 > t.y)) {
                                    int k[2];
                                    const int n = slow_3d(e.v0, __float_as_int(t.x), ix.ui(iu),
                                                          ix.jw[jj], e.sym, k, A0, a);
                                    b0 = k[0];
                                    if (n == 2) {
                                        b1 = k[1];
                                        mult = 1;
                                    }
                                }
                            }
                            s_rec[lane] = make_int4(b0 | (mult << 16), b1, iu, jj);
                            __syncwarp();
                            const int np = min(32, C - r0);
                            for (int p = g; p < np; p += G) {
                                if (g >= G) break;
                                const int4 r = s_rec[p];
                                const float val = s_uw[r.z * ncol + ch] * jw[r.w * ncol + ch];
                                const int rb0 = r.x & 0xffff;
                                if (rb0 < nb0) kahan_add(hs, hc, rb0, (r.x >> 16) == 2 ? 2.0f * val : val);
                                if (r.y < nb0) kahan_add(hs, hc, r.y, val);
                            }
                            __syncwarp();
                        }
                    } else if (MARKC) {
                        // (1) each lane bins one code per round: its bin (nb0: none) to
                        // s_bin, the symmetric multiplicity into the code's bit 12, the
                        // bin's count up by the lanes that share it
                        const unsigned long long *W1 = (const unsigned long long *)s_uw;
                        const unsigned long long *W2 = (const unsigned long long *)jw;
                        for (int r0 = 0; r0 < C; r0 += 32) {
                            const int sa = r0 + lane;
                            int b0 = nb0, b1 = nb0;
                            unsigned code = 0u;
                            if (sa < C) {
                                code = s_code[sa];
                                const PairV e = entry((int)code);
                                bool two = e.sym;
                                const float4 t = lut_entry_c<false>(e.v0, A0);
                                b0 = __float_as_int(t.x) + (e.v0 > t.y ? 1 : 0);
                                if ((e.v0 > t.z) & !(e.v0 > t.y)) {
                                    int k[2];
                                    const int n = slow_3d(e.v0, __float_as_int(t.x), ix.ui(e.iu),
                                                          ix.jw[e.jj], e.sym, k, A0, a);
                                    b0 = k[0];
                                    if (n == 2) {
                                        b1 = min(k[1], nb0);
                                        two = false;
                                    }
                                }
                                b0 = min(b0, nb0);
                                s_bin[sa] = (unsigned char)b0;
                                s_code[sa] = (unsigned short)(code | (two ? 0x1000u : 0u));
                            }
                            // a pair whose two orders fall in different bins: its second
                            // bin right away, one channel pair per lane (rare)
                            unsigned split = __ballot_sync(FULL, b1 < nb0);
                            while (split) {
                                const int l = __ffs(split) - 1;
                                split &= split - 1u;
                                const int bl = __shfl_sync(FULL, b1, l);
                                const unsigned cl = __shfl_sync(FULL, code, l);
                                if (lane < mP) {
                                    const unsigned long long v = f2_mul(W1[(cl & 127u) * mP + lane],
                                                                        W2[((cl >> 7) & 31u) * mP + lane]);
                                    kahan_f2(hs2[bl * mP + lane], hc2[bl * mP + lane],
                                             pk2(1.f, 1.f), v);
                                }
                            }
                            const unsigned peers = __match_any_sync(FULL, b0);
                            if (b0 < nb0 && lane == __ffs(peers) - 1) s_cnt[b0] += __popc(peers);
                            __syncwarp();
                        }
                        // (2) each bin's first record (exclusive scan of the counts)
                        unsigned nz[2] = {0u, 0u};  // bins holding records, 32 per word
                        {
                            int run = 0;
                            for (int bs = 0; bs < nb0; bs += 32) {
                                const int b = bs + lane;
                                const int c = b < nb0 ? s_cnt[b] : 0;
                                int incl = c;
#pragma unroll
                                for (int o = 1; o < 32; o <<= 1) {
                                    const int t = __shfl_up_sync(FULL, incl, o);
                                    if (lane >= o) incl += t;
                                }
                                if (b < nb0) s_cur[b] = run + incl - c;
                                run += __shfl_sync(FULL, incl, 31);
                                nz[bs >> 5] = __ballot_sync(FULL, c > 0);
                            }
                        }
                        __syncwarp();
                        // (3) the codes scattered by bin, in code order within a bin;
                        // s_cur[b] ends at the bin's end
                        for (int r0 = 0; r0 < C; r0 += 32) {
                            const int sa = r0 + lane;
                            const int b = sa < C ? (int)s_bin[sa] : nb0;
                            const unsigned peers = __match_any_sync(FULL, b);
                            const int rank = __popc(peers & ((1u << lane) - 1u));
                            const int base = b < nb0 ? s_cur[b] : 0;
                            __syncwarp();
                            if (b < nb0) {
                                s_rec2[base + rank] = s_code[sa];
                                if (rank == 0) s_cur[b] = base + __popc(peers);
                            }
                            __syncwarp();
                        }
                        // (4) per bin, lane (g, cp) sums the products of channel pair cp
                        // over records g, g + G, ...: runs of 8 in packed FP32, the runs
                        // compensated in registers, the G groups' totals by a shuffle
                        // tree, then one compensated add to the warp's (bin, pair) sums
                        const int G = 32 / mP, g = lane / mP, cp = lane - g * mP;
                        const unsigned long long ONE2 = pk2(1.f, 1.f);
                        for (int w = 0; w < 2; w++) {
                            unsigned bits = nz[w];
                            while (bits) {
                                const int b = 32 * w + __ffs(bits) - 1;
                                bits &= bits - 1u;
                                const int end = s_cur[b], st = end - s_cnt[b];
                                unsigned long long S = 0ull, NC = 0ull;
                                for (int p = st + g; p < end; p += 8 * G) {
                                    // this group's records of the run: as many
                                    // iterations as records, at most 8
                                    const int nk = min(8, (end - p + G - 1) / G);
                                    unsigned long long r = 0ull;
                                    for (int k = 0; k < nk; k++) {
                                        const unsigned rec = s_rec2[p + k * G];
                                        unsigned long long v = f2_mul(W1[(rec & 127u) * mP + cp],
                                                                      W2[((rec >> 7) & 31u) * mP + cp]);
                                        if (rec & 0x1000u) v = f2_add(v, v);
                                        r = f2_add(r, v);
                                    }
                                    kahan_f2(S, NC, ONE2, r);
                                }
                                unsigned long long v = f2_add(S, NC);
                                for (int o = 16; o >= mP; o >>= 1)
                                    v = f2_add(v, __shfl_xor_sync(FULL, v, o));
                                if (g == 0) kahan_f2(hs2[b * mP + cp], hc2[b * mP + cp], ONE2, v);
                            }
                        }
                        __syncwarp();
                        for (int b = lane; b < nb0; b += 32) s_cnt[b] = 0;
                        __syncwarp();
                    } else {
                        // lanes in GR regions of WL: lane (g, o) bins codes
                        // g * R / GR + t * WL + o at steps t (R = C rounded up to 32), so
                        // one instruction's lanes hold pairs of GR distant i-points
                        // (GR = 1: 32 consecutive codes).  The weighted 2-D sums add into
                        // the CTA's shared (hi, lo) pairs, where lanes of one i-point
                        // (same direction, so often the same bin) serialise: spread out,
                        // weighted (s, mu') took 65.7 -> 63.2 ms and weighted (rp, pi)
                        // 67.5 -> 66.4 ms on 10M points.  The plain counts lose (the
                        // 10M (s, mu') count 30.1 -> 30.9-31.3 ms at 2-32 regions): there
                        // one i-point's table and position loads are broadcasts.
                        constexpr int GR = MODE == MODE_SMUW ? 32 : MODE == MODE_XYZW ? 4 : 1;
                        constexpr int WL = 32 / GR;
                        const int rend = GR == 1 ? C : ((C + 31) & ~31);
                        const int rbase = GR == 1 ? lane : (lane / WL) * (rend / GR) + (lane % WL);
                        for (int r0 = 0; r0 < rend; r0 += 64) {
                            const int sa = rbase + r0 / GR, sb = sa + WL;
                            const bool ha = sa < C, hb = (GR == 1 || r0 + 32 < rend) && sb < C;
                            const PairV ea = entry(ha ? s_code[sa] : 0);
                            const PairV eb = entry(hb ? s_code[sb] : 0);
                            if (MODE == MODE_3D) {
                                // both pairs' table lookups first (independent chains
                                // the scheduler can overlap), then the updates
                                const int qa = lut_slot(ea.v0, A0), qb = lut_slot(eb.v0, A0);
                                const unsigned wa = s_l0[qa], wb = s_l0[qb];
                                const float2 pa = s_t0[qa], pb = s_t0[qb];
                                const float4 ta = make_float4(__int_as_float((int)(wa & 0xffffu)), pa.x, pa.y, 0.f);
                                const float4 tb = make_float4(__int_as_float((int)(wb & 0xffffu)), pb.x, pb.y, 0.f);
                                const bool sla = (ea.v0 > ta.z) & !(ea.v0 > ta.y);
                                const bool slb = (eb.v0 > tb.z) & !(eb.v0 > tb.y);
                                const int ba = __float_as_int(ta.x) + (ea.v0 > ta.y ? 1 : 0);
                                const int bb = __float_as_int(tb.x) + (eb.v0 > tb.y ? 1 : 0);
                                if (ha) {
                                    if (sla) bin_3d<true>(ea, hl, A0, ix, a);
                                    else hl[ba * 32] += ea.sym ? 2u : 1u;
                                }
                                if (hb) {
                                    if (slb) bin_3d<true>(eb, hl, A0, ix, a);
                                    else hl[bb * 32] += eb.sym ? 2u : 1u;
                                }
                            } else if (XYZF) {
                                const float4 a0 = lut_entry_c<false>(ea.v0, A0);
                                const float4 a1 = lut_entry_c<false>(ea.v1, A1);
                                const float4 b0 = lut_entry_c<false>(eb.v0, A0);
                                const float4 b1 = lut_entry_c<false>(eb.v1, A1);
                                const bool sla = ((ea.v0 > a0.z) & !(ea.v0 > a0.y)) |
                                                 ((ea.v1 > a1.z) & !(ea.v1 > a1.y));
                                const bool slb = ((eb.v0 > b0.z) & !(eb.v0 > b0.y)) |
                                                 ((eb.v1 > b1.z) & !(eb.v1 > b1.y));
                                const int ka = __float_as_int(a0.x) + (ea.v0 > a0.y ? 1 : 0);
                                const int ga = __float_as_int(a1.x) + (ea.v1 > a1.y ? 1 : 0);
                                const int kb = __float_as_int(b0.x) + (eb.v0 > b0.y ? 1 : 0);
                                const int gb = __float_as_int(b1.x) + (eb.v1 > b1.y ? 1 : 0);
                                if (ha) {
                                    if (sla) bin_entry(ea, cur_mock);
                                    else if ((ka < nb0) & (ga < nb1)) {
                                        if (CNT2) {
                                            if (copies) atomicAdd(&wh[ka * stride2 + ga], ea.sym ? 2u : 1u);
                                            else atomicAdd(&a.hist[(size_t)cur_mock * a.hist_stride +
                                                                   ka * stride2 + ga],
                                                           ea.sym ? 2ull : 1ull);
                                        }
                                        sink_add<XS>(wsink, ka * stride2 + ga, ea.sym ? 2 : 1, ea.w, ea.tg);
                                    }
                                }
                                if (hb) {
                                    if (slb) bin_entry(eb, cur_mock);
                                    else if ((kb < nb0) & (gb < nb1)) {
                                        if (CNT2) {
                                            if (copies) atomicAdd(&wh[kb * stride2 + gb], eb.sym ? 2u : 1u);
                                            else atomicAdd(&a.hist[(size_t)cur_mock * a.hist_stride +
                                                                   kb * stride2 + gb],
                                                           eb.sym ? 2ull : 1ull);
                                        }
                                        sink_add<XS>(wsink, kb * stride2 + gb, eb.sym ? 2 : 1, eb.w, eb.tg);
                                    }
                                }
                            } else if (MARK) {
                                const float4 ta = lut_entry_c<false>(ea.v0, A0);
                                const float4 tb = lut_entry_c<false>(eb.v0, A0);
                                const bool sla = (ea.v0 > ta.z) & !(ea.v0 > ta.y);
                                const bool slb = (eb.v0 > tb.z) & !(eb.v0 > tb.y);
                                const int ba = __float_as_int(ta.x) + (ea.v0 > ta.y ? 1 : 0);
                                const int bb = __float_as_int(tb.x) + (eb.v0 > tb.y ? 1 : 0);
                                if (ha) {
                                    if (sla) bin_entry(ea, cur_mock);
                                    else if (ba < nb0) kahan_add(hs, hc, ba, ea.sym ? 2.0f * ea.v1 : ea.v1);
                                }
                                if (hb) {
                                    if (slb) bin_entry(eb, cur_mock);
                                    else if (bb < nb0) kahan_add(hs, hc, bb, eb.sym ? 2.0f * eb.v1 : eb.v1);
                                }
                            } else if (SMUF && copies) {
                                // s slots and q = dxy / s^2 of both pairs, then their mu'
                                // slots and the neighbouring edges, then the updates
                                const float4 sa4 = lut_entry_c<true>(ea.v0, A0);
                                const float4 sb4 = lut_entry_c<true>(eb.v0, A0);
                                const float qa = __fdividef(ea.v1, ea.v0), qb = __fdividef(eb.v1, eb.v0);
                                const QBin qa4 = lut_q(qa, A1), qb4 = lut_q(qb, A1);
                                const int bsa = __float_as_int(sa4.x) + (ea.v0 > sa4.y ? 1 : 0);
                                const int bsb = __float_as_int(sb4.x) + (eb.v0 > sb4.y ? 1 : 0);
                                const int bqa = qa4.b, bqb = qb4.b;
                                const bool amba = ((ea.v0 > sa4.z) & !(ea.v0 > sa4.y)) |
                                                  !(qa - qa4.below > sa4.w) |
                                                  !(qa4.above - qa > sa4.w) | qa4.walk;
                                const bool ambb = ((eb.v0 > sb4.z) & !(eb.v0 > sb4.y)) |
                                                  !(qb - qb4.below > sb4.w) |
                                                  !(qb4.above - qb > sb4.w) | qb4.walk;
                                // (as bin_smu: past the s gate first, then the guard bands)
                                if (ha && bsa < nb0) {
                                    if (amba) bin_entry(ea, cur_mock);
                                    else if (bqa < nb1) {
                                        atomicAdd(&wh[bsa * stride2 + bqa], ea.sym ? 2u : 1u);
                                        sink_add<XS>(wsink, bsa * stride2 + bqa, ea.sym ? 2 : 1, ea.w);
                                    }
                                }
                                if (hb && bsb < nb0) {
                                    if (ambb) bin_entry(eb, cur_mock);
                                    else if (bqb < nb1) {
                                        atomicAdd(&wh[bsb * stride2 + bqb], eb.sym ? 2u : 1u);
                                        sink_add<XS>(wsink, bsb * stride2 + bqb, eb.sym ? 2 : 1, eb.w);
                                    }
                                }
                            } else {
                                if (ha) bin_entry(ea, cur_mock);
                                if (hb) bin_entry(eb, cur_mock);
                            }
                        }
                        if (RQM) rq_drain(cur_mock, 32u);
                        if (W2) {
                            w2_binned += (unsigned)C;
                            if (w2_binned >= GBP_W2_FLUSH) w2_move();
                        }
                    }
                    __syncwarp();
                };
                if (MARK || (MARKC && (!msort || GBP_MARKC_CODES < 2048))) {
                    stage2(m0, 0u);
                    stage2(0u, m1);
                } else {
                    stage2(m0, m1);
                }
                drained += 64;
                __syncwarp();
            }
        }
        // a lane adds at most 2 per pair of its own and a warp copy at most 64
        // per lane: flush long before a u32 could wrap
        if (!MARK && !MARKC && drained > a.flush_after) warp_flush(cur_mock);
    }
    if (cur_mock >= 0) warp_flush(cur_mock);
    if (lane == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
    if (W2) {
        // every warp has left the item loop (one mock per call): the CTA's totals
        __syncthreads();
        for (int b = tid; b < nbin; b += GBP_BLOCK) {
            const double v = s_wacc[b] + (double)s_whi[b] + (double)s_wlo[b];
            if (v != 0.0) atomicAdd(&a.histd[b], v);
        }
    }
    if (JACK) {
        // every warp has left the item loop: add the CTA's table to the global one
        __syncthreads();
        for (int i = tid; i < a.ntag * (nb0 + 1); i += GBP_BLOCK)
            if (s_tab[i]) atomicAdd(&a.htag[i], s_tab[i]);
    }
}

template <int MODE, int WF>
static cudaError_t launch_t(const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_count<MODE, WF>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_count<MODE, WF><<<grid, GBP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

template <int MODE, int WF>
static int occ_t(size_t smem) {
    int nblk = 0;
    if (cudaFuncSetAttribute(k_count<MODE, WF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_count<MODE, WF>, GBP_BLOCK, smem) !=
        cudaSuccess)
        return 0;
    return nblk;
}

cudaError_t gbp_launch_count(int mode, int wf, const CountArgs &a, int grid, size_t smem,
                             cudaStream_t st) {
    switch (mode) {
    case MODE_3D: return launch_t<MODE_3D, 1>(a, grid, smem, st);
    case MODE_3DS: return launch_t<MODE_3DS, 1>(a, grid, smem, st);
    case MODE_XYZ: return launch_t<MODE_XYZ, 1>(a, grid, smem, st);
    case MODE_SMU: return launch_t<MODE_SMU, 1>(a, grid, smem, st);
    case MODE_MARKC:
        return launch_t<MODE_MARKC, 1>(a, grid, smem, st);
    case MODE_JACK:
        return launch_t<MODE_JACK, 1>(a, grid, smem, st);
    case MODE_SMUW:
        return launch_t<MODE_SMUW, 1>(a, grid, smem, st);
    case MODE_JACKXYZ:
        return launch_t<MODE_JACKXYZ, 1>(a, grid, smem, st);
    case MODE_JACKW:
        return launch_t<MODE_JACKW, 1>(a, grid, smem, st);
    case MODE_JACKXYZW:
        return launch_t<MODE_JACKXYZW, 1>(a, grid, smem, st);
    case MODE_XYZW:
        if (wf == 1) return launch_t<MODE_XYZW, 1>(a, grid, smem, st);
        if (wf == 2) return launch_t<MODE_XYZW, 2>(a, grid, smem, st);
        return launch_t<MODE_XYZW, 0>(a, grid, smem, st);
    case MODE_MARK:
        if (wf == 1) return launch_t<MODE_MARK, 1>(a, grid, smem, st);
        if (wf == 2) return launch_t<MODE_MARK, 2>(a, grid, smem, st);
        return launch_t<MODE_MARK, 0>(a, grid, smem, st);
    default: return cudaErrorInvalidValue;
    }
}

int gbp_count_occupancy(int mode, int wf, size_t smem) {
    switch (mode) {
    case MODE_3D: return occ_t<MODE_3D, 1>(smem);
    case MODE_3DS: return occ_t<MODE_3DS, 1>(smem);
    case MODE_XYZ: return occ_t<MODE_XYZ, 1>(smem);
    case MODE_SMU: return occ_t<MODE_SMU, 1>(smem);
    case MODE_MARKC:
        return occ_t<MODE_MARKC, 1>(smem);
    case MODE_JACK:
        return occ_t<MODE_JACK, 1>(smem);
    case MODE_SMUW:
        return occ_t<MODE_SMUW, 1>(smem);
    case MODE_JACKXYZ:
        return occ_t<MODE_JACKXYZ, 1>(smem);
    case MODE_JACKW:
        return occ_t<MODE_JACKW, 1>(smem);
    case MODE_JACKXYZW:
        return occ_t<MODE_JACKXYZW, 1>(smem);
    case MODE_XYZW:
        if (wf == 1) return occ_t<MODE_XYZW, 1>(smem);
        if (wf == 2) return occ_t<MODE_XYZW, 2>(smem);
        return occ_t<MODE_XYZW, 0>(smem);
    case MODE_MARK:
        if (wf == 1) return occ_t<MODE_MARK, 1>(smem);
        if (wf == 2) return occ_t<MODE_MARK, 2>(smem);
        return occ_t<MODE_MARK, 0>(smem);
    default: return 0;
    }
}
