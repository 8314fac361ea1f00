// Device helpers shared by the count and adjoint kernels: float-bit table
// lookup of a bin, the per-edge walk, and the reference's exact FP64 pair
// arithmetic used for the guard-band recheck.
#pragma once
#include "gbp_internal.cuh"

struct AxisSm {
    const float4 *lut;      // adjoint: {b0, thr, lo, qband} per slot
    const float *hi;
    const float *lo;
    const double *E;
    int nb, S, B;
    float vlo, vhi;
    const unsigned *l32;    // count kernels: b0 | (threshold-pair index << 16) per slot;
                            // s of (s, mu'): pairs {that word, the slot's q error bound}
    const float2 *hl;       // threshold pairs (thr, lo): nb edges, the top, the always-walk pair
    const float4 *hq;       // q of (s, mu'): {thr, lo, hi of the edge below, lo of the edge above}
};

__device__ __forceinline__ int lut_slot(float v, const AxisSm &a) {
    float vc = fminf(fmaxf(v, a.vlo), a.vhi);
    return (int)(__float_as_uint(vc) >> a.S) - a.B;
}

__device__ __forceinline__ float4 lut_entry(float v, const AxisSm &a) {
    return a.lut[lut_slot(v, a)];
}

// The same entry from the compact tables: a 4-byte slot word and a shared
// threshold pair (few distinct addresses, so few bank conflicts).
// QB: the s table of (s, mu'), whose slot words sit beside the q error bounds.
template <bool QB>
__device__ __forceinline__ float4 lut_entry_c(float v, const AxisSm &a) {
    const int s = lut_slot(v, a);
    unsigned w;
    float qb = 0.f;
    if (QB) {
        const uint2 e = ((const uint2 *)a.l32)[s];
        w = e.x;
        qb = __uint_as_float(e.y);
    } else {
        w = a.l32[s];
    }
    const float2 t = a.hl[w >> 16];
    return make_float4(__int_as_float((int)(w & 0xffffu)), t.x, t.y, qb);
}

// The q axis of (s, mu'): q's bin, the guard values that q must keep clear of
// (the upper guard of its bin's lower edge, the lower guard of its upper edge;
// -3e38 / 3e38 where the bin has none), and whether its slot holds several edges.
struct QBin {
    int b;
    float below, above;
    bool walk;
};
__device__ __forceinline__ QBin lut_q(float q, const AxisSm &Q) {
    const unsigned w = Q.l32[lut_slot(q, Q)];
    const float4 t = Q.hq[w >> 16];
    const bool up = q > t.x;
    return QBin{(int)(w & 0xffffu) + (up ? 1 : 0), up ? t.x : t.z, up ? t.w : t.y,
                t.y < -3.0e38f};
}

// Build the compact tables in shared memory from the float4 table.  With qb
// the slot words are written as pairs {word, q error bound} (the s table of
// (s, mu')); with hq the threshold table is the q table's float4 form.
__device__ __forceinline__ void lut_compact(const float4 *lut, int T, const float *hi,
                                            const float *lo, int nb, unsigned *l32, float2 *hl,
                                            bool qb, float4 *hq, int tid, int nthr) {
    for (int s = tid; s < T; s += nthr) {
        const float4 e = lut[s];
        const int b0 = __float_as_int(e.x);
        // simple slot: (hi[b0], lo[b0]); top: (inf, inf) at nb; always-walk: (inf, -inf) at nb + 1
        const unsigned h = (b0 < nb && e.z == -INFINITY) ? nb + 1 : b0;
        const unsigned word = (unsigned)b0 | (h << 16);
        if (qb) ((uint2 *)l32)[s] = make_uint2(word, __float_as_uint(e.w));
        else l32[s] = word;
    }
    if (hq) {
        for (int k = tid; k < nb; k += nthr)
            hq[k] = make_float4(hi[k], lo[k], k > 0 ? hi[k - 1] : -3.0e38f,
                                k + 1 < nb ? lo[k + 1] : 3.0e38f);
        if (tid == 0) {
            hq[nb] = make_float4(INFINITY, 3.0e38f, nb > 0 ? hi[nb - 1] : -3.0e38f, 3.0e38f);
            hq[nb + 1] = make_float4(INFINITY, -INFINITY, -3.0e38f, 3.0e38f);
        }
        return;
    }
    for (int k = tid; k < nb; k += nthr) hl[k] = make_float2(hi[k], lo[k]);
    if (tid == 0) {
        hl[nb] = make_float2(INFINITY, INFINITY);
        hl[nb + 1] = make_float2(INFINITY, -INFINITY);
    }
}

// Walk from the table's start bin with the per-edge thresholds.  Returns the
// bin if the FP32 value decides it, or -1 - k if it is ambiguous at edge k.
__device__ __forceinline__ int walk_bin(float v, int b0, const AxisSm &a) {
    int k = b0;
    while (k < a.nb && v > a.hi[k]) k++;
    if (k < a.nb && v > a.lo[k]) return -1 - k;
    return k;
}

__device__ __forceinline__ int exact_bin(double v, int b0, const AxisSm &a) {
    int k = b0;
    while (k < a.nb && !(v <= a.E[k])) k++;
    return k;
}

// halotools' shift: x1tmp = x1 - x2shift, dx = x1tmp - x2 with x2shift in
// {-L, 0, +L}; for a pair inside the search range exactly one shift gives
// |dx| <= L/3, which is the one the reference's stencil visit applies.
__device__ __forceinline__ double ref_delta(double a, double b, double L, int pbc) {
    double d0 = __dsub_rn(a, b);
    if (!pbc) return d0;
    double dp = __dsub_rn(__dsub_rn(a, L), b);
    double dm = __dsub_rn(__dadd_rn(a, L), b);
    double best = d0;
    if (fabs(dp) < fabs(best)) best = dp;
    if (fabs(dm) < fabs(best)) best = dm;
    return best;
}

// FP64 position of sorted point `sorted` of sample `side` (0: sample 1), read
// from the caller's array, float32 rows upcast exactly.
__device__ __forceinline__ void ref_pos(const CountArgs &a, int side, int sorted, double p[3]) {
    const int64_t r = 3 * (int64_t)(side ? a.orig2[sorted] : a.orig1[sorted]);
    const void *x = side ? a.xyz2 : a.xyz1;
    if (side ? a.xyz2_f32 : a.xyz1_f32) {
        const float *f = (const float *)x + r;
        p[0] = (double)f[0];
        p[1] = (double)f[1];
        p[2] = (double)f[2];
    } else {
        const double *d = (const double *)x + r;
        p[0] = d[0];
        p[1] = d[1];
        p[2] = d[2];
    }
}

struct Exact3 {
    double dxy, dz2, s2;
};

__device__ __forceinline__ Exact3 exact_pair(const double *p, const double *q, const CountArgs &a) {
    double dx = ref_delta(p[0], q[0], a.L[0], a.pbc);
    double dy = ref_delta(p[1], q[1], a.L[1], a.pbc);
    double dz = ref_delta(p[2], q[2], a.L[2], a.pbc);
    Exact3 r;
    r.dxy = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    r.dz2 = __dmul_rn(dz, dz);
    r.s2 = __dadd_rn(r.dxy, r.dz2);
    return r;
}

// Packed FP32 pairs (low word = element 0).  sub/mul/fma.rn.f32x2 round each
// element exactly as the scalar FSUB/FMUL/FFMA do.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
    return ((unsigned long long)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Compensated (Kahan) add of the packed pair w * g to the packed sums s, with the
// compensation kept negated (nc = -c): y = w g - c, t = s + y, c = (t - s) - y,
// each element rounded as the scalar sum would be.
__device__ __forceinline__ void kahan_f2(unsigned long long &s, unsigned long long &nc,
                                         unsigned long long w, unsigned long long g) {
    const unsigned long long y = f2_fma(w, g, nc), t = f2_add(s, y);
    nc = f2_sub(y, f2_sub(t, s));
    s = t;
}

