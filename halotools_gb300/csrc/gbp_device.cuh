// Device helpers shared by the count and adjoint kernels: float-bit table
// lookup of a bin, the per-edge walk, and the reference's exact FP64 pair
// arithmetic used for the guard-band recheck.
#pragma once
#include "gbp_internal.cuh"

struct AxisSm {
    const float4 *lut;
    const float *hi;
    const float *lo;
    const double *E;
    int nb, S, B;
    float vlo, vhi;
};

__device__ __forceinline__ float4 lut_entry(float v, const AxisSm &a) {
    float vc = fminf(fmaxf(v, a.vlo), a.vhi);
    int idx = (int)(__float_as_uint(vc) >> a.S) - a.B;
    return a.lut[idx];
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

