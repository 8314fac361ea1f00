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
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *q = a.x64_2 + 3 * (int64_t)js;
    k[0] = exact_bin(exact_pair(p, q, a).s2, b0, A);
    if (!sym) return 1;
    k[1] = exact_bin(exact_pair(q, p, a).s2, b0, A);
    return 2;
}

template <bool LANE>
__device__ __forceinline__ void bin_3d(const float4 &e, unsigned *h, const AxisSm &A,
                                       const CountArgs &a) {
    const float v = e.x;
    const unsigned jw = __float_as_uint(e.w);
    const bool sym = jw & SYM_BIT;
    const unsigned w = sym ? 2u : 1u;
    float4 t = lut_entry(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        int n = slow_3d(v, __float_as_int(t.x), __float_as_int(e.z), (int)(jw & ~SYM_BIT), sym, k,
                        A, a);
        if (n == 0) {
            b = k[0];
        } else {
            for (int q = 0; q < n; q++) {
                if (LANE) h[k[q] * 32] += 1u;
                else if (k[q] < A.nb) atomicAdd(&h[k[q]], 1u);
            }
            return;
        }
    }
    if (LANE) h[b * 32] += w;
    else if (b < A.nb) atomicAdd(&h[b], w);
}

// ---------------- stage 2: marked (Kahan in lane-private FP32 pairs) ----------------
__device__ __forceinline__ void kahan_add(float *hs, float *hc, int b, float x) {
    float s = hs[b * 32], c = hc[b * 32];
    float y = x - c;
    float t = s + y;
    hc[b * 32] = (t - s) - y;
    hs[b * 32] = t;
}

__device__ __forceinline__ void bin_mark(const float4 &e, float *hs, float *hc, const AxisSm &A,
                                         const CountArgs &a) {
    const float v = e.x, wt = e.y;
    const unsigned jw = __float_as_uint(e.w);
    const bool sym = jw & SYM_BIT;
    float4 t = lut_entry(v, A);
    int b = __float_as_int(t.x) + (v > t.y ? 1 : 0);
    if ((v > t.z) & !(v > t.y)) {
        int k[2];
        int n = slow_3d(v, __float_as_int(t.x), __float_as_int(e.z), (int)(jw & ~SYM_BIT), sym, k,
                        A, a);
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

// ---------------- stage 2: (rp, pi) ----------------
__device__ __noinline__ void slow_xyz(float v0, float v1, int b0a, int b0b, int is, int js,
                                      bool sym, unsigned *hw, int stride, const AxisSm &A,
                                      const AxisSm &Bx, const CountArgs &a) {
    int ka = walk_bin(v0, b0a, A);
    int kb = walk_bin(v1, b0b, Bx);
    if (ka >= 0 && kb >= 0) {
        if (ka < A.nb && kb < Bx.nb) atomicAdd(&hw[ka * stride + kb], sym ? 2u : 1u);
        return;
    }
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *q = a.x64_2 + 3 * (int64_t)js;
    Exact3 r = exact_pair(p, q, a);
    int ea = ka >= 0 ? ka : exact_bin(r.dxy, b0a, A);
    int eb = kb >= 0 ? kb : exact_bin(r.dz2, b0b, Bx);
    if (ea < A.nb && eb < Bx.nb) atomicAdd(&hw[ea * stride + eb], 1u);
    if (!sym) return;
    Exact3 s = exact_pair(q, p, a);
    int fa = ka >= 0 ? ka : exact_bin(s.dxy, b0a, A);
    int fb = kb >= 0 ? kb : exact_bin(s.dz2, b0b, Bx);
    if (fa < A.nb && fb < Bx.nb) atomicAdd(&hw[fa * stride + fb], 1u);
}

__device__ __forceinline__ void bin_xyz(const float4 &e, unsigned *hw, int stride, const AxisSm &A,
                                        const AxisSm &Bx, const CountArgs &a) {
    const float v0 = e.x, v1 = e.y;
    const unsigned jw = __float_as_uint(e.w);
    const bool sym = jw & SYM_BIT;
    float4 e0 = lut_entry(v0, A);
    float4 e1 = lut_entry(v1, Bx);
    int ba = __float_as_int(e0.x) + (v0 > e0.y ? 1 : 0);
    int bb = __float_as_int(e1.x) + (v1 > e1.y ? 1 : 0);
    bool amb = ((v0 > e0.z) & !(v0 > e0.y)) | ((v1 > e1.z) & !(v1 > e1.y));
    if (amb) {
        slow_xyz(v0, v1, __float_as_int(e0.x), __float_as_int(e1.x), __float_as_int(e.z),
                 (int)(jw & ~SYM_BIT), sym, hw, stride, A, Bx, a);
        return;
    }
    if ((ba < A.nb) & (bb < Bx.nb)) atomicAdd(&hw[ba * stride + bb], sym ? 2u : 1u);
}

// ---------------- stage 2: (s, mu') ----------------
// v = s^2 on axis 0; q = dxy / s^2 on axis 1, whose FP32 error depends on s:
// the s table's 4th field holds the q error bound for the slot's smallest s.
__device__ __noinline__ void slow_smu(float v, float q, float qb, int b0s, int is, int js,
                                      bool sym, unsigned *hw, int stride, const AxisSm &A,
                                      const AxisSm &Q, const CountArgs &a) {
    int ks = walk_bin(v, b0s, A);
    int kq = -1;
    if (ks >= 0 && ks < A.nb && v > 0.0f) {
        int g = 0;
        while (g < Q.nb && q > Q.hi[g] + qb) g++;
        if (!(g < Q.nb && q > Q.lo[g] - qb)) kq = g;
    }
    if (ks >= A.nb) return;  // beyond the s gate: never counted
    if (ks >= 0 && kq >= 0) {
        if (kq < Q.nb) atomicAdd(&hw[ks * stride + kq], sym ? 2u : 1u);
        return;
    }
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *qq = a.x64_2 + 3 * (int64_t)js;
    for (int o = 0; o < (sym ? 2 : 1); o++) {
        Exact3 r = o == 0 ? exact_pair(p, qq, a) : exact_pair(qq, p, a);
        int es = exact_bin(r.s2, 0, A);
        if (es >= A.nb) continue;
        double mu2 = (r.s2 > 0.0) ? __ddiv_rn(r.dxy, r.s2) : 0.0;
        int eq = exact_bin(mu2, 0, Q);
        if (eq >= Q.nb) continue;
        atomicAdd(&hw[es * stride + eq], 1u);
    }
}

__device__ __forceinline__ void bin_smu(const float4 &e, unsigned *hw, int stride, const AxisSm &A,
                                        const AxisSm &Q, const CountArgs &a) {
    const float v = e.x, dxy = e.y;
    const unsigned jw = __float_as_uint(e.w);
    const bool sym = jw & SYM_BIT;
    float4 e0 = lut_entry(v, A);
    int bs = __float_as_int(e0.x) + (v > e0.y ? 1 : 0);
    if (bs >= A.nb) return;  // beyond the s gate
    float q = __fdividef(dxy, v);
    float qb = e0.w;
    float4 e1 = lut_entry(q, Q);
    int bq = __float_as_int(e1.x) + (q > e1.y ? 1 : 0);
    // nearest edges around q must be farther than qb
    float below = bq > 0 ? Q.hi[bq - 1] : -3.0e38f;
    float above = bq < Q.nb ? Q.lo[bq] : 3.0e38f;
    bool amb = ((v > e0.z) & !(v > e0.y)) | !(q - below > qb) | !(above - q > qb) |
               (e1.y > 3.0e38f);
    if (amb) {
        slow_smu(v, q, qb, __float_as_int(e0.x), __float_as_int(e.z), (int)(jw & ~SYM_BIT), sym,
                 hw, stride, A, Q, a);
        return;
    }
    if (bq < Q.nb) atomicAdd(&hw[bs * stride + bq], sym ? 2u : 1u);
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

// ---------------- kernel ----------------
template <int MODE, int WF>
__global__ void __launch_bounds__(GBP_BLOCK, 3) k_count(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr bool TWO = (MODE == MODE_XYZ || MODE == MODE_SMU);
    constexpr bool MARK = (MODE == MODE_MARK);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, nb1 = TWO ? a.ax[1].nb : 0;
    const int T0 = a.ax[0].T, T1 = TWO ? a.ax[1].T : 0;
    const int copies = a.hist_copies;
    const int nw = MARK ? a.nw : 0;
    const int jwb = MARK ? (WF == 0 ? 8 * nw : 4) : 0;
    const SmemLayout L = gbp_smem_layout(MODE, T0, T1, nb0, nb1, a.nsten, copies, jwb);
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    float4 *s_lut1 = (float4 *)(smem + L.off_lut1);
    float4 *s_j = (float4 *)(smem + L.off_j);
    float *s_jw = (float *)(smem + L.off_jw);
    double *s_jw64 = (double *)(smem + L.off_jw);
    float4 *s_q = (float4 *)(smem + L.off_q) + warp * GBP_QCAP;
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    double *s_E1 = (double *)(smem + L.off_E1);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    float *s_hi1 = (float *)(smem + L.off_hi1);
    float *s_lo1 = (float *)(smem + L.off_lo1);
    int *s_off = (int *)(smem + L.off_off);
    int *s_cstart = (int *)(smem + L.off_cstart);
    int *s_pre = (int *)(smem + L.off_pre);
    unsigned *s_hist = (unsigned *)(smem + L.off_hist);
    __shared__ int s_item;
    __shared__ int s_nitems;

    for (int i = tid; i < T0; i += GBP_BLOCK) s_lut0[i] = a.ax[0].lut[i];
    for (int i = tid; i < T1; i += GBP_BLOCK) s_lut1[i] = a.ax[1].lut[i];
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
    const int hist_words = (MODE == MODE_3D) ? GBP_WARPS * (nb0 + 1) * 32
                         : MARK ? GBP_WARPS * (nb0 + 1) * 32 * 2 : copies * nbin;
    for (int i = tid; i < hist_words; i += GBP_BLOCK) s_hist[i] = 0u;
    if (tid == 0) s_nitems = *a.nitems;

    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    AxisSm A1{s_lut1, s_hi1, s_lo1, s_E1, nb1, TWO ? a.ax[1].S : 0, TWO ? a.ax[1].B : 0,
              TWO ? a.ax[1].vlo : 0.f, TWO ? a.ax[1].vhi : 0.f};
    const int stride2 = nb1 + 1;
    unsigned *hl = s_hist + warp * (nb0 + 1) * 32 + lane;          // 1-D: lane-private column
    float *hs = (float *)s_hist + warp * (nb0 + 1) * 32 + lane;     // marked: sums
    float *hc = hs + GBP_WARPS * (nb0 + 1) * 32;                    // marked: compensations
    unsigned *hw = s_hist + (warp % copies) * nbin;                // shared copy of this warp
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    const float top0 = a.top0, top1 = a.top1;
    const unsigned ltmask = (1u << lane) - 1u;
    unsigned long long since_flush = 0, cand = 0;
    int qn = 0;  // entries in this warp's queue (warp-uniform)
    int cur_mock = -1;

    // Bin what is left in every warp's queue, then add the shared histograms
    // to mock `mk`'s global histogram and clear them.  Called by all threads.
    auto flush_all = [&](int mk) {
        __syncwarp();
        if (lane < qn) {
            const float4 e = s_q[lane];
            if (MODE == MODE_3D) bin_3d<true>(e, hl, A0, a);
            else if (MODE == MODE_3DS) bin_3d<false>(e, hw, A0, a);
            else if (MODE == MODE_XYZ) bin_xyz(e, hw, stride2, A0, A1, a);
            else if (MODE == MODE_SMU) bin_smu(e, hw, stride2, A0, A1, a);
            else if (MARK) bin_mark(e, hs, hc, A0, a);
        }
        qn = 0;
        __syncthreads();
        unsigned long long *gh = a.hist + (size_t)mk * a.hist_stride;
        if (MODE == MODE_3D) {
            for (int b = warp; b < nb0 + 1; b += GBP_WARPS) {
                unsigned long long s = 0;
                for (int w = 0; w < GBP_WARPS; w++) s += s_hist[(w * (nb0 + 1) + b) * 32 + lane];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (lane == 0 && s) atomicAdd(&gh[b], s);
            }
        } else if (MARK) {
            double *gd = a.histd + (size_t)mk * a.hist_stride;
            const float *S = (const float *)s_hist;
            const float *C = S + GBP_WARPS * (nb0 + 1) * 32;
            for (int b = warp; b < nb0; b += GBP_WARPS) {
                double s = 0.0;
                for (int w = 0; w < GBP_WARPS; w++) {
                    int idx = (w * (nb0 + 1) + b) * 32 + lane;
                    s += (double)S[idx] - (double)C[idx];
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (lane == 0 && s != 0.0) atomicAdd(&gd[b], s);
            }
        } else {
            for (int b = tid; b < nbin; b += GBP_BLOCK) {
                unsigned long long s = 0;
                for (int w = 0; w < copies; w++) s += s_hist[w * nbin + b];
                if (s) atomicAdd(&gh[b], s);
            }
        }
        __syncthreads();
        for (int i = tid; i < hist_words; i += GBP_BLOCK) s_hist[i] = 0u;
        __syncthreads();
    };
    __syncthreads();

    while (true) {
        if (tid == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= s_nitems) break;
        const int4 item = a.items[it];
        const int mock = item.x / a.ncells_mock;
        const int cell = item.x - mock * a.ncells_mock, ifirst = item.y, icnt = item.z;
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
        if (mock != cur_mock) {
            // batched mocks: a new mock's histogram starts here
            if (cur_mock >= 0) flush_all(cur_mock);
            cur_mock = mock;
        }
        const int keybase = mock * a.ncells_mock;
        for (int s = tid; s < a.nsten; s += GBP_BLOCK) {
            int pk = s_off[s];
            int x = cx + (pk & 255) - 64, y = cy + ((pk >> 8) & 255) - 64,
                z = cz + ((pk >> 16) & 255) - 64;
            bool ok = true;
            if (a.pbc) {
                x = x < 0 ? x + n0 : (x >= n0 ? x - n0 : x);
                y = y < 0 ? y + n1 : (y >= n1 ? y - n1 : y);
                z = z < 0 ? z + n2 : (z >= n2 ? z - n2 : z);
            } else {
                ok = x >= 0 && x < n0 && y >= 0 && y < n1 && z >= 0 && z < n2;
            }
            int st = 0, cn = 0;
            if (ok) {
                int c2 = keybase + (x * n1 + y) * n2 + z;
                st = a.start2[c2];
                cn = a.start2[c2 + 1] - st;
            }
            s_cstart[s] = st;
            s_pre[s] = cn;
        }
        __syncthreads();
        if (warp == 0) {
            // exclusive scan of the stencil cell counts, 32 entries per step
            int carry = 0;
            for (int b = 0; b < a.nsten; b += 32) {
                int idx = b + lane;
                int v = idx < a.nsten ? s_pre[idx] : 0;
                int incl = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                if (idx < a.nsten) s_pre[idx] = carry + incl - v;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) s_pre[a.nsten] = carry;
        }
        __syncthreads();
        const int total = s_pre[a.nsten];
        const int nselfj = a.nself ? s_pre[1] : 0;
        const int wpg = (icnt + 31) >> 5;
        const int G = GBP_WARPS / wpg;
        const int grp = warp / wpg;
        const int within = (warp % wpg) * 32 + lane;
        const bool in_group = grp < G;
        const bool active_i = in_group && within < icnt;
        float4 ui = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(-1));
        if (active_i) ui = a.pos1[ifirst + within];
        const int iself = __float_as_int(ui.w);
        float wi32 = 0.f;
        double wi64[5] = {0, 0, 0, 0, 0};
        if (MARK && active_i) {
            if (WF == 0) {
                for (int k = 0; k < nw; k++) wi64[k] = a.w64_1[(int64_t)(ifirst + within) * nw + k];
            } else {
                wi32 = a.w1[ifirst + within];
            }
        }
        cand += (unsigned long long)icnt * (unsigned long long)total;

        for (int base = 0; base < total; base += GBP_JCAP) {
            const int len = min(GBP_JCAP, total - base);
            for (int f = tid; f < len; f += GBP_BLOCK) {
                const int g = base + f;
                int lo = 0, hi = a.nsten - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (s_pre[mid] <= g) lo = mid; else hi = mid - 1;
                }
                const int j = s_cstart[lo] + (g - s_pre[lo]);
                float4 p = a.pos2[j];
                float4 D = s_D[lo];
                s_j[f] = make_float4(p.x + D.x, p.y + D.y, p.z + D.z, p.w);
                if (MARK) {
                    if (WF == 0) {
                        for (int k = 0; k < nw; k++) s_jw64[f * nw + k] = a.w64_2[(int64_t)j * nw + k];
                    } else {
                        s_jw[f] = a.w2[j];
                    }
                }
            }
            __syncthreads();
            if (in_group) {
                const int split = min(max(nselfj - base, 0), len);
                for (int seg = 0; seg < 2; seg++) {
                    // seg 0: own cell in auto mode (ordered pairs, i == j excluded);
                    // seg 1: the rest (each unordered pair once in auto mode)
                    const int jbeg = seg == 0 ? grp : split + ((grp - split) % G + G) % G;
                    const int jend = seg == 0 ? split : len;
                    const unsigned symbit = (seg == 1 && a.nself) ? SYM_BIT : 0u;
#pragma unroll 2
                    for (int jj = jbeg; jj < jend; jj += G) {
                        const float4 t = s_j[jj];
                        const float dx = ui.x - t.x, dy = ui.y - t.y, dz = ui.z - t.z;
                        float v0, v1 = 0.f;
                        bool in;
                        if (MODE == MODE_XYZ) {
                            v0 = fmaf(dy, dy, dx * dx);
                            v1 = dz * dz;
                            in = (v0 <= top0) & (v1 <= top1);
                        } else if (MODE == MODE_SMU) {
                            v1 = fmaf(dy, dy, dx * dx);
                            v0 = fmaf(dz, dz, v1);
                            in = v0 <= top0;
                        } else {
                            v0 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                            in = v0 <= top0;
                        }
                        const bool self = seg == 0 && __float_as_int(t.w) == iself;
                        if (MARK) {
                            if (WF == 1) v1 = wi32 * s_jw[jj];
                            else if (WF == 2) v1 = wi32 + s_jw[jj];
                            else if (in) v1 = (float)wfunc64(a.wfunc, wi64, s_jw64 + jj * nw);
                            // (i, i): separation exactly 0, its weight goes straight to that bin
                            if (self && a.self_bin < nb0) kahan_add(hs, hc, a.self_bin, v1);
                        }
                        in = in & !self;
                        const unsigned m = __ballot_sync(0xffffffffu, in);
                        if (m) {
                            if (in) {
                                const int pos = qn + __popc(m & ltmask);
                                s_q[pos] = make_float4(v0, v1, ui.w,
                                                       __uint_as_float(__float_as_uint(t.w) | symbit));
                            }
                            qn += __popc(m);
                            if (qn >= 32) {
                                // stage 2 on the top 32 entries, all lanes busy
                                __syncwarp();
                                const float4 e = s_q[qn - 32 + lane];
                                if (MODE == MODE_3D) bin_3d<true>(e, hl, A0, a);
                                else if (MODE == MODE_3DS) bin_3d<false>(e, hw, A0, a);
                                else if (MODE == MODE_XYZ) bin_xyz(e, hw, stride2, A0, A1, a);
                                else if (MODE == MODE_SMU) bin_smu(e, hw, stride2, A0, A1, a);
                                else if (MARK) bin_mark(e, hs, hc, A0, a);
                                qn -= 32;
                                __syncwarp();
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
        // a lane adds at most 2 per queued pair it drains; flush long before u32 overflow
        if (!MARK) {
            since_flush += 2ull * (unsigned long long)total *
                           (MODE == MODE_3D ? 1ull : (unsigned long long)(GBP_BLOCK / copies)) + 64ull;
            if (since_flush > (1ull << 31)) {
                flush_all(cur_mock);
                since_flush = 0;
            }
        }
    }
    if (cur_mock >= 0) flush_all(cur_mock);
    if (tid == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
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
    case MODE_MARK:
        if (wf == 1) return occ_t<MODE_MARK, 1>(smem);
        if (wf == 2) return occ_t<MODE_MARK, 2>(smem);
        return occ_t<MODE_MARK, 0>(smem);
    default: return 0;
    }
}
