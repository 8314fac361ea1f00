// Pair-count kernels (sm_103a).  Replace the cell walks of
// npairs_3d_engine.pyx:103-182, npairs_xy_z_engine.pyx:143-194 and
// npairs_s_mu_engine.pyx:150-229.
//
// Work decomposition: a persistent grid pulls work items (cell, first i,
// i count <= 256) from an atomic cursor.  Each thread holds one i-point (FP32,
// relative to its cell) in registers; the points of the item's stencil cells
// are staged through shared memory with the cell offset o*c already added, so
// the inner loop is a broadcast LDS.128, three FSUB, one FMUL + two FFMA and a
// float-bit table lookup.  When the i count is small the CTA's warps split
// the staged j range into groups instead of idling.
//
// Exactness: the FP32 squared distance is compared with FP32 thresholds that
// bracket each FP64 edge by a rigorous error bound (built on the host).  A pair
// whose FP32 value falls inside a bracket is re-evaluated in FP64 with the
// reference's own operation order, ((x1 - shift) - x2) squared and summed left
// to right, unfused (npairs_3d_engine.pyx:167-176), so integer counts equal the
// reference's.
//
// Histograms: 1-D counts go to lane-private u32 bins in shared memory (no
// atomics, no bank conflicts: bin-major, lane-minor); 2-D counts go to one
// shared u32 histogram per warp with shared atomics.  Both are flushed to a
// global u64 histogram at the end (and early, before any u32 could overflow).
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

// ---------------- 3-D ----------------
// lane_stride 32: lane-private bins; 0: shared copy updated with atomics.
__device__ __noinline__ int slow_3d(float v, int b0, int is, int js, unsigned w,
                                    unsigned *hl, int lane_stride, const AxisSm &A,
                                    const CountArgs &a) {
    int k = walk_bin(v, b0, A);
    if (k >= 0) return k;
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *q = a.x64_2 + 3 * (int64_t)js;
    int k1 = exact_bin(exact_pair(p, q, a).s2, b0, A);
    if (w == 1) return k1;
    int k2 = exact_bin(exact_pair(q, p, a).s2, b0, A);
    if (lane_stride) {
        hl[k1 * lane_stride] += 1u;
        hl[k2 * lane_stride] += 1u;
    } else {
        if (k1 < A.nb) atomicAdd(&hl[k1], 1u);
        if (k2 < A.nb) atomicAdd(&hl[k2], 1u);
    }
    return -1;
}

// LANE: lane-private bins (stride 32 words per bin); otherwise a shared copy
// updated with atomics (wide histograms).
template <bool LANE>
__device__ __forceinline__ void pair_3d(const float4 &ui, const float4 &t, unsigned w,
                                        unsigned *hl, const AxisSm &A, const CountArgs &a) {
    float dx = ui.x - t.x, dy = ui.y - t.y, dz = ui.z - t.z;
    float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float4 e = lut_entry(v, A);
    int b = __float_as_int(e.x) + (v > e.y ? 1 : 0);
    if ((v > e.z) & !(v > e.y)) {
        b = slow_3d(v, __float_as_int(e.x), __float_as_int(ui.w), __float_as_int(t.w), w, hl,
                    LANE ? 32 : 0, A, a);
        if (b < 0) return;
    }
    if (LANE) hl[b * 32] += w;
    else if (b < A.nb) atomicAdd(&hl[b], w);
}

// ---------------- (rp, pi) ----------------
__device__ __noinline__ void slow_xyz(float v0, float v1, int b0a, int b0b, int is, int js,
                                      unsigned w, unsigned *hw, int stride, const AxisSm &A,
                                      const AxisSm &Bx, const CountArgs &a) {
    int ka = walk_bin(v0, b0a, A);
    int kb = walk_bin(v1, b0b, Bx);
    if (ka >= 0 && kb >= 0) {
        if (ka < A.nb && kb < Bx.nb) atomicAdd(&hw[ka * stride + kb], w);
        return;
    }
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *q = a.x64_2 + 3 * (int64_t)js;
    Exact3 r = exact_pair(p, q, a);
    int ea = ka >= 0 ? ka : exact_bin(r.dxy, b0a, A);
    int eb = kb >= 0 ? kb : exact_bin(r.dz2, b0b, Bx);
    if (ea < A.nb && eb < Bx.nb) atomicAdd(&hw[ea * stride + eb], 1u);
    if (w == 1) return;
    Exact3 s = exact_pair(q, p, a);
    int fa = ka >= 0 ? ka : exact_bin(s.dxy, b0a, A);
    int fb = kb >= 0 ? kb : exact_bin(s.dz2, b0b, Bx);
    if (fa < A.nb && fb < Bx.nb) atomicAdd(&hw[fa * stride + fb], 1u);
}

__device__ __forceinline__ void pair_xyz(const float4 &ui, const float4 &t, unsigned w,
                                         unsigned *hw, int stride, const AxisSm &A,
                                         const AxisSm &Bx, const CountArgs &a) {
    float dx = ui.x - t.x, dy = ui.y - t.y, dz = ui.z - t.z;
    float v0 = fmaf(dy, dy, dx * dx);
    float v1 = dz * dz;
    float4 e0 = lut_entry(v0, A);
    float4 e1 = lut_entry(v1, Bx);
    int ba = __float_as_int(e0.x) + (v0 > e0.y ? 1 : 0);
    int bb = __float_as_int(e1.x) + (v1 > e1.y ? 1 : 0);
    bool amb = ((v0 > e0.z) & !(v0 > e0.y)) | ((v1 > e1.z) & !(v1 > e1.y));
    if (amb) {
        slow_xyz(v0, v1, __float_as_int(e0.x), __float_as_int(e1.x), __float_as_int(ui.w),
                 __float_as_int(t.w), w, hw, stride, A, Bx, a);
        return;
    }
    if ((ba < A.nb) & (bb < Bx.nb)) atomicAdd(&hw[ba * stride + bb], w);
}

// ---------------- (s, mu') ----------------
// v = s^2 on axis 0; q = dxy / s^2 on axis 1, whose FP32 error depends on s:
// the s table's 4th field holds the q error bound for the slot's smallest s.
__device__ __noinline__ void slow_smu(float v, float q, float qb, int b0s, int is, int js,
                                      unsigned w, unsigned *hw, int stride, const AxisSm &A,
                                      const AxisSm &Q, const CountArgs &a) {
    int ks = walk_bin(v, b0s, A);
    int kq = -1;
    if (ks >= 0 && ks < A.nb && v > 0.0f) {
        // q decided only if it is farther than qb from every edge it could straddle
        int g = 0;
        while (g < Q.nb && q > Q.hi[g] + qb) g++;
        if (!(g < Q.nb && q > Q.lo[g] - qb)) kq = g;
    }
    if (ks >= A.nb) return;  // beyond the s gate: never counted
    if (ks >= 0 && kq >= 0) {
        if (kq < Q.nb) atomicAdd(&hw[ks * stride + kq], w);
        return;
    }
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *qq = a.x64_2 + 3 * (int64_t)js;
    for (int o = 0; o < (w == 1 ? 1 : 2); o++) {
        Exact3 r = o == 0 ? exact_pair(p, qq, a) : exact_pair(qq, p, a);
        int es = exact_bin(r.s2, 0, A);
        if (es >= A.nb) continue;
        double mu2 = (r.s2 > 0.0) ? __ddiv_rn(r.dxy, r.s2) : 0.0;
        int eq = exact_bin(mu2, 0, Q);
        if (eq >= Q.nb) continue;
        atomicAdd(&hw[es * stride + eq], 1u);
    }
}

__device__ __forceinline__ void pair_smu(const float4 &ui, const float4 &t, unsigned w,
                                         unsigned *hw, int stride, const AxisSm &A,
                                         const AxisSm &Q, const CountArgs &a) {
    float dx = ui.x - t.x, dy = ui.y - t.y, dz = ui.z - t.z;
    float dxy = fmaf(dy, dy, dx * dx);
    float v = fmaf(dz, dz, dxy);
    float4 e0 = lut_entry(v, A);
    int bs = __float_as_int(e0.x) + (v > e0.y ? 1 : 0);
    if (bs >= A.nb) return;  // beyond the s gate (the common case for far pairs)
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
        slow_smu(v, q, qb, __float_as_int(e0.x), __float_as_int(ui.w), __float_as_int(t.w), w,
                 hw, stride, A, Q, a);
        return;
    }
    if (bq >= Q.nb) return;  // beyond the mu' gate
    atomicAdd(&hw[bs * stride + bq], w);
}

// ---------------- kernel ----------------
template <int MODE>
__global__ void __launch_bounds__(GBP_BLOCK) k_count(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr bool TWO = (MODE == MODE_XYZ || MODE == MODE_SMU);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, nb1 = TWO ? a.ax[1].nb : 0;
    const int T0 = a.ax[0].T, T1 = TWO ? a.ax[1].T : 0;
    const int copies = a.hist_copies;
    const SmemLayout L = gbp_smem_layout(MODE, T0, T1, nb0, nb1, a.nsten, copies);
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    float4 *s_lut1 = (float4 *)(smem + L.off_lut1);
    float4 *s_j = (float4 *)(smem + L.off_j);
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
    const int hist_words = (MODE == MODE_3D) ? GBP_WARPS * (nb0 + 1) * 32 : copies * nbin;
    for (int i = tid; i < hist_words; i += GBP_BLOCK) s_hist[i] = 0u;
    if (tid == 0) s_nitems = *a.nitems;

    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    AxisSm A1{s_lut1, s_hi1, s_lo1, s_E1, nb1, TWO ? a.ax[1].S : 0, TWO ? a.ax[1].B : 0,
              TWO ? a.ax[1].vlo : 0.f, TWO ? a.ax[1].vhi : 0.f};
    const int stride2 = nb1 + 1;
    unsigned *hl = s_hist + warp * (nb0 + 1) * 32 + lane;          // 3-D: lane-private column
    unsigned *hw = s_hist + (warp % copies) * nbin;                // shared copy of this warp
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    unsigned long long since_flush = 0, cand = 0;
    __syncthreads();

    while (true) {
        if (tid == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= s_nitems) break;
        const int4 item = a.items[it];
        const int cell = item.x, ifirst = item.y, icnt = item.z;
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
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
                int c2 = (x * n1 + y) * n2 + z;
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
        float4 ui = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(0));
        if (in_group && within < icnt) ui = a.pos1[ifirst + within];
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
                float4 p = a.pos2[s_cstart[lo] + (g - s_pre[lo])];
                float4 D = s_D[lo];
                s_j[f] = make_float4(p.x + D.x, p.y + D.y, p.z + D.z, p.w);
            }
            __syncthreads();
            if (in_group) {
                const int split = min(max(nselfj - base, 0), len);
                const unsigned wrest = a.nself ? 2u : 1u;
                int jj = grp;
                // own-cell segment: every ordered pair once, except (i, i), whose
                // FP64 separation is exactly 0 and is added on the host
                const int iself = __float_as_int(ui.w);
                if (MODE == MODE_3D) {
#pragma unroll 4
                    for (; jj < split; jj += G)
                        if (__float_as_int(s_j[jj].w) != iself) pair_3d<true>(ui, s_j[jj], 1u, hl, A0, a);
#pragma unroll 4
                    for (; jj < len; jj += G) pair_3d<true>(ui, s_j[jj], wrest, hl, A0, a);
                } else if (MODE == MODE_3DS) {
#pragma unroll 4
                    for (; jj < split; jj += G)
                        if (__float_as_int(s_j[jj].w) != iself) pair_3d<false>(ui, s_j[jj], 1u, hw, A0, a);
#pragma unroll 4
                    for (; jj < len; jj += G) pair_3d<false>(ui, s_j[jj], wrest, hw, A0, a);
                } else if (MODE == MODE_XYZ) {
#pragma unroll 2
                    for (; jj < split; jj += G)
                        if (__float_as_int(s_j[jj].w) != iself) pair_xyz(ui, s_j[jj], 1u, hw, stride2, A0, A1, a);
#pragma unroll 2
                    for (; jj < len; jj += G) pair_xyz(ui, s_j[jj], wrest, hw, stride2, A0, A1, a);
                } else if (MODE == MODE_SMU) {
#pragma unroll 2
                    for (; jj < split; jj += G)
                        if (__float_as_int(s_j[jj].w) != iself) pair_smu(ui, s_j[jj], 1u, hw, stride2, A0, A1, a);
#pragma unroll 2
                    for (; jj < len; jj += G) pair_smu(ui, s_j[jj], wrest, hw, stride2, A0, A1, a);
                }
            }
            __syncthreads();
        }
        // a lane adds at most 2 per staged j it visits; flush long before u32 overflow
        since_flush += 2ull * (unsigned long long)total *
                       (MODE == MODE_3D ? 1ull : (unsigned long long)(GBP_BLOCK / copies));
        if (since_flush > (1ull << 31)) {
            for (int i = tid; i < hist_words; i += GBP_BLOCK) {
                unsigned v = s_hist[i];
                if (v) {
                    int bin = (MODE == MODE_3D) ? (i / 32) % (nb0 + 1) : i % nbin;
                    atomicAdd(&a.hist[bin], (unsigned long long)v);
                    s_hist[i] = 0u;
                }
            }
            since_flush = 0;
            __syncthreads();
        }
    }
    // final flush: reduce the copies and add to the global histogram
    __syncthreads();
    if (MODE == MODE_3D) {
        for (int b = warp; b < nb0 + 1; b += GBP_WARPS) {
            unsigned long long s = 0;
            for (int w = 0; w < GBP_WARPS; w++) s += s_hist[(w * (nb0 + 1) + b) * 32 + lane];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0 && s) atomicAdd(&a.hist[b], s);
        }
    } else {
        for (int b = tid; b < nbin; b += GBP_BLOCK) {
            unsigned long long s = 0;
            for (int w = 0; w < copies; w++) s += s_hist[w * nbin + b];
            if (s) atomicAdd(&a.hist[b], s);
        }
    }
    if (tid == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

template <int MODE>
static cudaError_t set_smem_attr(size_t smem) {
    return cudaFuncSetAttribute(k_count<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

cudaError_t gbp_launch_count(int mode, const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    switch (mode) {
    case MODE_3D:
        e = set_smem_attr<MODE_3D>(smem);
        if (e == cudaSuccess) k_count<MODE_3D><<<grid, GBP_BLOCK, smem, st>>>(a);
        break;
    case MODE_XYZ:
        e = set_smem_attr<MODE_XYZ>(smem);
        if (e == cudaSuccess) k_count<MODE_XYZ><<<grid, GBP_BLOCK, smem, st>>>(a);
        break;
    case MODE_SMU:
        e = set_smem_attr<MODE_SMU>(smem);
        if (e == cudaSuccess) k_count<MODE_SMU><<<grid, GBP_BLOCK, smem, st>>>(a);
        break;
    case MODE_3DS:
        e = set_smem_attr<MODE_3DS>(smem);
        if (e == cudaSuccess) k_count<MODE_3DS><<<grid, GBP_BLOCK, smem, st>>>(a);
        break;
    default:
        return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int gbp_count_occupancy(int mode, size_t smem) {
    int nblk = 0;
    cudaError_t e = cudaSuccess;
    switch (mode) {
    case MODE_3D:
        set_smem_attr<MODE_3D>(smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_count<MODE_3D>, GBP_BLOCK, smem);
        break;
    case MODE_XYZ:
        set_smem_attr<MODE_XYZ>(smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_count<MODE_XYZ>, GBP_BLOCK, smem);
        break;
    case MODE_SMU:
        set_smem_attr<MODE_SMU>(smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_count<MODE_SMU>, GBP_BLOCK, smem);
        break;
    case MODE_3DS:
        set_smem_attr<MODE_3DS>(smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_count<MODE_3DS>, GBP_BLOCK, smem);
        break;
    default:
        return 0;
    }
    return e == cudaSuccess ? nblk : 0;
}
