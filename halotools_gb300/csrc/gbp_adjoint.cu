// Hand-written reverse pass for occupation-weighted pair counts (no reference
// counterpart: halotools has no gradients).
//
// Forward (marked mode, weight function 1): C_k = sum over ordered pairs of
// w_i w_j [d_ij <= r_k], self-pairs included.  For an upstream gradient g_k,
//   dL/dw_m = sum_j w_j (G(d_mj) + G(d_jm)),  G(d) = sum_{k: d <= r_k} g_k,
// which is 2 sum_j w_j G(d_mj) except where the two orders of a pair fall in
// different bins (guard-band pairs, re-evaluated in FP64 both ways here).
//
// k_gather<false> (adjoint): gather-only over the full stencil (no symmetric
// half: no scatter), two i-points per lane; a packed range test marks the
// in-range j-slots, then each lane bins its own pairs and accumulates w_j G(bin)
// in registers with a compensated (Kahan) FP32 sum, added to dL/dw per item.
//
// k_gather<true> (npairs_per_object_3d, npairs_per_object_3d_engine.pyx): the
// same walk with lane-private per-point bin counters in shared memory, added to
// the (N1, nbins + 1) table per item; counts[i][k] = #j with d_ij^2 <= rbins[k]^2
// in the reference's (x_i - shift) - x_j order.
//
// k_zheng07_w / k_zheng07_vjp: Zheng07 mean occupations
// (zheng07_components.py:149-153, 455-470) as per-halo weights and the
// vector-Jacobian product sum_m gw_m dw_m/dtheta for theta =
// (logMmin, sigma_logM, logM0, logM1, alpha).
#include "gbp_device.cuh"

__device__ __noinline__ float slow_adj(float v, int b0, int is, int js, const float *gt,
                                       const AxisSm &A, const CountArgs &a) {
    int k = walk_bin(v, b0, A);
    if (k >= 0) return gt[k];
    if (is < 0 || js < 0) return 0.f;  // never a real pair
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, is, p);
    ref_pos(a, 1, js, q);
    int k1 = exact_bin(exact_pair(p, q, a).s2, b0, A);
    int k2 = exact_bin(exact_pair(q, p, a).s2, b0, A);
    return 0.5f * (gt[k1] + gt[k2]);
}

// Bin of one ordered pair (i, j) in the reference's order when the FP32 value
// cannot decide it (per-object counts).
__device__ __noinline__ int slow_one(float v, int b0, int is, int js, const AxisSm &A,
                                     const CountArgs &a) {
    int k = walk_bin(v, b0, A);
    if (k >= 0) return k;
    if (is < 0 || js < 0) return A.nb;  // never a real pair
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, is, p);
    ref_pos(a, 1, js, q);
    return exact_bin(exact_pair(p, q, a).s2, b0, A);
}

// Warp-centric like the count kernel: each warp pulls (block chunk, stencil
// group) items, two i-points per lane, 32 j-points per step.
template <bool POBJ>
__global__ void __launch_bounds__(GBP_BLOCK, 2) k_gather(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, T0 = a.ax[0].T;
    const SmemLayout L = gbp_smem_layout(POBJ ? MODE_POBJ : MODE_ADJ, T0, 0, nb0, 0, a.nsten, 0, 4);
    if (gbp_smem_too_small(L.total, a.err)) return;
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    float4 *jb = (float4 *)(smem + L.off_j) + warp * 32;
    // the same j-points with each coordinate twice, for the packed range test
    ulonglong2 *jxy = (ulonglong2 *)(smem + L.off_j2) + warp * 32;
    unsigned long long *jzz = (unsigned long long *)(smem + L.off_j2 + GBP_JCAP * 16) + warp * 32;
    float *jw = (float *)(smem + L.off_jw) + warp * 32;
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    int *s_off = (int *)(smem + L.off_off);
    float *s_gt = (float *)(smem + L.off_hist + GBP_BLOCK * 8);
    // per-object: this warp's lane-private counters [i-point 0/1][bin][lane]
    const int nbc = nb0 + 1;
    unsigned *cnt = (unsigned *)(smem + L.off_hist) + warp * 2 * nbc * 32 + lane;
    if (POBJ)
        for (int i = 0; i < 2 * nbc; i++) cnt[i * 32] = 0u;

    for (int i = tid; i < T0; i += GBP_BLOCK) s_lut0[i] = a.ax[0].lut[i];
    for (int i = tid; i < nb0; i += GBP_BLOCK) {
        s_E0[i] = a.ax[0].E[i];
        s_hi0[i] = a.ax[0].hi[i];
        s_lo0[i] = a.ax[0].lo[i];
    }
    if (!POBJ)
        for (int i = tid; i <= nb0; i += GBP_BLOCK) s_gt[i] = a.gt[i];
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    const int nitems = *a.nitems;
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    // range-test threshold with the slack of the count kernels (never drops a pair
    // that the binning would count)
    const float R0 = fmaf(a.top0, 0x1p-18f, a.top0) + 1.0e-30f;
    const unsigned long long RR0 = pk2(R0, R0);
    unsigned long long cand = 0;
    __syncthreads();

    while (true) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.counter, 1);
        it = __shfl_sync(FULL, it, 0);
        if (it >= nitems) break;
        const int4 item = a.items[it];
        const int cell = item.x, ifirst = item.y;
        const int icnt = item.z & 127, s0 = (item.z >> 7) & 1023, s1 = (item.z >> 17) & 1023;
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
        float4 u0 = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(0));
        float4 u1 = u0;
        if (lane < icnt) u0 = a.pos1[ifirst + lane];
        if (lane + 32 < icnt) u1 = a.pos1[ifirst + 32 + lane];
        const unsigned long long UX = pk2(u0.x, u1.x), UY = pk2(u0.y, u1.y), UZ = pk2(u0.z, u1.z);
        float acc0 = 0.f, cmp0 = 0.f, acc1 = 0.f, cmp1 = 0.f;  // Kahan: sum ~ acc - cmp
        for (int sb = s0; sb < s1; sb += 32) {
            const int s = sb + lane;
            int st = 0, cn = 0;
            float4 D = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s < s1) {
                D = s_D[s];
                const int key = gbp_run_key(s_off[s], cx, cy, cz, a.n, a.pbc, 0, a.bf3);
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
            cand += (unsigned long long)icnt * (unsigned long long)T;
            for (int f0 = 0; f0 < T; f0 += 32) {
                const int f = f0 + lane;
                int k = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(FULL, incl, k + step - 1);
                    if (v <= f) k += step;
                }
                k &= 31;
                const int stk = __shfl_sync(FULL, st, k);
                const int exk = __shfl_sync(FULL, incl - cn, k);
                const float Dx = __shfl_sync(FULL, D.x, k), Dy = __shfl_sync(FULL, D.y, k),
                            Dz = __shfl_sync(FULL, D.z, k);
                if (f < T) {
                    const int j = stk + (f - exk);
                    const float4 p = a.pos2[j];
                    const float tx = p.x + Dx, ty = p.y + Dy, tz = p.z + Dz;
                    jb[lane] = make_float4(tx, ty, tz, p.w);
                    jxy[lane] = make_ulonglong2(pk2(tx, tx), pk2(ty, ty));
                    jzz[lane] = pk2(tz, tz);
                    if (!POBJ) jw[lane] = a.w2[j];
                }
                __syncwarp();
                const int nj = min(32, T - f0);
                // range test of both i-points against all 32 slots (packed f32x2,
                // v exactly as below); slot jj lands in bit 31 - jj of the out-mask
                unsigned o0 = 0u, o1 = 0u;
#pragma unroll 8
                for (int jj = 0; jj < 32; jj++) {
                    const ulonglong2 txy = jxy[jj];
                    const unsigned long long dX = f2_sub(UX, txy.x), dY = f2_sub(UY, txy.y),
                                             dZ = f2_sub(UZ, jzz[jj]);
                    const unsigned long long d =
                        f2_sub(RR0, f2_fma(dZ, dZ, f2_fma(dY, dY, f2_mul(dX, dX))));
                    o0 = __funnelshift_l((unsigned)d, o0, 1);
                    o1 = __funnelshift_l((unsigned)(d >> 32), o1, 1);
                }
                const unsigned valid = nj >= 32 ? 0xffffffffu : ((1u << nj) - 1u);
                unsigned m0 = __brev(~o0) & valid, m1 = __brev(~o1) & valid;
                // each lane bins only its own in-range pairs: g = G(d_ij), and
                // accumulates w_j g for the i-point the pair belongs to
                while (m0 | m1) {
                    const bool first = m0 != 0u;
                    const int jj = 31 - __clz(first ? m0 : m1);
                    if (first) m0 ^= 1u << jj;
                    else m1 ^= 1u << jj;
                    const float4 u = first ? u0 : u1;
                    const float4 t = jb[jj];
                    const float dx = u.x - t.x, dy = u.y - t.y, dz = u.z - t.z;
                    const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    const float4 e = lut_entry(v, A0);
                    int b = __float_as_int(e.x) + (v > e.y ? 1 : 0);
                    if (POBJ) {
                        if ((v > e.z) & !(v > e.y))
                            b = slow_one(v, __float_as_int(e.x), __float_as_int(u.w),
                                         __float_as_int(t.w), A0, a);
                        cnt[((first ? 0 : nbc) + b) * 32] += 1u;
                        continue;
                    }
                    const float g = ((v > e.z) & !(v > e.y))
                                        ? slow_adj(v, __float_as_int(e.x), __float_as_int(u.w),
                                                   __float_as_int(t.w), s_gt, A0, a)
                                        : s_gt[b];
                    const float acc = first ? acc0 : acc1, cmp = first ? cmp0 : cmp1;
                    const float y = fmaf(jw[jj], g, -cmp), s2 = acc + y, c2 = (s2 - acc) - y;
                    if (first) {
                        acc0 = s2;
                        cmp0 = c2;
                    } else {
                        acc1 = s2;
                        cmp1 = c2;
                    }
                }
                __syncwarp();
            }
        }
        if (POBJ) {
            // this item's counts of the lane's two points, added to their rows
            for (int h = 0; h < 2; h++) {
                const int i = lane + 32 * h;
                const bool real = i < icnt;
                unsigned *row = real ? a.pobj + (size_t)a.orig[ifirst + i] * nbc : nullptr;
                for (int k = 0; k < nbc; k++) {
                    const unsigned c = cnt[(h * nbc + k) * 32];
                    if (c) {
                        if (real) atomicAdd(&row[k], c);
                        cnt[(h * nbc + k) * 32] = 0u;
                    }
                }
            }
        } else {
            if (lane < icnt)
                atomicAdd(&a.grad[a.orig[ifirst + lane]], 2.0 * ((double)acc0 - (double)cmp0));
            if (lane + 32 < icnt)
                atomicAdd(&a.grad[a.orig[ifirst + 32 + lane]], 2.0 * ((double)acc1 - (double)cmp1));
        }
    }
    if (lane == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

// Bins of one pair in both orders (k1 == k2 when FP32 decides), as slow_adj forms
// its mean over the two orders
__device__ __noinline__ int2 slow_adj_bins(float v, int b0, int is, int js, const AxisSm &A,
                                           const CountArgs &a) {
    int k = walk_bin(v, b0, A);
    if (k >= 0) return make_int2(k, k);
    if (is < 0 || js < 0) return make_int2(A.nb, A.nb);  // never a real pair
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, is, p);
    ref_pos(a, 1, js, q);
    return make_int2(exact_bin(exact_pair(p, q, a).s2, b0, A),
                     exact_bin(exact_pair(q, p, a).s2, b0, A));
}

// k_gather_ch: the adjoint gather over up to NCH weight channels at once (one
// parameter draw per channel): each in-range pair is binned once, then channel c
// adds w_j^c G^c(bin) to the i-point's sum in registers, so the distance work is
// shared by all channels.  The G table is bin-major and the channels go in packed
// f32x2 pairs: a pair costs 16-byte loads of G and w_j and one packed FMA per two
// channels into a run of at most 8 pairs; each run is then one packed
// compensated (Kahan) add.  Error bound per point and item for same-sign terms:
// 7u per run plus about 2u for the compensated sum of the runs.
// GBP_ADJC_BATCHES j batches are staged before the walk, and a lane walks the
// in-range pairs of all of them in one loop: its trip count is then its total
// over the batches, which varies far less between lanes than one batch's.
template <int NCH>
__global__ void __launch_bounds__(GBP_BLOCK, 2) k_gather_ch(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, T0 = a.ax[0].T, nch = a.nw;
    const SmemLayout L = gbp_smem_layout(MODE_ADJC, T0, 0, nb0, 0, a.nsten, 0, 4 * NCH);
    if (gbp_smem_too_small(L.total, a.err)) return;
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    constexpr int NB = GBP_ADJC_BATCHES;
    static_assert(NB == 4, "the walk keeps the slots' masks in two 64-bit words");
    float4 *jb = (float4 *)(smem + L.off_j) + warp * 32 * NB;
    ulonglong2 *jxy = (ulonglong2 *)(smem + L.off_j2) + warp * 32;
    unsigned long long *jzz = (unsigned long long *)(smem + L.off_j2 + GBP_JCAP * 16) + warp * 32;
    float *jw = (float *)(smem + L.off_jw) + warp * 32 * NB * NCH;
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    int *s_off = (int *)(smem + L.off_off);
    const int nbc = nb0 + 1;
    float *s_gt = (float *)(smem + L.off_hist);  // [bin][channel]
    for (int i = tid; i < T0; i += GBP_BLOCK) s_lut0[i] = a.ax[0].lut[i];
    for (int i = tid; i < nb0; i += GBP_BLOCK) {
        s_E0[i] = a.ax[0].E[i];
        s_hi0[i] = a.ax[0].hi[i];
        s_lo0[i] = a.ax[0].lo[i];
    }
    for (int i = tid; i < NCH * nbc; i += GBP_BLOCK) {
        const int k = i / NCH, c = i - k * NCH;
        s_gt[i] = c < nch ? a.gt[c * nbc + k] : 0.f;
    }
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    const int nitems = *a.nitems;
    const int n1 = a.n[1], n2 = a.n[2];
    const float R0 = fmaf(a.top0, 0x1p-18f, a.top0) + 1.0e-30f;
    const unsigned long long RR0 = pk2(R0, R0);
    unsigned long long cand = 0;
    __syncthreads();

    while (true) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.counter, 1);
        it = __shfl_sync(FULL, it, 0);
        if (it >= nitems) break;
        const int4 item = a.items[it];
        const int cell = item.x, ifirst = item.y;
        const int icnt = item.z & 127, s0 = (item.z >> 7) & 1023, s1 = (item.z >> 17) & 1023;
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
        float4 u0 = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(0));
        float4 u1 = u0;
        if (lane < icnt) u0 = a.pos1[ifirst + lane];
        if (lane + 32 < icnt) u1 = a.pos1[ifirst + 32 + lane];
        const unsigned long long UX = pk2(u0.x, u1.x), UY = pk2(u0.y, u1.y), UZ = pk2(u0.z, u1.z);
        // packed channel pairs (2q, 2q + 1) of the two points: sum ~ acc + ncm
        constexpr int NH = NCH / 2;
        unsigned long long acc0[NH], ncm0[NH], acc1[NH], ncm1[NH];
#pragma unroll
        for (int q = 0; q < NH; q++) acc0[q] = ncm0[q] = acc1[q] = ncm1[q] = 0ull;
        // the in-range pairs of one point over the staged slots (ma: slots 0-63,
        // mb: slots 64-127), highest slot of each word first: runs of up to 8
        // products summed by packed FMA, each run then one compensated add
        auto gather = [&](unsigned long long ma, unsigned long long mb, const float4 &u,
                          unsigned long long *acc, unsigned long long *ncm) {
            unsigned long long run[NH];
#pragma unroll
            for (int q = 0; q < NH; q++) run[q] = 0ull;
            int nr = 0;
            while (ma | mb) {
                const bool first = ma != 0ull;
                const int bit = 63 - __clzll(first ? ma : mb);
                if (first) ma ^= 1ull << bit;
                else mb ^= 1ull << bit;
                const int jj = bit + (first ? 0 : 64);
                const float4 t = jb[jj];
                const float dx = u.x - t.x, dy = u.y - t.y, dz = u.z - t.z;
                const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float4 e = lut_entry(v, A0);
                int2 kk;
                if ((v > e.z) & !(v > e.y)) {
                    kk = slow_adj_bins(v, __float_as_int(e.x), __float_as_int(u.w),
                                       __float_as_int(t.w), A0, a);
                } else {
                    const int b = __float_as_int(e.x) + (v > e.y ? 1 : 0);
                    kk = make_int2(b, b);
                }
                const ulonglong2 *wr = (const ulonglong2 *)(jw + jj * NCH);
                const ulonglong2 *gr = (const ulonglong2 *)(s_gt + kk.x * NCH);
                unsigned long long g[NH], w[NH];
#pragma unroll
                for (int q = 0; q < NH / 2; q++) {
                    const ulonglong2 gq = gr[q], wq = wr[q];
                    g[2 * q] = gq.x;
                    g[2 * q + 1] = gq.y;
                    w[2 * q] = wq.x;
                    w[2 * q + 1] = wq.y;
                }
                if (kk.x != kk.y) {
                    // the mean over the two orders: 0.5 (G[k1] + G[k2])
                    const ulonglong2 *hr = (const ulonglong2 *)(s_gt + kk.y * NCH);
                    const unsigned long long half = pk2(0.5f, 0.5f);
#pragma unroll
                    for (int q = 0; q < NH / 2; q++) {
                        const ulonglong2 hq = hr[q];
                        g[2 * q] = f2_mul(half, f2_add(g[2 * q], hq.x));
                        g[2 * q + 1] = f2_mul(half, f2_add(g[2 * q + 1], hq.y));
                    }
                }
#pragma unroll
                for (int q = 0; q < NH; q++) run[q] = f2_fma(w[q], g[q], run[q]);
                if (++nr == 8) {
#pragma unroll
                    for (int q = 0; q < NH; q++) {
                        kahan_f2(acc[q], ncm[q], pk2(1.f, 1.f), run[q]);
                        run[q] = 0ull;
                    }
                    nr = 0;
                }
            }
            if (nr) {
#pragma unroll
                for (int q = 0; q < NH; q++) kahan_f2(acc[q], ncm[q], pk2(1.f, 1.f), run[q]);
            }
        };
        for (int sb = s0; sb < s1; sb += 32) {
            const int s = sb + lane;
            int st = 0, cn = 0;
            float4 D = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s < s1) {
                D = s_D[s];
                const int key = gbp_run_key(s_off[s], cx, cy, cz, a.n, a.pbc, 0, a.bf3);
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
            cand += (unsigned long long)icnt * (unsigned long long)T;
            for (int f00 = 0; f00 < T; f00 += 32 * NB) {
                // masks of the NB batches' slots: bits 0-63 in *a, 64-127 in *b
                unsigned long long m0a = 0ull, m0b = 0ull, m1a = 0ull, m1b = 0ull;
#pragma unroll
                for (int bt = 0; bt < NB; bt++) {
                const int f0 = f00 + 32 * bt;
                if (f0 >= T) break;  // warp-uniform
                const int f = f0 + lane;
                int k = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(FULL, incl, k + step - 1);
                    if (v <= f) k += step;
                }
                k &= 31;
                const int stk = __shfl_sync(FULL, st, k);
                const int exk = __shfl_sync(FULL, incl - cn, k);
                const float Dx = __shfl_sync(FULL, D.x, k), Dy = __shfl_sync(FULL, D.y, k),
                            Dz = __shfl_sync(FULL, D.z, k);
                int jg = -1;  // the slot's sorted j index (-1: padding)
                if (f < T) {
                    const int j = stk + (f - exk);
                    jg = j;
                    const float4 p = a.pos2[j];
                    const float tx = p.x + Dx, ty = p.y + Dy, tz = p.z + Dz;
                    jb[32 * bt + lane] = make_float4(tx, ty, tz, p.w);
                    jxy[lane] = make_ulonglong2(pk2(tx, tx), pk2(ty, ty));
                    jzz[lane] = pk2(tz, tz);
                }
                {
                    // the slots' weight rows: lanes over (slot, channel), coalesced
                    // read-only loads all issued before the contiguous stores
#pragma unroll
                    for (int u0 = 0; u0 < NCH; u0 += 4) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const int t = 32 * (u0 + u) + lane, c = t % NCH;
                            const int js = __shfl_sync(FULL, jg, t / NCH);
                            v[u] = (js >= 0 && c < nch) ? __ldg(&a.w2[(int64_t)js * nch + c]) : 0.f;
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++) jw[32 * NCH * bt + 32 * (u0 + u) + lane] = v[u];
                    }
                }
                __syncwarp();
                const int nj = min(32, T - f0);
                unsigned o0 = 0u, o1 = 0u;
#pragma unroll 8
                for (int jj = 0; jj < 32; jj++) {
                    const ulonglong2 txy = jxy[jj];
                    const unsigned long long dX = f2_sub(UX, txy.x), dY = f2_sub(UY, txy.y),
                                             dZ = f2_sub(UZ, jzz[jj]);
                    const unsigned long long d =
                        f2_sub(RR0, f2_fma(dZ, dZ, f2_fma(dY, dY, f2_mul(dX, dX))));
                    o0 = __funnelshift_l((unsigned)d, o0, 1);
                    o1 = __funnelshift_l((unsigned)(d >> 32), o1, 1);
                }
                const unsigned valid = nj >= 32 ? 0xffffffffu : ((1u << nj) - 1u);
                const unsigned long long w0 = __brev(~o0) & valid, w1 = __brev(~o1) & valid;
                const int sh = 32 * (bt & 1);
                if (bt < 2) {
                    m0a |= w0 << sh;
                    m1a |= w1 << sh;
                } else {
                    m0b |= w0 << sh;
                    m1b |= w1 << sh;
                }
                __syncwarp();  // the next batch restages the stage-1 slots
                }
                gather(m0a, m0b, u0, acc0, ncm0);
                gather(m1a, m1b, u1, acc1, ncm1);
                __syncwarp();
            }
        }
        // this item's sums of the lane's two points: dL/dw rows (caller's order)
        auto lo = [](unsigned long long v) { return (double)__uint_as_float((unsigned)v); };
        auto hi = [](unsigned long long v) { return (double)__uint_as_float((unsigned)(v >> 32)); };
#pragma unroll
        for (int q = 0; q < NH; q++) {
            const int c = 2 * q;
            if (lane < icnt) {
                double *row = a.grad + (int64_t)a.orig[ifirst + lane] * nch;
                if (c < nch) atomicAdd(&row[c], 2.0 * (lo(acc0[q]) + lo(ncm0[q])));
                if (c + 1 < nch) atomicAdd(&row[c + 1], 2.0 * (hi(acc0[q]) + hi(ncm0[q])));
            }
            if (lane + 32 < icnt) {
                double *row = a.grad + (int64_t)a.orig[ifirst + 32 + lane] * nch;
                if (c < nch) atomicAdd(&row[c], 2.0 * (lo(acc1[q]) + lo(ncm1[q])));
                if (c + 1 < nch) atomicAdd(&row[c + 1], 2.0 * (hi(acc1[q]) + hi(ncm1[q])));
            }
        }
    }
    if (lane == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

// k_gather_c1: the batched adjoint over up to NCH (16) channels in one pass, one
// i-point per lane (items of at most 32 points), so that the 16 channels' sums
// fit in registers.  The two 8-channel passes of k_gather_ch each repeat the
// staging, the range tests and the binning of every pair; here they are done
// once.  Stage 1 packs two consecutive j-slots into each f32x2 operation.  The
// per-pair channel work, the runs of 8 and their compensated sums are those of
// k_gather_ch (error bound per point and item for same-sign terms: 7u per run
// plus about 2u for the compensated sum of the runs).
template <int NCH>
__global__ void __launch_bounds__(GBP_BLOCK, 2) k_gather_c1(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int NB = GBP_ADJC_BATCHES;
    static_assert(NB == 4, "the walk keeps the slots' masks in two 64-bit words");
    static_assert(NCH % 8 == 0, "channels go in groups of 8 (two 16-byte loads)");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, T0 = a.ax[0].T, nch = a.nw;
    const SmemLayout L = gbp_smem_layout(MODE_ADJC, T0, 0, nb0, 0, a.nsten, 0, 4 * NCH);
    if (gbp_smem_too_small(L.total, a.err)) return;
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    float4 *jb = (float4 *)(smem + L.off_j) + warp * 32 * NB;
    // the current batch's slots for stage 1: x, y, z arrays, read as pairs
    float *jx = (float *)(smem + L.off_j2) + warp * 96;
    float *jy = jx + 32, *jz = jx + 64;
    float *jw = (float *)(smem + L.off_jw) + warp * 32 * NB * NCH;
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    int *s_off = (int *)(smem + L.off_off);
    const int nbc = nb0 + 1;
    // The staged weight rows go chunk-major: 16-byte chunk q (channels 4q..4q+3)
    // of slot r at (q * 128 + r), so that lanes reading chunk q of different
    // slots fall in different banks (64-byte rows put every row's chunk q in
    // the same two bank groups).
    float *s_gt = (float *)(smem + L.off_hist);  // [bin][channel]
    for (int i = tid; i < T0; i += GBP_BLOCK) s_lut0[i] = a.ax[0].lut[i];
    for (int i = tid; i < nb0; i += GBP_BLOCK) {
        s_E0[i] = a.ax[0].E[i];
        s_hi0[i] = a.ax[0].hi[i];
        s_lo0[i] = a.ax[0].lo[i];
    }
    for (int i = tid; i < NCH * nbc; i += GBP_BLOCK) {
        const int k = i / NCH, c = i - k * NCH;
        s_gt[i] = c < nch ? a.gt[c * nbc + k] : 0.f;
    }
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    const int nitems = *a.nitems;
    const int n1 = a.n[1], n2 = a.n[2];
    const float R0 = fmaf(a.top0, 0x1p-18f, a.top0) + 1.0e-30f;
    const unsigned long long RR0 = pk2(R0, R0);
    unsigned long long cand = 0;
    __syncthreads();

    while (true) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.counter, 1);
        it = __shfl_sync(FULL, it, 0);
        if (it >= nitems) break;
        const int4 item = a.items[it];
        const int cell = item.x, ifirst = item.y;
        const int icnt = item.z & 127, s0 = (item.z >> 7) & 1023, s1 = (item.z >> 17) & 1023;
        const int cz = cell % n2, cy = (cell / n2) % n1, cx = cell / (n1 * n2);
        float4 u = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(0));
        if (lane < icnt) u = a.pos1[ifirst + lane];
        const unsigned long long UX = pk2(u.x, u.x), UY = pk2(u.y, u.y), UZ = pk2(u.z, u.z);
        constexpr int NH = NCH / 2;  // packed channel pairs
        unsigned long long acc[NH], ncm[NH];
#pragma unroll
        for (int q = 0; q < NH; q++) acc[q] = ncm[q] = 0ull;
        // the lane's in-range pairs over the staged slots (ma: slots 0-63, mb:
        // 64-127), highest slot of each word first
        auto gather = [&](unsigned long long ma, unsigned long long mb) {
            unsigned long long run[NH];
#pragma unroll
            for (int q = 0; q < NH; q++) run[q] = 0ull;
            int nr = 0;
            while (ma | mb) {
                const bool first = ma != 0ull;
                const int bit = 63 - __clzll(first ? ma : mb);
                if (first) ma ^= 1ull << bit;
                else mb ^= 1ull << bit;
                const int jj = bit + (first ? 0 : 64);
                const float4 t = jb[jj];
                const float dx = u.x - t.x, dy = u.y - t.y, dz = u.z - t.z;
                const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float4 e = lut_entry(v, A0);
                int2 kk;
                if ((v > e.z) & !(v > e.y)) {
                    kk = slow_adj_bins(v, __float_as_int(e.x), __float_as_int(u.w),
                                       __float_as_int(t.w), A0, a);
                } else {
                    const int b = __float_as_int(e.x) + (v > e.y ? 1 : 0);
                    kk = make_int2(b, b);
                }
                // channels in groups of 8: two 16-byte loads of G and of w_j each
#pragma unroll
                for (int h = 0; h < NCH / 8; h++) {
                    unsigned long long g[4], w[4];
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const int cq = 2 * h + q;
                        const ulonglong2 gq = *(const ulonglong2 *)(s_gt + kk.x * NCH + 4 * cq);
                        const ulonglong2 wq = *(const ulonglong2 *)(jw + (cq * 32 * NB + jj) * 4);
                        g[2 * q] = gq.x;
                        g[2 * q + 1] = gq.y;
                        w[2 * q] = wq.x;
                        w[2 * q + 1] = wq.y;
                    }
                    if (kk.x != kk.y) {
                        // the mean over the two orders: 0.5 (G[k1] + G[k2])
                        const unsigned long long half = pk2(0.5f, 0.5f);
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            const ulonglong2 hq =
                                *(const ulonglong2 *)(s_gt + kk.y * NCH + 4 * (2 * h + q));
                            g[2 * q] = f2_mul(half, f2_add(g[2 * q], hq.x));
                            g[2 * q + 1] = f2_mul(half, f2_add(g[2 * q + 1], hq.y));
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) run[4 * h + q] = f2_fma(w[q], g[q], run[4 * h + q]);
                }
                if (++nr == 8) {
#pragma unroll
                    for (int q = 0; q < NH; q++) {
                        kahan_f2(acc[q], ncm[q], pk2(1.f, 1.f), run[q]);
                        run[q] = 0ull;
                    }
                    nr = 0;
                }
            }
            if (nr) {
#pragma unroll
                for (int q = 0; q < NH; q++) kahan_f2(acc[q], ncm[q], pk2(1.f, 1.f), run[q]);
            }
        };
        for (int sb = s0; sb < s1; sb += 32) {
            const int s = sb + lane;
            int st = 0, cn = 0;
            float4 D = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s < s1) {
                D = s_D[s];
                const int key = gbp_run_key(s_off[s], cx, cy, cz, a.n, a.pbc, 0, a.bf3);
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
            cand += (unsigned long long)icnt * (unsigned long long)T;
            for (int f00 = 0; f00 < T; f00 += 32 * NB) {
                unsigned long long ma = 0ull, mb = 0ull;
#pragma unroll
                for (int bt = 0; bt < NB; bt++) {
                    const int f0 = f00 + 32 * bt;
                    if (f0 >= T) break;  // warp-uniform
                    const int f = f0 + lane;
                    int k = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int vv = __shfl_sync(FULL, incl, k + step - 1);
                        if (vv <= f) k += step;
                    }
                    k &= 31;
                    const int stk = __shfl_sync(FULL, st, k);
                    const int exk = __shfl_sync(FULL, incl - cn, k);
                    const float Dx = __shfl_sync(FULL, D.x, k), Dy = __shfl_sync(FULL, D.y, k),
                                Dz = __shfl_sync(FULL, D.z, k);
                    int jg = -1;  // the slot's sorted j index (-1: padding)
                    if (f < T) {
                        const int j = stk + (f - exk);
                        jg = j;
                        const float4 p = a.pos2[j];
                        const float tx = p.x + Dx, ty = p.y + Dy, tz = p.z + Dz;
                        jb[32 * bt + lane] = make_float4(tx, ty, tz, p.w);
                        jx[lane] = tx;
                        jy[lane] = ty;
                        jz[lane] = tz;
                    } else {
                        // padding: at -FAR, 2 FAR from an idle lane's point, and masked
                        jx[lane] = -GBP_FAR;
                        jy[lane] = -GBP_FAR;
                        jz[lane] = -GBP_FAR;
                    }
                    {
                        // the slots' weight rows: lanes over (slot, channel), coalesced
                        // read-only loads all issued before the contiguous stores
#pragma unroll
                        for (int u0 = 0; u0 < NCH; u0 += 4) {
                            float vw[4];
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                const int t = 32 * (u0 + q) + lane, c = t % NCH;
                                const int js = __shfl_sync(FULL, jg, t / NCH);
                                vw[q] = (js >= 0 && c < nch) ? __ldg(&a.w2[(int64_t)js * nch + c]) : 0.f;
                            }
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                const int t = 32 * (u0 + q) + lane, c = t % NCH;
                                const int r = 32 * bt + t / NCH;  // the slot's row
                                jw[((c >> 2) * 32 * NB + r) * 4 + (c & 3)] = vw[q];
                            }
                        }
                    }
                    __syncwarp();
                    // stage 1: slots 2k and 2k + 1 in one packed operation; v as the
                    // gather forms it, then R - v, whose sign bits are appended to o
                    const int nj = min(32, T - f0);
                    unsigned o = 0u;
                    const unsigned long long *jx2 = (const unsigned long long *)jx;
                    const unsigned long long *jy2 = (const unsigned long long *)jy;
                    const unsigned long long *jz2 = (const unsigned long long *)jz;
#pragma unroll 8
                    for (int kk2 = 0; kk2 < 16; kk2++) {
                        const unsigned long long dX = f2_sub(UX, jx2[kk2]), dY = f2_sub(UY, jy2[kk2]),
                                                 dZ = f2_sub(UZ, jz2[kk2]);
                        const unsigned long long d =
                            f2_sub(RR0, f2_fma(dZ, dZ, f2_fma(dY, dY, f2_mul(dX, dX))));
                        o = __funnelshift_l((unsigned)d, o, 1);
                        o = __funnelshift_l((unsigned)(d >> 32), o, 1);
                    }
                    const unsigned valid = nj >= 32 ? 0xffffffffu : ((1u << nj) - 1u);
                    const unsigned long long w0 = __brev(~o) & valid;
                    const int sh = 32 * (bt & 1);
                    if (bt < 2) ma |= w0 << sh;
                    else mb |= w0 << sh;
                    __syncwarp();  // the next batch restages the stage-1 slots
                }
                gather(ma, mb);
                __syncwarp();
            }
        }
        // this item's sums of the lane's point: its dL/dw row (caller's order)
        if (lane < icnt) {
            double *row = a.grad + (int64_t)a.orig[ifirst + lane] * nch;
#pragma unroll
            for (int q = 0; q < NH; q++) {
                const int c = 2 * q;
                const double lo = (double)__uint_as_float((unsigned)acc[q]) +
                                  (double)__uint_as_float((unsigned)ncm[q]);
                const double hi = (double)__uint_as_float((unsigned)(acc[q] >> 32)) +
                                  (double)__uint_as_float((unsigned)(ncm[q] >> 32));
                if (c < nch) atomicAdd(&row[c], 2.0 * lo);
                if (c + 1 < nch) atomicAdd(&row[c + 1], 2.0 * hi);
            }
        }
    }
    if (lane == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

cudaError_t gbp_launch_adjoint_ch(const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    if (a.nw > GBP_ADJ_CH) {
        cudaError_t e = cudaFuncSetAttribute(k_gather_c1<GBP_ADJ_CH_MAX>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gather_c1<GBP_ADJ_CH_MAX><<<grid, GBP_BLOCK, smem, st>>>(a);
        return cudaGetLastError();
    }
    cudaError_t e = cudaFuncSetAttribute(k_gather_ch<GBP_ADJ_CH>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_gather_ch<GBP_ADJ_CH><<<grid, GBP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

template <class K>
static int occupancy_of(K kernel, size_t smem) {
    int nblk = 0;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, kernel, GBP_BLOCK, smem) != cudaSuccess)
        return 0;
    return nblk;
}

int gbp_adjoint_ch_occupancy(size_t smem, int nw) {
    return nw > GBP_ADJ_CH ? occupancy_of(k_gather_c1<GBP_ADJ_CH_MAX>, smem)
                           : occupancy_of(k_gather_ch<GBP_ADJ_CH>, smem);
}

template <bool POBJ>
static cudaError_t gather_launch(const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_gather<POBJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_gather<POBJ><<<grid, GBP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

template <bool POBJ>
static int gather_occupancy(size_t smem) {
    int nblk = 0;
    if (cudaFuncSetAttribute(k_gather<POBJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_gather<POBJ>, GBP_BLOCK, smem) !=
        cudaSuccess)
        return 0;
    return nblk;
}

cudaError_t gbp_launch_adjoint(const CountArgs &a, int grid, size_t smem, cudaStream_t st,
                               bool per_object) {
    return per_object ? gather_launch<true>(a, grid, smem, st) : gather_launch<false>(a, grid, smem, st);
}

int gbp_adjoint_occupancy(size_t smem, bool per_object) {
    return per_object ? gather_occupancy<true>(smem) : gather_occupancy<false>(smem);
}

// ---------------- Zheng07 weights ----------------
__device__ __forceinline__ void zheng07_terms(double M, const Zheng07 &t, double *ncen,
                                              double *nsat, double *x, double *r) {
    const double logM = log10(M);
    *x = (logM - t.logMmin) * t.inv_sigma;
    *ncen = 0.5 * (1.0 + erf(*x));
    *r = (M - t.M0) * t.inv_M1;
    *nsat = M > t.M0 ? pow(*r, t.alpha) : 0.0;
}

__global__ void k_zheng07_w(const double *__restrict__ mass, int64_t n, Zheng07 th,
                            double *__restrict__ w) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double nc, ns, x, r;
    zheng07_terms(mass[i], th, &nc, &ns, &x, &r);
    w[i] = nc + ns;
}

__global__ void k_zheng07_vjp(const double *__restrict__ mass, int64_t n, Zheng07 th,
                              const double *__restrict__ gw, double *__restrict__ out5) {
    __shared__ double red[5][GBP_WARPS];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d[5] = {0, 0, 0, 0, 0};
    if (i < n) {
        const double M = mass[i], g = gw[i];
        double nc, ns, x, r;
        zheng07_terms(M, th, &nc, &ns, &x, &r);
        // d/dx of (1 + erf x)/2 is exp(-x^2)/sqrt(pi)
        const double dphi = exp(-x * x) * 0.56418958354775628695;
        d[0] = g * (-dphi * th.inv_sigma);       // logMmin
        d[1] = g * (-dphi * x * th.inv_sigma);   // sigma_logM
        const double ln10 = 2.30258509299404568402;
        if (ns > 0.0) {
            d[2] = g * (th.alpha * ns / r) * (-th.M0 * ln10 * th.inv_M1);  // logM0
            d[3] = g * (-th.alpha * ln10 * ns);                  // logM1
            d[4] = g * (ns * log(r));                            // alpha
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        double v = d[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = 0.0;
        for (int w = 0; w < GBP_WARPS; w++) v += red[threadIdx.x][w];
        atomicAdd(&out5[threadIdx.x], v);
    }
}

// ---------------- Zheng07 weights for many parameter vectors ----------------
// The occupations in FP32 (the counting kernels multiply the weights in FP32
// anyway, and GB300's FP64 units are slow) from an FP64 log10 M computed once per
// halo; W is (n, M) row-major: halo i, draw m.
// Per halo, once per call: log10 M (FP64) and M, each split into the nearest
// float and the float nearest the remainder (0 beside an infinite part, so that
// M = 0 gives log10 M = -inf and <Ncen> = 0 as in FP64)
__global__ void k_zheng07_prep(const double *__restrict__ mass, int64_t n,
                               float4 *__restrict__ hl) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double M = mass[i], lm = log10(M);
        const float lh = (float)lm, mh = (float)M;
        hl[i] = make_float4(lh, isfinite(lh) ? (float)(lm - (double)lh) : 0.f, mh,
                            isfinite(mh) ? (float)(M - (double)mh) : 0.f);
    }
}

// x = (log10 M - logMmin) / sigma_logM, r = (M - M0) / M1 and the FP32 mean
// occupations of one (halo, draw); d = M - M0 decides M > M0 with the sign of
// the FP64 difference
__device__ __forceinline__ void zheng07_terms_f(const float4 &h, const Zheng07F &t, float *ncen,
                                                float *nsat, float *x, float *r) {
    *x = ((h.x - t.lmin_hi) + (h.y - t.lmin_lo)) * t.inv_sigma;
    *ncen = 0.5f * (1.0f + erff(*x));
    const float d = (h.z - t.m0_hi) + (h.w - t.m0_lo);
    *r = d * t.inv_m1;
    *nsat = d > 0.0f ? powf(*r, t.alpha) : 0.0f;
}

__device__ __forceinline__ Zheng07F zheng07_f_load(const Zheng07F *th, int m) {
    const float4 *p = (const float4 *)(th + m);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    return Zheng07F{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

// W[i][m] for every (halo i, draw m): one element per thread, 32-bit indices
// while n * nth stays below 2^30
template <class I>
__global__ void k_zheng07_wb(const float4 *__restrict__ hl, I total, int nth,
                             const Zheng07F *__restrict__ th, double *__restrict__ W) {
    for (I e = blockIdx.x * (I)blockDim.x + threadIdx.x; e < total;
         e += (I)gridDim.x * blockDim.x) {
        const I i = e / (I)nth;
        const int m = (int)(e - i * (I)nth);
        float nc, ns, x, r;
        zheng07_terms_f(hl[i], zheng07_f_load(th, m), &nc, &ns, &x, &r);
        W[e] = (double)nc + (double)ns;
    }
}

// out[m][5] += sum_i gW[i][m] dw_i/dtheta_m: warp gw keeps draw m = gw % nth and
// strides over 32-halo chunks.  Each lane sums its terms in FP32 with Kahan
// compensation; the lanes' totals reduce in FP64 by shuffles to one add each.
__global__ void k_zheng07_vjpb(const float4 *__restrict__ hl, int64_t n,
                               const Zheng07F *__restrict__ th, int nth,
                               const double *__restrict__ gW, int nwarps, double *out) {
    const int gw = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (gw >= nwarps) return;  // (whole warps)
    const int m = gw % nth, wstep = nwarps / nth;
    const Zheng07F t = zheng07_f_load(th, m);
    const float ln10 = 2.302585093f;
    float s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
    auto add = [&](int k, float v) {
        const float y = v - c[k], u = s[k] + y;
        c[k] = (u - s[k]) - y;
        s[k] = u;
    };
    for (int64_t ch = gw / nth; ch * 32 < n; ch += wstep) {
        const int64_t i = ch * 32 + lane;
        if (i >= n) continue;
        const float g = (float)gW[i * nth + m];
        float nc, ns, x, r;
        zheng07_terms_f(hl[i], t, &nc, &ns, &x, &r);
        // d/dx of (1 + erf x)/2 is exp(-x^2)/sqrt(pi)
        const float dphi = expf(-x * x) * 0.5641895835f;
        add(0, g * (-dphi * t.inv_sigma));      // logMmin
        add(1, g * (-dphi * x * t.inv_sigma));  // sigma_logM
        if (ns > 0.0f) {
            add(2, g * (t.alpha * ns / r * t.c2));  // logM0
            add(3, g * (-t.alpha * ln10 * ns));     // logM1
            add(4, g * (ns * logf(r)));             // alpha
        }
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
        double v = (double)s[k] - (double)c[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.0) atomicAdd(&out[m * 5 + k], v);
    }
}

cudaError_t gbp_launch_zheng07_wb(const double *mass, float4 *hl, int64_t n, const Zheng07F *th,
                                  int nth, double *W, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_zheng07_prep<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, st>>>(mass, n,
                                                                                           hl);
    const int64_t total = n * nth;
    const unsigned g = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
    // 32-bit indices while the last grid stride cannot pass INT_MAX (stride < 2^20)
    if (total < ((int64_t)1 << 30))
        k_zheng07_wb<int><<<g, 256, 0, st>>>(hl, (int)total, nth, th, W);
    else
        k_zheng07_wb<int64_t><<<g, 256, 0, st>>>(hl, total, nth, th, W);
    return cudaGetLastError();
}

cudaError_t gbp_launch_zheng07_vjpb(const double *mass, float4 *hl, int64_t n, const Zheng07F *th,
                                    int nth, const double *gW, double *out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_zheng07_prep<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, st>>>(mass, n,
                                                                                           hl);
    // a whole number of warps per draw
    const int64_t chunks = (n + 31) / 32;
    const int per = (int)std::max<int64_t>(1, std::min<int64_t>(chunks, (152 * 16 * 8) / nth));
    const int nwarps = per * nth;
    k_zheng07_vjpb<<<(unsigned)((nwarps + 7) / 8), 256, 0, st>>>(hl, n, th, nth, gW, nwarps, out);
    return cudaGetLastError();
}

cudaError_t gbp_launch_zheng07_w(const double *mass, int64_t n, Zheng07 th, double *w,
                                 cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_zheng07_w<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(mass, n, th, w);
    return cudaGetLastError();
}

cudaError_t gbp_launch_zheng07_vjp(const double *mass, int64_t n, Zheng07 th, const double *gw,
                                   double *out5, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out5, 0, 5 * sizeof(double), st);
    if (e != cudaSuccess || n <= 0) return e;
    k_zheng07_vjp<<<(unsigned)((n + 255) / 256), GBP_BLOCK, 0, st>>>(mass, n, th, gw, out5);
    return cudaGetLastError();
}
