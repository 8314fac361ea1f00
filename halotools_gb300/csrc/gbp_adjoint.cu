// Hand-written reverse pass for occupation-weighted pair counts (no reference
// counterpart: halotools has no gradients).
//
// Forward (marked mode, weight function 1): C_k = sum over ordered pairs of
// w_i w_j [d_ij <= r_k], self-pairs included.  For an upstream gradient g_k,
//   dL/dw_m = sum_j w_j (G(d_mj) + G(d_jm)),  G(d) = sum_{k: d <= r_k} g_k,
// which is 2 sum_j w_j G(d_mj) except where the two orders of a pair fall in
// different bins (guard-band pairs, re-evaluated in FP64 both ways here).
//
// k_adjoint: gather-only; each thread owns one point m of a work item and
// walks the full stencil (no symmetric half: no scatter, no atomics per
// point), accumulating w_j G(bin) in registers with a compensated (Kahan)
// FP32 sum; the j-groups of an item are reduced in shared memory at the end.
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
    atomicAdd(a.nrecheck, 1ull);
    const double *p = a.x64_1 + 3 * (int64_t)is;
    const double *q = a.x64_2 + 3 * (int64_t)js;
    int k1 = exact_bin(exact_pair(p, q, a).s2, b0, A);
    int k2 = exact_bin(exact_pair(q, p, a).s2, b0, A);
    return 0.5f * (gt[k1] + gt[k2]);
}

__global__ void __launch_bounds__(GBP_BLOCK, 3) k_adjoint(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb0 = a.ax[0].nb, T0 = a.ax[0].T;
    const SmemLayout L = gbp_smem_layout(MODE_ADJ, T0, 0, nb0, 0, a.nsten, 1, 4);
    float4 *s_lut0 = (float4 *)(smem + L.off_lut0);
    float4 *s_j = (float4 *)(smem + L.off_j);
    float *s_jw = (float *)(smem + L.off_jw);
    float4 *s_D = (float4 *)(smem + L.off_D);
    double *s_E0 = (double *)(smem + L.off_E0);
    float *s_hi0 = (float *)(smem + L.off_hi0);
    float *s_lo0 = (float *)(smem + L.off_lo0);
    int *s_off = (int *)(smem + L.off_off);
    int *s_cstart = (int *)(smem + L.off_cstart);
    int *s_pre = (int *)(smem + L.off_pre);
    float2 *s_part = (float2 *)(smem + L.off_hist);
    float *s_gt = (float *)(smem + L.off_hist + GBP_BLOCK * 8);
    __shared__ int s_item;
    __shared__ int s_nitems;

    for (int i = tid; i < T0; i += GBP_BLOCK) s_lut0[i] = a.ax[0].lut[i];
    for (int i = tid; i < nb0; i += GBP_BLOCK) {
        s_E0[i] = a.ax[0].E[i];
        s_hi0[i] = a.ax[0].hi[i];
        s_lo0[i] = a.ax[0].lo[i];
    }
    for (int i = tid; i <= nb0; i += GBP_BLOCK) s_gt[i] = a.gt[i];
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    if (tid == 0) s_nitems = *a.nitems;
    AxisSm A0{s_lut0, s_hi0, s_lo0, s_E0, nb0, a.ax[0].S, a.ax[0].B, a.ax[0].vlo, a.ax[0].vhi};
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    const float top0 = a.top0;
    unsigned long long cand = 0;
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
        const int wpg = (icnt + 31) >> 5;
        const int G = GBP_WARPS / wpg;
        const int grp = warp / wpg;
        const int within = (warp % wpg) * 32 + lane;
        const bool in_group = grp < G;
        float4 ui = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, __int_as_float(0));
        if (in_group && within < icnt) ui = a.pos1[ifirst + within];
        float acc = 0.f, comp = 0.f;  // Kahan: true sum ~ acc - comp
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
                s_jw[f] = a.w2[j];
            }
            __syncthreads();
            if (in_group) {
#pragma unroll 2
                for (int jj = grp; jj < len; jj += G) {
                    const float4 t = s_j[jj];
                    const float dx = ui.x - t.x, dy = ui.y - t.y, dz = ui.z - t.z;
                    const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (__any_sync(0xffffffffu, v <= top0)) {
                        float4 e = lut_entry(v, A0);
                        int b = __float_as_int(e.x) + (v > e.y ? 1 : 0);
                        float gv;
                        if ((v > e.z) & !(v > e.y))
                            gv = slow_adj(v, __float_as_int(e.x), __float_as_int(ui.w),
                                          __float_as_int(t.w), s_gt, A0, a);
                        else
                            gv = s_gt[b];
                        const float y = fmaf(s_jw[jj], gv, -comp);
                        const float s2 = acc + y;
                        comp = (s2 - acc) - y;
                        acc = s2;
                    }
                }
            }
            __syncthreads();
        }
        // reduce the j-groups of this item and write dL/dw in the caller's order
        s_part[tid] = make_float2(acc, comp);
        __syncthreads();
        if (in_group && grp == 0 && within < icnt) {
            double sum = 0.0;
            for (int g2 = 0; g2 < G; g2++) {
                float2 pc = s_part[(g2 * wpg + (warp % wpg)) * 32 + lane];
                sum += (double)pc.x - (double)pc.y;
            }
            a.grad[a.orig[ifirst + within]] = 2.0 * sum;
        }
        __syncthreads();
    }
    if (tid == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

cudaError_t gbp_launch_adjoint(const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_adjoint<<<grid, GBP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

int gbp_adjoint_occupancy(size_t smem) {
    int nblk = 0;
    if (cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_adjoint, GBP_BLOCK, smem) !=
        cudaSuccess)
        return 0;
    return nblk;
}

// ---------------- Zheng07 weights ----------------
__device__ __forceinline__ void zheng07_terms(double M, const Zheng07 &t, double *ncen,
                                              double *nsat, double *x, double *r) {
    const double logM = log10(M);
    *x = (logM - t.logMmin) / t.sigma;
    *ncen = 0.5 * (1.0 + erf(*x));
    const double M0 = exp10(t.logM0), M1 = exp10(t.logM1);
    *r = (M - M0) / M1;
    *nsat = M > M0 ? pow(*r, t.alpha) : 0.0;
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
        d[0] = g * (-dphi / th.sigma);       // logMmin
        d[1] = g * (-dphi * x / th.sigma);   // sigma_logM
        const double ln10 = 2.30258509299404568402;
        if (ns > 0.0) {
            const double M0 = exp10(th.logM0), M1 = exp10(th.logM1);
            d[2] = g * (th.alpha * ns / r) * (-M0 * ln10 / M1);  // logM0
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
