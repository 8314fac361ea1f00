// Per-object neighbour counts in per-point spheres or cylinders: the engines of
// counts_in_cylinders (counts_in_cells/engines/counts_in_cylinders_engine.pyx:
// 255-281) and of the isolation functions (isolation_functions/engines/
// spherical_isolation_engine.pyx:190-199, cylindrical_isolation_engine.pyx:
// 198-208, marked_spherical_isolation_engine.pyx:225-235,
// marked_cylindrical_isolation_engine.pyx:232-243).
//
// A pair (i, j) is a neighbour of i when, in the reference's FP64 order
// (dx = (x_i - shift) - x_j),
//   sphere:   dx^2 + dy^2 + dz^2 < r_i^2
//   cylinder: dx^2 + dy^2 < rp_i^2 and dz^2 < pi_i^2
// (strict), with r_i^2 = r_i * r_i in FP64; the isolation functions also need a
// separation > 0 and a marking function equal to 1, counts_in_cylinders an
// optional mass-fraction condition.
//
// k_neigh_thr computes each sample-1 point's FP32 guard thresholds once.
// k_neigh walks the full stencil (a gather: each i sees all its j), two
// i-points per lane, 32 j-points per step; a pair whose FP32 value falls inside
// the guard band, or at separation 0, is decided in FP64.  OUT selects what is
// written per point: 0 the count, 1 a has-neighbour flag, 2 the pair list at
// the point's offsets (a second pass after the counts).
#include "gbp_device.cuh"

// |v32 - v64| bound for v a sum of m squares near E (the count kernels' model)
__device__ __forceinline__ double neigh_band(double E, int m, const double *e) {
    const double E1 = E * (1.0 + 0x1p-10) + 1e-300;
    const double cmax = e[0], K = e[1], Lmax = e[2];
    const double d = 0x1p-24 * (4.0 * cmax + K * cmax + (K + 1.0) * cmax + sqrt(E1)) * 1.02 +
                     0x1p-46 * Lmax;
    const double sm = sqrt((double)m);
    return 2.0 * d * sm * sqrt(E1) + m * d * d + (m + 1) * 0x1p-24 * E1 + m * 0x1p-50 * E1;
}

// (lo, hi) with v32 < lo proving v64 < E and v32 > hi proving v64 > E
__device__ __forceinline__ float2 neigh_thr2(double E, int m, const double *e) {
    const double b = 2.0 * neigh_band(E, m, e);
    return make_float2(__double2float_rd(E - b), __double2float_ru(E + b));
}

__global__ void k_neigh_thr(const CountArgs a, int n1) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1; i += gridDim.x * blockDim.x) {
        const int nw = a.nw;
        const double r = a.w64_1[(size_t)i * nw];
        // counts_in_cylinders_engine.pyx:107-112: rp_max * rp_max in FP64
        const double r2 = __dmul_rn(r, r);
        float4 t;
        if (a.ngeo == 0) {
            const float2 s = neigh_thr2(r2, 3, a.nerr);
            t = make_float4(s.x, s.y, 0.f, 0.f);
        } else {
            const double p = a.w64_1[(size_t)i * nw + 1];
            const float2 s = neigh_thr2(r2, 2, a.nerr);
            const float2 z = neigh_thr2(__dmul_rn(p, p), 1, a.nerr);
            t = make_float4(s.x, s.y, z.x, z.y);
        }
        a.nthr[i] = t;
    }
}

// marking functions of the conditional isolation functions
// (isolation_criteria_marking_functions.pyx:30-136) on FP64 marks
__device__ __forceinline__ bool iso_cond(int id, const double *w1, const double *w2) {
    switch (id) {
    case 0: return true;
    case 1: return w1[0] > w2[0];
    case 2: return w1[0] < w2[0];
    case 3: return w1[0] == w2[0];
    case 4: return w1[0] != w2[0];
    case 5: return w1[0] > (w2[0] + w1[1]);
    case 6: return w1[0] < (w2[0] + w1[1]);
    default: return false;
    }
}

// The pair's condition (marks are columns 2.. of the sorted FP64 rows)
__device__ __forceinline__ bool neigh_cond(const CountArgs &a, int si, int sj) {
    if (a.ncond == 0) return true;
    const double *m1 = a.w64_1 + (size_t)si * a.nw + 2;
    const double *m2 = a.w64_2 + (size_t)sj * a.nw + 2;
    if (a.ncond >= 10) return iso_cond(a.ncond - 10, m1, m2);
    // conditions.pyx MassFrac.func: mass2[j] / mass1[i] within (fmin, fmax)
    double f;
    if (m1[0] == 0.0) f = (m2[0] == 0.0) ? 1.0 : INFINITY;
    else f = __ddiv_rn(m2[0], m1[0]);
    const bool t1 = a.nceq[0] ? (a.ncpar[0] <= f) : (a.ncpar[0] < f);
    const bool t2 = a.nceq[1] ? (f <= a.ncpar[1]) : (f < a.ncpar[1]);
    return t1 && t2;
}

// FP64 decision for a pair the FP32 values cannot settle (sorted indices)
__device__ __noinline__ bool neigh_exact(const CountArgs &a, int si, int sj, double r2, double p2) {
    atomicAdd(a.nrecheck, 1ull);
    double p[3], q[3];
    ref_pos(a, 0, si, p);
    ref_pos(a, 1, sj, q);
    const Exact3 e = exact_pair(p, q, a);
    const bool in = a.ngeo == 0 ? (e.s2 < r2) : (e.dxy < r2) & (e.dz2 < p2);
    if (!in) return false;
    if (a.nexcl0 && !(__dadd_rn(e.dz2, e.dxy) > 0.0)) return false;
    return true;
}

template <int GEO, int OUT>
__global__ void __launch_bounds__(GBP_BLOCK, 2) k_neigh(const CountArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // (4 bytes per j-point in the jw region: the j-slots' sorted indices)
    const SmemLayout L = gbp_smem_layout(MODE_NEIGH, a.ax[0].T, GEO ? a.ax[1].T : 0, a.ax[0].nb,
                                         GEO ? a.ax[1].nb : 0, a.nsten, 0, 4);
    if (gbp_smem_too_small(L.total, a.err)) return;
    int *jsl = (int *)(smem + L.off_jw) + warp * 32;  // sorted index of each j-slot
    ulonglong2 *jxy = (ulonglong2 *)(smem + L.off_j2) + warp * 32;
    unsigned long long *jzz = (unsigned long long *)(smem + L.off_j2 + GBP_JCAP * 16) + warp * 32;
    float4 *s_D = (float4 *)(smem + L.off_D);
    int *s_off = (int *)(smem + L.off_off);
    for (int i = tid; i < a.nsten; i += GBP_BLOCK) {
        s_off[i] = a.sten[i];
        s_D[i] = a.stenD[i];
    }
    const int nitems = *a.nitems;
    const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
    (void)n0;
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
        // two i-points per lane: position, sorted index and thresholds (idle: never in)
        float4 u0 = make_float4(GBP_FAR, GBP_FAR, GBP_FAR, 0.f), u1 = u0;
        float4 t0 = make_float4(-1.f, -1.f, -1.f, -1.f), t1 = t0;
        const int si0 = ifirst + lane, si1 = ifirst + 32 + lane;
        if (lane < icnt) { u0 = a.pos1[si0]; t0 = a.nthr[si0]; }
        if (lane + 32 < icnt) { u1 = a.pos1[si1]; t1 = a.nthr[si1]; }
        const unsigned long long UX = pk2(u0.x, u1.x), UY = pk2(u0.y, u1.y), UZ = pk2(u0.z, u1.z);
        unsigned c0 = 0, c1 = 0;  // neighbours found (OUT 0 / 1), or slots written (OUT 2)
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
                    jsl[lane] = j;
                    jxy[lane] = make_ulonglong2(pk2(tx, tx), pk2(ty, ty));
                    jzz[lane] = pk2(tz, tz);
                }
                __syncwarp();
                const int nj = min(32, T - f0);
                for (int jj = 0; jj < nj; jj++) {
                    const ulonglong2 txy = jxy[jj];
                    const unsigned long long dX = f2_sub(UX, txy.x), dY = f2_sub(UY, txy.y),
                                             dZ = f2_sub(UZ, jzz[jj]);
                    // v exactly as the count kernels form it: xy = fma(dy, dy, dx dx),
                    // sphere = fma(dz, dz, xy), z = dz dz
                    const unsigned long long vxy = f2_fma(dY, dY, f2_mul(dX, dX));
                    const unsigned long long vz = f2_mul(dZ, dZ);
                    const unsigned long long vs = f2_fma(dZ, dZ, vxy);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const float4 t = h ? t1 : t0;
                        const float a0 = __uint_as_float(h ? (unsigned)((GEO ? vxy : vs) >> 32)
                                                           : (unsigned)(GEO ? vxy : vs));
                        const float az = __uint_as_float(h ? (unsigned)(vz >> 32) : (unsigned)vz);
                        // in: provably inside; out: provably outside; else FP64
                        bool in, out;
                        if (GEO == 0) {
                            in = a0 < t.x;
                            out = !(a0 <= t.y);
                        } else {
                            in = (a0 < t.x) & (az < t.z);
                            out = !(a0 <= t.y) | !(az <= t.w);
                        }
                        if (out) continue;
                        const int si = h ? si1 : si0, sj = jsl[jj];
                        if (in && a.nexcl0) {
                            // a neighbour must be apart: separation 0 in FP32 may be
                            // a distinct point an ulp away; the point itself never is
                            const float sv = GEO ? a0 + az : a0;
                            if (sv == 0.0f) {
                                if (a.same && si == sj) continue;
                                in = false;  // decide in FP64
                            }
                        }
                        if (!in) {
                            const double r = a.w64_1[(size_t)si * a.nw];
                            const double p = GEO ? a.w64_1[(size_t)si * a.nw + 1] : 0.0;
                            if (!neigh_exact(a, si, sj, __dmul_rn(r, r), __dmul_rn(p, p))) continue;
                        }
                        if (!neigh_cond(a, si, sj)) continue;
                        if (OUT == 2) {
                            // pair list: the point's next slot (caller indices)
                            const int oi = a.orig1[si];
                            const unsigned slot = atomicAdd(&a.pcur[oi], 1u);
                            const long long at = a.poff[oi] + slot;
                            if (at < a.poff[oi + 1]) {
                                a.pairs[2 * at] = (unsigned)oi;
                                a.pairs[2 * at + 1] = (unsigned)a.orig2[sj];
                            } else {
                                atomicOr(a.err, GBP_ERR_PAIR_SLOTS);  // more pairs than counted
                            }
                        } else {
                            if (h) c1++; else c0++;
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (OUT != 2) {
            // this item's neighbours of the lane's points, added to their rows
            if (lane < icnt && c0) {
                const int oi = a.orig1[si0];
                if (OUT == 0) atomicAdd(&a.pobj[oi], c0);
                else a.pobj[oi] = 1u;
            }
            if (lane + 32 < icnt && c1) {
                const int oi = a.orig1[si1];
                if (OUT == 0) atomicAdd(&a.pobj[oi], c1);
                else a.pobj[oi] = 1u;
            }
        }
    }
    if (lane == 0 && cand) atomicAdd(a.nrecheck + 1, cand);
}

template <int GEO, int OUT>
static cudaError_t neigh_launch_t(const CountArgs &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_neigh<GEO, OUT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_neigh<GEO, OUT><<<grid, GBP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t gbp_launch_neigh(const CountArgs &a, int n1, int out, int grid, size_t smem,
                             cudaStream_t st) {
    const int tb = 256, tg = std::max(1, std::min((n1 + tb - 1) / tb, 152 * 8));
    k_neigh_thr<<<tg, tb, 0, st>>>(a, n1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (a.ngeo == 0) {
        if (out == 0) return neigh_launch_t<0, 0>(a, grid, smem, st);
        if (out == 1) return neigh_launch_t<0, 1>(a, grid, smem, st);
        return neigh_launch_t<0, 2>(a, grid, smem, st);
    }
    if (out == 0) return neigh_launch_t<1, 0>(a, grid, smem, st);
    if (out == 1) return neigh_launch_t<1, 1>(a, grid, smem, st);
    return neigh_launch_t<1, 2>(a, grid, smem, st);
}

int gbp_neigh_occupancy(size_t smem) {
    int nblk = 0;
    if (cudaFuncSetAttribute(k_neigh<1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, k_neigh<1, 0>, GBP_BLOCK, smem) !=
        cudaSuccess)
        return 0;
    return nblk;
}
