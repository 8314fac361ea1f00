// Cell-list build on the GPU: a counting sort that replaces the reference's
// argsort/searchsorted mesh (halotools rectangular_mesh.py:118-222).
//
// k_digitize   one thread per point: cell key, rank within the cell (one atomic
//              per distinct cell of a warp), FP32 block-relative coordinates.
//              Positions outside [0, L] or non-finite raise the error word.
// scan         exclusive prefix sum of the cell counts (three-kernel tile scan)
// k_scatter    one thread per point: writes the sorted FP32 record and the
//              sorted -> caller's row map (the FP64 recheck reads the caller's
//              positions through it); the warp then copies its points' weight
//              rows with lanes over (point, column), so that reads and writes
//              are whole rows.
// items        one work item per (block, chunk of <= GBP_TI points).
//
// Roofline: HBM-bound, about 12-24 B (positions) + 24 B read and 44 B written
// per point over the two passes.
#include "gbp_internal.cuh"

#include <algorithm>

#define SCAN_THREADS 1024
#define SCAN_TILE (SCAN_THREADS * 4)

// Block corners kb * bf * c per dimension: FP64 for FP64 input; for float32
// input an unevaluated float pair (hi, lo) with hi + lo = the corner to 2^-48,
// so that the cell-relative offset is formed in FP32 alone.
#define GBP_CORNERS 256

template <class T>
__global__ void __launch_bounds__(256) k_digitize(const T *__restrict__ xyz, int64_t npts, MeshDev m,
                                                  int *__restrict__ cellid, int *__restrict__ rank,
                                                  int *__restrict__ count, float4 *__restrict__ rel,
                                                  int *err) {
    constexpr bool F32 = sizeof(T) == 4;
    __shared__ double s_cd[F32 ? 1 : 3 * GBP_CORNERS];
    __shared__ float2 s_cf[F32 ? 3 * GBP_CORNERS : 1];
    for (int t = threadIdx.x; t < 3 * GBP_CORNERS; t += blockDim.x) {
        const int d = t / GBP_CORNERS, kb = t - d * GBP_CORNERS;
        const double C = (double)(kb * m.bf) * m.c[d];
        if (F32) {
            const float hi = __double2float_rn(C);
            s_cf[t] = make_float2(hi, __double2float_rn(C - (double)hi));
        } else {
            s_cd[t] = C;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i - lane < npts; i += stride) {
        // every lane of the warp stays to the end (the cell match is warp-wide)
        const bool live = i < npts;
        int c = -1;
        float u[3] = {0.f, 0.f, 0.f};
        if (live) {
            int mock = 0;
            if (m.offsets) {  // largest mock with offsets[mock] <= i
                int lo = 0, hi = m.nmocks - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (m.offsets[mid] <= i) lo = mid; else hi = mid - 1;
                }
                mock = lo;
            }
            int ib[3], il[3];
            bool bad = false;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const T x = xyz[3 * i + d];
                // also catches NaN; a float compares exactly against the largest float <= L
                if (F32 ? !(x >= T(0) && (float)x <= m.Lf[d]) : !(x >= T(0) && (double)x <= m.L[d]))
                    bad = true;
                // the cell only needs to be right to a few ulps: the stencil's pruning
                // and the error bound allow a point that far outside its cell
                int k = F32 ? (int)floorf((float)x * m.inv_cf[d]) : (int)floor((double)x * m.inv_c[d]);
                k = k < 0 ? 0 : (k >= m.n[d] ? m.n[d] - 1 : k);
                ib[d] = k / m.bf;
                il[d] = k - ib[d] * m.bf;
                // offset from the block corner
                if (F32) {
                    const float2 C = s_cf[d * GBP_CORNERS + ib[d]];
                    u[d] = ((float)x - C.x) - C.y;
                } else {
                    u[d] = __double2float_rn(__dsub_rn((double)x, s_cd[d * GBP_CORNERS + ib[d]]));
                }
            }
            if (bad) {
                atomicOr(err, 1);
                ib[0] = ib[1] = ib[2] = il[0] = il[1] = il[2] = 0;
                // far from everything, including idle lanes (+FAR) and padding (-FAR)
                u[0] = u[1] = u[2] = -0.5f * GBP_FAR;
            }
            // block-major key: a block's fine cells (and so its points) are contiguous
            const int bf = m.bf;
            c = (int)(mock * m.ncells) +
                ((ib[0] * m.nb[1] + ib[1]) * m.nb[2] + ib[2]) * (bf * bf * bf) +
                (il[0] * bf + il[1]) * bf + il[2];
        }
        // points of one cell in one warp share a single atomic (input order often
        // follows the clustering, e.g. satellites listed with their host)
        const unsigned peers = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if (live && lane == leader) base = atomicAdd(&count[c], __popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (live) {
            cellid[i] = c;
            rank[i] = base + __popc(peers & ((1u << lane) - 1u));
            rel[i] = make_float4(u[0], u[1], u[2], __int_as_float((int)i));
        }
    }
}

__global__ void k_scatter(int64_t npts, const int *__restrict__ cellid, const int *__restrict__ rank,
                          const int *__restrict__ start, const float4 *__restrict__ rel,
                          float4 *__restrict__ pos32, int *__restrict__ orig,
                          const double *__restrict__ w, int nw, float *__restrict__ w32,
                          double *__restrict__ w64) {
    // launched with whole warps (blocks of 256): every lane stays for the shuffles
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int dst = -1;
    if (i < npts) {
        dst = start[cellid[i]] + rank[i];
        float4 r = rel[i];
        r.w = __int_as_float(dst);
        pos32[dst] = r;
        orig[dst] = (int)i;
    }
    if (w) {
        // the warp's 32 rows: element t = (point t / nw, column t % nw)
        const int64_t i0 = i - lane;
        for (int t0 = 0; t0 < 32 * nw; t0 += 32) {
            const int t = t0 + lane, p = t / nw, k = t - p * nw;
            const int d = __shfl_sync(0xffffffffu, dst, p & 31);
            if (p < 32 && i0 + p < npts) {
                const double v = w[(i0 + p) * nw + k];
                w32[(int64_t)d * nw + k] = __double2float_rn(v);
                if (w64) w64[(int64_t)d * nw + k] = v;
            }
        }
    }
}

// ---- exclusive scan of n ints into n+1 outputs (out[n] = total) ----
__global__ void k_scan_tile(const int *__restrict__ in, int *__restrict__ out, int64_t n,
                            int *__restrict__ tile_sums) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * 4;
    int v[4];
    int s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int64_t idx = base + k;
        v[k] = (idx < n) ? in[idx] : 0;
        s += v[k];
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int ws = (lane < SCAN_THREADS / 32) ? warp_sums[lane] : 0;
        int wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = wi - ws;
        if (lane == 31 && tile_sums) tile_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    int run = warp_sums[warp] + incl - s;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int64_t idx = base + k;
        if (idx <= n) out[idx] = run;
        run += v[k];
    }
}

__global__ void k_scan_add(int *__restrict__ out, int64_t n, const int *__restrict__ offs) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * 4;
    int add = offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int64_t idx = base + k;
        if (idx <= n) out[idx] += add;
    }
}

// The device array whose entries add up to the total of the n counts that
// gbp_scan_exclusive just summed: the counts themselves when they fit one tile,
// else the per-tile sums it leaves at the start of its scratch (a few KB).  The
// caller adds them in int64 to check that the int32 prefix did not wrap.
void gbp_scan_parts(const int *d_in, int64_t n, const int *d_tmp, const int **parts,
                    int64_t *nparts) {
    const int64_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE;
    *parts = tiles == 1 ? d_in : d_tmp;
    *nparts = tiles == 1 ? n : tiles;
}

size_t gbp_scan_tmp_ints(int64_t n) {
    size_t total = 0;
    int64_t m = n + 1;
    while (m > SCAN_TILE) {
        int64_t tiles = (m + SCAN_TILE - 1) / SCAN_TILE;
        total += (size_t)tiles * 2 + 2;
        m = tiles;
    }
    return total + 16;
}

cudaError_t gbp_scan_exclusive(const int *d_in, int *d_out, int64_t n, int *d_tmp,
                               cudaStream_t st, int *launches) {
    int64_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        k_scan_tile<<<1, SCAN_THREADS, 0, st>>>(d_in, d_out, n, nullptr);
        if (launches) *launches += 1;
        return cudaGetLastError();
    }
    int *sums = d_tmp;                 // tiles
    int *sums_scan = d_tmp + tiles;    // tiles + 1
    k_scan_tile<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(d_in, d_out, n, sums);
    if (launches) *launches += 1;
    cudaError_t e = gbp_scan_exclusive(sums, sums_scan, tiles, d_tmp + 2 * tiles + 2, st, launches);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(d_out, n, sums_scan);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t gbp_build_cells(const void *d_xyz, int xyz_f32, int64_t npts, const MeshDev &m,
                            int *d_cellid, int *d_rank, int *d_count, int *d_start, int *d_scan_tmp,
                            float4 *d_pos32, int *d_orig, const double *d_w,
                            int nw, float *d_w32, double *d_w64, int *d_err, cudaStream_t st,
                            int *launches) {
    const int64_t nkeys = m.ncells * (int64_t)(m.offsets ? m.nmocks : 1);
    cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(int) * (size_t)nkeys, st);
    if (e != cudaSuccess) return e;
    // the FP32 relative records are staged in the pos32 buffer's twin (d_pos32 + npts)
    float4 *rel = d_pos32 + npts;
    unsigned g = (unsigned)((npts + 255) / 256);
    // digitise: a grid-stride loop over a few waves of CTAs (each builds the corner table once)
    const unsigned gd = (unsigned)std::min<int64_t>((npts + 255) / 256, 152 * 8);
    if (npts > 0) {
        if (xyz_f32)
            k_digitize<float><<<gd, 256, 0, st>>>((const float *)d_xyz, npts, m, d_cellid, d_rank,
                                                 d_count, rel, d_err);
        else
            k_digitize<double><<<gd, 256, 0, st>>>((const double *)d_xyz, npts, m, d_cellid, d_rank,
                                                  d_count, rel, d_err);
        if (launches) *launches += 1;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    e = gbp_scan_exclusive(d_count, d_start, nkeys, d_scan_tmp, st, launches);
    if (e != cudaSuccess) return e;
    if (npts > 0) {
        k_scatter<<<g, 256, 0, st>>>(npts, d_cellid, d_rank, d_start, rel, d_pos32, d_orig, d_w, nw,
                                     d_w32, d_w64);
        if (launches) *launches += 1;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Work items: (block key, first i-point, packed {i count <= ti, first and
// one-past-last stencil entry}).  A block's i-points are cut into chunks of
// ti (GBP_TI, or fewer for kernels that hold one point per lane); its stencil runs are cut into consecutive groups of at most `jcap`
// j-points (a group closes before the run that would overflow it), so every
// item costs at most GBP_TI * jcap pair evaluations plus one run.
struct ItemPlanDev {
    const int *start1, *start2;
    int64_t nkeys;  // block keys
    int ncm;        // blocks per mock
    int bf3;        // fine cells per block
    int n[3];       // blocks per dimension
    int pbc;
    const int *sten;
    const float4 *stenD;
    int nsten;
    int jcap;
    int ti;  // i-points per item
};

__device__ __forceinline__ int stencil_count(const ItemPlanDev &P, int keybase, int cx, int cy,
                                             int cz, int s) {
    const int key = gbp_run_key(P.sten[s], cx, cy, cz, P.n, P.pbc, keybase, P.bf3);
    if (key < 0) return 0;
    return P.start2[key + __float_as_int(P.stenD[s].w)] - P.start2[key];
}

// emit == false: count the items of every key; true: write them at off[key]
template <bool EMIT>
__global__ void k_items(ItemPlanDev P, int *__restrict__ nitem, const int *__restrict__ off,
                        int4 *__restrict__ items, int cap, int *__restrict__ nitems_total,
                        int *__restrict__ overflow) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (EMIT && k == 0) *nitems_total = min(off[P.nkeys], cap);
    if (EMIT && k == 0 && off[P.nkeys] > cap) *overflow = 1;
    if (k >= P.nkeys) return;
    const int first = P.start1[k * P.bf3], cnt = P.start1[(k + 1) * P.bf3] - first;
    const int q = (cnt + P.ti - 1) / P.ti;
    const int mock = (int)(k / P.ncm), cell = (int)(k - (int64_t)mock * P.ncm);
    const int cz = cell % P.n[2], cy = (cell / P.n[2]) % P.n[1], cx = cell / (P.n[1] * P.n[2]);
    const int keybase = mock * P.ncm;
    int o = EMIT ? off[k] : 0;
    int groups = 0, acc = 0, s0 = 0;
    if (cnt > 0) {
        for (int s = 0; s <= P.nsten; s++) {
            const int cn = s < P.nsten ? stencil_count(P, keybase, cx, cy, cz, s) : 0;
            const bool close = s == P.nsten ? acc > 0 : (acc > 0 && acc + cn > P.jcap);
            if (close) {
                if (EMIT) {
                    for (int c = 0; c < q; c++) {
                        const int num = min(P.ti, cnt - c * P.ti);
                        if (o < cap)
                            items[o] = make_int4((int)k, first + c * P.ti,
                                                 num | (s0 << 7) | (s << 17), 0);
                        o++;
                    }
                }
                groups++;
                acc = 0;
                s0 = s;
            }
            acc += cn;
        }
    }
    if (!EMIT) nitem[k] = q * groups;
}

cudaError_t gbp_build_items(const ItemPlan &ip, int4 *d_items, int cap, int *d_nitems,
                            int *d_overflow, int *d_tmp, int *d_scan_tmp, cudaStream_t st,
                            int *launches) {
    ItemPlanDev P;
    P.start1 = ip.start1;
    P.start2 = ip.start2;
    P.nkeys = ip.nkeys;
    P.ncm = ip.ncm;
    P.bf3 = ip.bf3;
    for (int d = 0; d < 3; d++) P.n[d] = ip.n[d];
    P.pbc = ip.pbc;
    P.sten = ip.sten;
    P.stenD = ip.stenD;
    P.nsten = ip.nsten;
    P.jcap = ip.jcap;
    P.ti = ip.ti > 0 && ip.ti <= GBP_TI ? ip.ti : GBP_TI;
    unsigned g = (unsigned)((ip.nkeys + 255) / 256);
    int *nitem = d_tmp;
    int *off = d_tmp + ip.nkeys + 1;
    k_items<false><<<g, 256, 0, st>>>(P, nitem, nullptr, nullptr, cap, nullptr, nullptr);
    if (launches) *launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = gbp_scan_exclusive(nitem, off, ip.nkeys, d_scan_tmp, st, launches);
    if (e != cudaSuccess) return e;
    k_items<true><<<g, 256, 0, st>>>(P, nitem, off, d_items, cap, d_nitems, d_overflow);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
