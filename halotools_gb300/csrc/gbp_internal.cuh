// Internal definitions shared by the gbpairs CUDA translation units.
//
// Data layout in HBM (one sample; the auto-correlation path sorts once):
//   pos32[N]  float4  block-relative FP32 coordinates (x - bx*bf*cx, ...) in
//                     block-major cell-sorted order, .w = sorted index (int bits)
//   orig[N]   int     sorted position -> caller's row (the FP64 recheck reads
//                     the caller's positions through it)
//   start[ncells+1]   CSR offsets of each fine cell's points (block-major keys)
// A count kernel walks work items (block, first point, point count, stencil
// group) and, per item, streams the stencil runs' points through shared memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GBP_BLOCK 256
#define GBP_WARPS (GBP_BLOCK / 32)
#define GBP_TI 64           // max i-points per work item (two per lane of one warp)
#define GBP_JCAP_ITEM 2048  // j-points per work item (stencil group cap)
#define GBP_JCAP (GBP_WARPS * 32)  // staged j-points: 32 per warp
#define GBP_LUT_MAX 1024    // float-bit lookup slots per axis
#define GBP_QCAP 0          // per-warp queue of in-range pairs (entries; unused)
#define GBP_NB_MAX 1024     // edges per axis
#define GBP_NB_LANE 64      // 1-D histograms up to this size use lane-private bins
#define GBP_SMAX 512        // stencil cells
#define GBP_FAR 1.0e18f     // coordinate of an idle lane: far outside every edge

enum { MODE_3D = 0, MODE_XYZ = 1, MODE_SMU = 2, MODE_MARK = 3, MODE_ADJ = 4, MODE_3DS = 5,
       MODE_MARKC = 6,    // product marks (id 1) over several channels in one pass
       MODE_JACK = 7,     // jackknife: counts plus a (tag, bin) table of pair ends
       MODE_POBJ = 8,     // per-object counts (gather walk of the adjoint)
       MODE_XYZW = 9,     // (rp, pi) sums of a marking function (marked_npairs_xy_z)
       MODE_SMUW = 10,    // (s, mu') counts and w1 * w2 sums (weighted_npairs_s_mu)
       MODE_JACKXYZ = 11,    // (rp, pi) counts plus a global (tag, bin) table of pair ends
       MODE_NEIGH = 12,      // per-object neighbours in per-point spheres / cylinders
       MODE_JACKW = 13,      // weighted jackknife, 3-D: w1 w2 sums plus an FP64 (tag, bin) table
       MODE_JACKXYZW = 14,   // weighted jackknife, (rp, pi)
       MODE_ADJC = 15 };     // adjoint over several weight channels (parameter draws)

// channels of one batched adjoint launch
#define GBP_ADJ_CH 8
// ... and up to GBP_ADJ_CH_MAX in one pass with one i-point per lane (items of 32)
#define GBP_ADJ_CH_MAX 16
// channels a batched adjoint launch stages per j-point: 8, or 16 past 8
__host__ __device__ inline int gbp_adjc_nch(int nw) { return nw <= GBP_ADJ_CH ? GBP_ADJ_CH : GBP_ADJ_CH_MAX; }
// batched adjoint: 32-point j batches staged per pass; a lane walks the in-range
// pairs of all of them in one loop, which evens out the lanes' trip counts
#define GBP_ADJC_BATCHES 4

// Pair geometry of a count mode: (rp, pi) cylinders or (s, mu') cones; every
// other mode measures 3-D separations
__host__ __device__ constexpr bool gbp_mode_xyz(int m) {
    return m == MODE_XYZ || m == MODE_XYZW || m == MODE_JACKXYZ || m == MODE_JACKXYZW;
}
__host__ __device__ constexpr bool gbp_mode_smu(int m) { return m == MODE_SMU || m == MODE_SMUW; }

// The weighted 2-D modes add each pair's weight to a per-CTA FP32 pair
// (hi, lo): hi by atomic add, lo by the exact rounding error of that add
// (TwoSum on the value the atomic returned).  Warps move (hi, lo) into a per-CTA
// FP64 sum every GBP_W2_FLUSH binned pairs, and the CTA adds that to the global
// FP64 histogram once at the end.
#define GBP_W2_FLUSH 2048
__host__ __device__ inline int gbp_w2_bytes(int nbin) {
    return 2 * ((nbin * 4 + 15) / 16 * 16) + nbin * 8;
}

// One binning axis: squared quantity v compared with edges E'[0..nb-1]
// (non-decreasing); bin(v) = smallest k with v <= E'[k], nb if none.
// hi/lo are FP32 thresholds: v32 > hi[k] proves v64 > E'[k]; v32 <= lo[k]
// proves v64 <= E'[k].  lut[s] = {b0 (int bits), thr, lo, qband}.
struct AxisDev {
    const float4 *lut;
    const float *hi;
    const float *lo;
    const double *E;
    int nb;
    int T;      // lut slots
    int S;      // right shift of the float bits
    int B;      // first slot's shifted-bits value
    float vlo;  // clamp range of v before the lookup
    float vhi;
};

struct CountArgs {
    const float4 *pos1;
    const float4 *pos2;
    const void *xyz1;       // caller's positions on the device, (N, 3); the FP64 recheck
    const void *xyz2;       // reads them through orig1 / orig2
    int xyz1_f32, xyz2_f32; // positions are float32 (upcast exactly)
    const int *orig1;       // sorted position -> row of xyz1
    const int *orig2;       // sorted position -> row of xyz2
    const int *start2;
    const int4 *items;
    const int *nitems;      // device scalar (written by the item builder)
    int *counter;           // work-item cursor, zero before launch
    unsigned long long flush_after;  // early flush of the u32 histogram words (j-batches x 64)
    const int *sten;        // runs: block offset (ox+64) | (oy+64)<<8 | (oz+64)<<16 | first cell<<24
    const float4 *stenD;    // FP32 block offsets o*bf*c and (bits of) the run length
    int nsten;
    int nself;              // 1 if stencil[0] is the own block counted once (auto mode), else 0
    int n[3];               // blocks per dimension
    int bf3;                // fine cells per block
    int pbc;
    double L[3];
    AxisDev ax[2];
    int hist_stride;        // histogram words per mock (global histogram is [mock][bin])
    int ncells_mock;        // blocks per mock: work-item key = mock * ncells_mock + block
    int hist_copies;        // shared histogram copies (2-D and wide 1-D): 8 = one per warp, or 1
    unsigned long long *hist;   // global differential histogram(s)
    unsigned long long *htag;   // jackknife: (ntag, nb0 + 1) counts of pair ends by tag
    unsigned *pobj;             // per-object: (N1, nb0 + 1) counts, caller's order
    int *err;                   // error word: bit 1 = shared-memory layout larger than the launch
    int ntag;                   // jackknife: number of tags (N_samples + 1)
    unsigned long long *nrecheck;
    float top0, top1;       // above these a pair is out of range on that axis
    // marked / adjoint
    const float *w1;        // sorted weights, (N1, nw) FP32
    const float *w2;
    const double *w64_1;    // sorted FP64 weights (marking functions evaluated in FP64)
    const double *w64_2;
    int nw;
    int wfunc;
    int self_bin;           // bin of separation 0 (marked auto mode adds f(w_i, w_i) there)
    double *histd;          // FP64 weighted histogram (marked)
    // adjoint
    const float *gt;        // gt[b] = sum of the upstream gradient over cumulative bins >= b
    const int *orig;        // sorted position -> caller's index
    double *grad;           // dL/dw in the caller's order
    // per-object neighbours (MODE_NEIGH): sample 1 rows of w64_1 hold
    // {r or rp, pi, marks...}, sample 2 rows {0, 0, marks...}
    float4 *nthr;           // per sorted sample-1 point: FP32 guard thresholds
    double nerr[3];         // error model: cell size bound, reach, box size bound
    int ngeo;               // 0: sphere s^2 < r^2; 1: cylinder dxy^2 < rp^2 and dz^2 < pi^2
    int nexcl0;             // isolation: a neighbour needs separation > 0
    int ncond;              // 0 none; 1 mass fraction; 10 + id: isolation marking function id
    double ncpar[2];        // mass fraction limits (fmin, fmax)
    int nceq[2];            // mass fraction: lower / upper bound inclusive
    int same;               // sample 2 is sample 1 (same indices)
    const long long *poff;  // pair list: first slot of each caller-order sample-1 point (n1 + 1)
    unsigned *pcur;         // pair list: slots taken per point
    unsigned *pairs;        // pair list: (i1, i2) caller indices
};

// Shared-memory layout of the count kernel, identical on host and device.
// jw: bytes of staged weights per j-point (marked mode), copies: shared
// histogram copies (2-D and wide 1-D modes).
struct SmemLayout {
    int off_lut0, off_lut1, off_hl0, off_hl1, off_j, off_j2, off_jw, off_q, off_code, off_rec, off_rq,
        off_D, off_E0, off_E1, off_hi0, off_lo0, off_hi1, off_lo1, off_off, off_hist, total;
};

// Deferred FP64 rechecks of the (s, mu') mode: each warp keeps a ring of
// GBP_RQCAP pairs {i, j, walk starts, flags} and its tail counter, and
// re-evaluates them 32 at a time with every lane busy.
#define GBP_RQCAP 96

// Stage-2 i-slots per warp: the lane's first point at slot lane, its second at
// lane + 48, so that the two never share a shared-memory bank.
#define GBP_USLOTS 80
// Items of at most this many i-points run stage 1 transposed (lanes over the
// j-slots, a loop over the i-points): cheaper than 32 j-steps per lane when the
// item is small
#ifndef GBP_TRANSPOSE
#define GBP_TRANSPOSE 20
#endif
__host__ __device__ inline int gbp_uslot(int iu) { return iu + ((iu >> 5) << 4); }

__host__ __device__ inline int gbp_align(int x, int a) { return (x + a - 1) / a * a; }

// Product marks over several channels (MODE_MARKC): the channels are staged and
// summed in packed FP32 pairs, the number of pairs a power of two (zero columns
// pad the last ones), so that 32 lanes split into (pair group, channel pair).
__host__ __device__ inline int gbp_markc_pairs(int nw) {
    int p = 1;
    while (2 * p < nw) p <<= 1;
    return p;
}
// With GBP_MARKC_SORTED to GBP_MARKC_SORTED_MAX channel pairs (5 to 16
// channels), MARKC sorts each code batch by bin and sums the products bin by
// bin; otherwise each lane adds its own channel's products round by round to
// lane-private columns (with 17 to 32 channels the sort scratch would push the
// shared memory past the per-CTA limit from about 23 bins on).
#define GBP_MARKC_SORTED 4
#define GBP_MARKC_SORTED_MAX 8
__host__ __device__ inline bool gbp_markc_sorted(int nw) {
    const int p = gbp_markc_pairs(nw);
    return p >= GBP_MARKC_SORTED && p <= GBP_MARKC_SORTED_MAX;
}
// MARKC staged columns per point: packed pairs (zero-padded) in the sorted form,
// the channels themselves otherwise
__host__ __device__ inline int gbp_markc_cols(int nw) {
    return gbp_markc_sorted(nw) ? 2 * gbp_markc_pairs(nw) : nw;
}
// MARKC sorted form: a code batch holds the pairs of both i-halves of a 32-point
// j batch (64 x 32 codes), so a sort spreads its per-bin cost over twice the pairs
#ifndef GBP_MARKC_CODES
#define GBP_MARKC_CODES 2048
#endif
// MARKC per-warp scratch of one code batch (sorted form): each code's bin (u8),
// the codes sorted by bin (u16), and two counters per bin
__host__ __device__ inline int gbp_markc_sort_bytes(int nb0) {
    return gbp_align(GBP_MARKC_CODES * 3 + 8 * (nb0 + 1), 16);
}

__host__ __device__ inline SmemLayout gbp_smem_layout(int mode, int T0, int T1, int nb0, int nb1,
                                                      int nsten, int copies, int jw,
                                                      int ntag = 0) {
    SmemLayout L;
    int o = 0;
    // adjoint: float4 tables {b0, thr, lo, qband}; count kernels: u32 table
    // {b0 | threshold-pair index << 16} and the threshold pairs (hi, lo)
    const bool adj = mode == MODE_ADJ || mode == MODE_POBJ || mode == MODE_NEIGH ||
                     mode == MODE_ADJC;  // gather kernels
    // ((s, mu'): the s words paired with the q error bounds; the q thresholds as
    // float4 {thr, lo, hi below, lo above})
    const bool smu = gbp_mode_smu(mode);
    // (3-D counts: the slot words, then each slot's own threshold pair)
    const bool lutd = mode == MODE_3D;
    L.off_lut0 = o;
    o += adj ? T0 * 16 : lutd ? gbp_align(T0 * 4, 16) + gbp_align(T0 * 8, 16)
                              : gbp_align(T0 * (smu ? 8 : 4), 16);
    L.off_lut1 = o; o += adj ? T1 * 16 : gbp_align(T1 * 4, 16);
    L.off_hl0 = o; o += adj ? 0 : gbp_align((nb0 + 2) * 8, 16);
    L.off_hl1 = o; o += adj ? 0 : gbp_align((nb1 + 2) * (smu ? 16 : 8), 16);
    const int jb = mode == MODE_ADJC ? GBP_ADJC_BATCHES : 1;  // j batches staged at once
    L.off_j = o; o += jb * GBP_JCAP * 16;   // adjoint: float4 per j; count: x, y, z, index arrays
    L.off_j2 = o; o += GBP_JCAP * 24;   // (x,x,y,y), (z,z) per j
    L.off_jw = o; o += gbp_align(jb * GBP_JCAP * jw, 16);
    L.off_q = o;
    o += adj ? 0 : GBP_WARPS * GBP_USLOTS * 16 +
                       gbp_align(GBP_WARPS * GBP_USLOTS * (jw > 4 ? jw : 4), 16);
    // codes of one 32-point j batch: 64 x 32 (marked modes other than the sorted
    // channel form: one i-point at a time, 32 x 32)
    const bool msort = mode == MODE_MARKC && gbp_markc_sorted(jw / 4);
    L.off_code = o;
    o += adj ? 0
             : GBP_WARPS * ((mode == MODE_MARK || (mode == MODE_MARKC && !msort)) ? 1024
                            : msort ? GBP_MARKC_CODES : 2048) * 2;
    L.off_rec = o;
    o += mode != MODE_MARKC ? 0
         : msort ? GBP_WARPS * gbp_markc_sort_bytes(nb0)
                 : GBP_WARPS * 32 * 16;  // binned pairs of one round {bin, second bin, i, j}
    L.off_rq = o; o += smu ? GBP_WARPS * (GBP_RQCAP * 16 + 16) : 0;
    L.off_D = o; o += nsten * 16;
    L.off_E0 = o; o += gbp_align(nb0 * 8, 16);
    L.off_E1 = o; o += gbp_align(nb1 * 8, 16);
    L.off_hi0 = o; o += gbp_align(nb0 * 4, 16);
    L.off_lo0 = o; o += gbp_align(nb0 * 4, 16);
    L.off_hi1 = o; o += gbp_align(nb1 * 4, 16);
    L.off_lo1 = o; o += gbp_align(nb1 * 4, 16);
    L.off_off = o; o += gbp_align(nsten * 4, 16);
    L.off_hist = o;
    int hist_bytes;
    if (mode == MODE_3D) {
        hist_bytes = GBP_WARPS * (nb0 + 1) * 32 * 4;          // lane-private u32
    } else if (mode == MODE_JACK) {
        // lane-private u32 counts, then the CTA's u64 (tag, bin) table
        hist_bytes = gbp_align(GBP_WARPS * (nb0 + 1) * 32 * 4, 16) + ntag * (nb0 + 1) * 8;
    } else if (mode == MODE_MARK || (mode == MODE_MARKC && !msort)) {
        hist_bytes = GBP_WARPS * (nb0 + 1) * 32 * 4 * 2;      // lane-private FP32 sum + compensation
    } else if (mode == MODE_MARKC) {
        // per warp, (bin, channel pair): packed FP32 sums + packed compensations
        hist_bytes = GBP_WARPS * (nb0 + 1) * (jw / 8) * 16;
    } else if (mode == MODE_ADJ) {
        hist_bytes = GBP_BLOCK * 8 + gbp_align((nb0 + 1) * 4, 16);  // partial sums + gt table
    } else if (mode == MODE_ADJC) {
        hist_bytes = gbp_align((jw / 4) * (nb0 + 1) * 4, 16);      // gt table per channel
    } else if (mode == MODE_NEIGH) {
        hist_bytes = 0;                                       // counters live in registers
    } else if (mode == MODE_POBJ) {
        hist_bytes = GBP_WARPS * 2 * (nb0 + 1) * 32 * 4;      // lane-private counters, 2 points
    } else if (mode == MODE_3DS) {
        hist_bytes = copies * (nb0 + 1) * 4;                  // shared u32 copies (wide 1-D)
    } else {
        hist_bytes = copies * (nb0 + 1) * (nb1 + 1) * 4;      // shared u32 copies (2-D)
        if (mode == MODE_XYZW || mode == MODE_SMUW || mode == MODE_JACKW ||
            mode == MODE_JACKXYZW)                            // then the CTA's weighted sums
            hist_bytes = gbp_align(hist_bytes, 16) + gbp_w2_bytes((nb0 + 1) * (nb1 + 1));
    }
    o += gbp_align(hist_bytes, 16);
    L.total = o;
    return L;
}

#define GBP_ERR_SMEM_LAYOUT 2
#define GBP_ERR_PAIR_SLOTS 4  // a pair-list pass found more pairs than the counts gave

// True (and the error bit set) when the kernel's own shared-memory layout does
// not fit the dynamic shared memory it was launched with; the kernel then
// returns before touching shared memory.
__device__ __forceinline__ bool gbp_smem_too_small(int total, int *err) {
    unsigned dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    if ((unsigned)total <= dyn) return false;
    if (threadIdx.x == 0 && err) atomicOr(err, GBP_ERR_SMEM_LAYOUT);
    return true;
}

// Fine-cell key of stencil run `pk` seen from block (cx, cy, cz) of the mock
// whose first block key is `keybase`; -1 when the neighbour block lies outside
// a non-periodic box.
__device__ __forceinline__ int gbp_run_key(int pk, int cx, int cy, int cz, const int n[3], int pbc,
                                           int keybase, int bf3) {
    int x = cx + (pk & 255) - 64, y = cy + ((pk >> 8) & 255) - 64, z = cz + ((pk >> 16) & 255) - 64;
    if (pbc) {
        x = x < 0 ? x + n[0] : (x >= n[0] ? x - n[0] : x);
        y = y < 0 ? y + n[1] : (y >= n[1] ? y - n[1] : y);
        z = z < 0 ? z + n[2] : (z >= n[2] ? z - n[2] : z);
    } else if (x < 0 || x >= n[0] || y < 0 || y >= n[1] || z < 0 || z >= n[2]) {
        return -1;
    }
    return (keybase + (x * n[1] + y) * n[2] + z) * bf3 + ((pk >> 24) & 127);
}

// ---- launchers (defined in the .cu files) ----
struct MeshDev {
    int n[3];                   // fine cells per dimension
    int bf;                     // fine cells per block edge (keys are block-major)
    int nb[3];                  // blocks per dimension
    double c[3];
    double inv_c[3];            // 1 / c, rounded (only picks the cell)
    float inv_cf[3];            // the same in FP32 (float32 input)
    float Lf[3];                // largest float <= L (range check of float32 input)
    double L[3];
    int64_t ncells;             // cells per mock
    const int64_t *offsets;     // device, nmocks+1 point offsets (null: one sample)
    int nmocks;                 // samples sorted together; cell key = mock * ncells + cell
};

// Digitise, count, scan and scatter one sample (or a batch of mocks) into the
// cell-sorted layout.  xyz_f32: positions are float32 (upcast exactly).
cudaError_t gbp_build_cells(const void *d_xyz, int xyz_f32, int64_t npts, const MeshDev &m, int *d_cellid,
                            int *d_rank, int *d_count, int *d_start, int *d_scan_tmp,
                            float4 *d_pos32, int *d_orig, const double *d_w,
                            int nw, float *d_w32, double *d_w64, int *d_err, cudaStream_t st,
                            int *launches);
// Work items (cell key, first i, packed {count, stencil range}) for every
// non-empty cell of the sorted sample 1; writes at most `cap` items and sets
// *d_overflow if more were needed.
struct ItemPlan {
    const int *start1, *start2;   // over fine-cell keys
    int64_t nkeys;                // block keys (all mocks)
    int ncm;                      // blocks per mock
    int bf3;                      // fine cells per block
    int n[3];                     // blocks per dimension
    int pbc;
    const int *sten;      // device
    const float4 *stenD;  // device (run lengths in .w)
    int nsten;
    int jcap;
    int ti = GBP_TI;      // i-points per item (at most GBP_TI)
};
cudaError_t gbp_build_items(const ItemPlan &ip, int4 *d_items, int cap, int *d_nitems,
                            int *d_overflow, int *d_tmp, int *d_scan_tmp, cudaStream_t st,
                            int *launches);
cudaError_t gbp_scan_exclusive(const int *d_in, int *d_out, int64_t n, int *d_tmp,
                               cudaStream_t st, int *launches);
size_t gbp_scan_tmp_ints(int64_t n);
void gbp_scan_parts(const int *d_in, int64_t n, const int *d_tmp, const int **parts,
                    int64_t *nparts);

// mode: MODE_*; wf: marking-function template (1 product, 2 sum, 0 any id in FP64)
cudaError_t gbp_launch_count(int mode, int wf, const CountArgs &a, int grid, size_t smem,
                             cudaStream_t st);
int gbp_count_occupancy(int mode, int wf, size_t smem);
cudaError_t gbp_count_set_smem(size_t smem);
// the gather kernel: adjoint (dL/dw), or per-object counts when per_object
cudaError_t gbp_launch_adjoint(const CountArgs &a, int grid, size_t smem, cudaStream_t st,
                               bool per_object = false);
int gbp_adjoint_occupancy(size_t smem, bool per_object = false);
// batched adjoint: up to GBP_ADJ_CH weight channels (a.nw) per launch
cudaError_t gbp_launch_adjoint_ch(const CountArgs &a, int grid, size_t smem, cudaStream_t st);
int gbp_adjoint_ch_occupancy(size_t smem, int nw);
// per-object neighbours: thresholds pre-pass then k_neigh<geometry, out>
// (out 0 counts, 1 has-neighbour flags, 2 pair list)
cudaError_t gbp_launch_neigh(const CountArgs &a, int n1, int out, int grid, size_t smem,
                             cudaStream_t st);
int gbp_neigh_occupancy(size_t smem);
struct Zheng07 {
    double logMmin, sigma, logM0, logM1, alpha;
    // derived on the host once per call (FP64 transcendentals are slow on the GPU)
    double M0, M1, inv_sigma, inv_M1;
};
cudaError_t gbp_launch_zheng07_w(const double *mass, int64_t n, Zheng07 th, double *w,
                                 cudaStream_t st);
cudaError_t gbp_launch_zheng07_vjp(const double *mass, int64_t n, Zheng07 th, const double *gw,
                                   double *out5, cudaStream_t st);
// Single-precision form of one parameter vector for the batched kernels.  The
// per-draw differences log10 M - logMmin and M - M0 are formed from hi + lo
// float splits of both sides: hi - hi is exact when the two lie within a factor
// of 2 (Sterbenz), and the lo parts carry the rest, so the cancellation costs no
// FP64 arithmetic per (halo, draw).
struct Zheng07F {
    float lmin_hi, lmin_lo, m0_hi, m0_lo, inv_sigma, inv_m1, alpha, c2;
};
inline Zheng07F gbp_zheng07_f(const Zheng07 &t) {
    Zheng07F f;
    f.lmin_hi = (float)t.logMmin;
    f.lmin_lo = (float)(t.logMmin - (double)f.lmin_hi);
    f.m0_hi = (float)t.M0;
    f.m0_lo = (float)(t.M0 - (double)f.m0_hi);
    f.inv_sigma = (float)t.inv_sigma;
    f.inv_m1 = (float)t.inv_M1;
    f.alpha = (float)t.alpha;
    f.c2 = (float)(-t.M0 * 2.30258509299404568402 * t.inv_M1);  // d r / d logM0
    return f;
}
// many parameter vectors (th: nth device structs): W (n, nth) and out (nth, 5)
// (hl: n float4 of scratch for the halos' hi + lo splits of log10 M and M)
cudaError_t gbp_launch_zheng07_wb(const double *mass, float4 *hl, int64_t n, const Zheng07F *th,
                                  int nth, double *W, cudaStream_t st);
cudaError_t gbp_launch_zheng07_vjpb(const double *mass, float4 *hl, int64_t n, const Zheng07F *th,
                                    int nth, const double *gW, double *out, cudaStream_t st);
// Zheng07 mocks on the GPU (gbp_hod.cu): thetas as (n, 5) rows converted by
// gbp_hod_thetas into gbp_hod_theta_bytes() each
cudaError_t gbp_hod_count(const double *mass, double *logm, int64_t nh, const void *thetas,
                          int nth, unsigned long long seed, int *count, cudaStream_t st);
cudaError_t gbp_hod_write(const double *xyz, const double *mass, const double *logm,
                          const double *conc, const double *rvir, int64_t nh, const void *thetas,
                          int nth, unsigned long long seed, const int *off, double L, float *gal,
                          cudaStream_t st);
size_t gbp_hod_theta_bytes();
void gbp_hod_thetas(const double *theta, int nth, void *out);
cudaError_t gbp_run_ffma_probe(int nsm, cudaStream_t st, float *ms_out, double *flops_out);
