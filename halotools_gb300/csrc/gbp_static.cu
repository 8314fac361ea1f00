// Allocation-free variant of the npairs_3d pipeline.
//
// Some callers cannot allocate device memory when they count pairs: a
// process whose device memory has been handed to another framework's caching
// allocator (cudaMalloc would fail or fragment it), or a latency-critical
// loop where a cudaMalloc/cudaFree, each of which can synchronise the whole
// device, is not acceptable.  gbp_npairs_3d_static serves them: it runs the
// same cell-list build and count kernels as gbp_npairs_3d, but every scratch
// buffer (sorted positions, cell lists, work items, tables, histogram) lives
// in the file-scope device array below.  It calls no cudaMalloc, cudaFree,
// cudaMallocHost or other allocating routine, device or host.
//
// The array is GBP_STATIC_SCRATCH_BYTES (16 MiB); every GPU that loads
// this library holds it until the process exits.  Limits: at most
// GBP_STATIC_MAX_POINTS points (auto-correlation of one sample), at most 64
// bin edges; larger inputs are rejected with GBP_ERR_INVALID.
//
// The array is shared by every call on a device and keeps the previous call's
// contents; each call clears what must start at zero (cell counts, histogram,
// work cursor, error word) on its own stream.  Calls whose work overlaps on the
// GPU (different streams, or different host threads on one device) race on the
// array and give wrong counts: serialise them.
//
// Each call copies its bin and stencil tables from host stack memory into the
// array; a stream that is being captured would record copies from memory that
// no longer exists when the graph replays, so such a stream is refused.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>

#include "../../include/gbpairs.h"
#include "gbp_host.h"
#include "gbp_internal.cuh"

using namespace gbp;

namespace {

constexpr int64_t SP = GBP_STATIC_MAX_POINTS;
constexpr int64_t SC = GBP_STATIC_MAX_CELLS;
constexpr int SNB = 64;

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
// scratch layout (byte offsets)
constexpr size_t O_CELLID = 0;
constexpr size_t O_RANK = O_CELLID + al(SP * 4);
constexpr size_t O_ORIG = O_RANK + al(SP * 4);
constexpr size_t O_POS32 = O_ORIG + al(SP * 4);
constexpr size_t O_COUNT = O_POS32 + al(2 * SP * 16);
constexpr size_t O_START = O_COUNT + al((SC + 1) * 4);
constexpr size_t O_SCAN = O_START + al((SC + 1) * 4);
constexpr size_t O_ITEMS = O_SCAN + al(4096 * 4);
constexpr int64_t SITEMS = 2 * SC + SP / GBP_TI + 65536;  // work-item capacity
constexpr size_t O_ITMP = O_ITEMS + al(SITEMS * 16);
constexpr size_t O_LUT = O_ITMP + al(2 * (SC + 2) * 4);
constexpr size_t O_E = O_LUT + al(GBP_LUT_MAX * 16);
constexpr size_t O_HI = O_E + al(SNB * 8);
constexpr size_t O_LO = O_HI + al(SNB * 4);
constexpr size_t O_STEN = O_LO + al(SNB * 4);
constexpr size_t O_STEND = O_STEN + al(GBP_STEN_CAP * 4);
constexpr size_t O_HIST = O_STEND + al(GBP_STEN_CAP * 16);
constexpr size_t O_MISC = O_HIST + al((SNB + 1) * 8);
constexpr size_t O_END = O_MISC + al(8 * 8);
static_assert(O_END <= GBP_STATIC_SCRATCH_BYTES, "scratch layout exceeds the static array");

}  // namespace

// The scratch itself.  In host code this name is only a stand-in for the
// device symbol, never a device address: host code gets the address from
// cudaGetSymbolAddress (below) and passes that pointer to the kernels.
static __device__ __align__(256) unsigned char g_gbp_scratch[GBP_STATIC_SCRATCH_BYTES];

namespace {

const int MAX_DEVICES = 64;
// device address per device, looked up once (first calls from several host
// threads may each look it up; they store the same value)
std::atomic<unsigned char *> g_scratch_ptr[MAX_DEVICES];

// Once per device, with that device current: look up the array's address.
// It stays valid for the life of the device's primary context; calls after a
// cudaDeviceReset are not supported.
cudaError_t scratch_for_device(int dev, unsigned char **out) {
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    unsigned char *p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        void *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&q, g_gbp_scratch);
        if (e != cudaSuccess) return e;
        p = static_cast<unsigned char *>(q);
        g_scratch_ptr[dev].store(p, std::memory_order_release);
    }
    *out = p;
    return cudaSuccess;
}

// Cumulative counts from the differential histogram, plus the n self-pairs
// (separation exactly 0) in bin `self_bin`; every count is -1 if the
// digitiser flagged a position outside the box or not finite (misc word 2),
// or the work items overflowed their part of the scratch (misc word 3).
__global__ void k_static_finalize(const unsigned long long *hist, const unsigned long long *misc,
                                  int nb, int self_bin, long long nself, long long *counts) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int err = reinterpret_cast<const int *>(misc)[2] | reinterpret_cast<const int *>(misc)[3];
    long long run = 0;
    for (int k = 0; k < nb; k++) {
        run += (long long)hist[k] + (k == self_bin ? nself : 0);
        counts[k] = err ? -1 : run;
    }
}

}  // namespace

extern "C" int gbp_npairs_3d_static(const double *xyz, int64_t n, const double *rbins,
                                    int32_t nbins, const double *period3, int32_t pbc,
                                    int64_t *counts, void *stream) {
    if (!xyz || !rbins || !period3 || !counts) return GBP_ERR_INVALID;
    if (n < 1 || n > SP) return GBP_ERR_INVALID;           // 1 .. GBP_STATIC_MAX_POINTS points
    if (nbins < 2 || nbins > SNB) return GBP_ERR_INVALID;  // 2 .. 64 edges
    if (pbc != 0 && pbc != 1) return GBP_ERR_INVALID;
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0) || !std::isfinite(period3[d])) return GBP_ERR_INVALID;
    double rmax = max_nan(rbins, nbins);
    double search[3] = {rmax, rmax, rmax};
    for (int d = 0; d < 3; d++) {
        if (!(search[d] <= period3[d] / 3.0)) return GBP_ERR_RANGE;
        if (!(search[d] > 0)) return GBP_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap_status) != cudaSuccess) return GBP_ERR_CUDA;
    if (cap_status != cudaStreamCaptureStatusNone) return GBP_ERR_INVALID;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GBP_ERR_CUDA;
    unsigned char *W = nullptr;
    if (scratch_for_device(dev, &W) != cudaSuccess) return GBP_ERR_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GBP_ERR_CUDA;

    // host planning on fixed storage (no heap)
    Geometry g;
    int64_t cap = 1;
    while ((cap + 1) * (cap + 1) * (cap + 1) <= SC) cap++;
    choose_grid(g, period3, search, pbc, n, 0, cap);
    build_stencil(g, search, 0, true);
    ErrModel em = err_model(g);
    double E[SNB];
    float hi[SNB], lo[SNB];
    float4 lut[GBP_LUT_MAX];  // 32 KB of stack
    edges_top_walk(rbins, nbins, E);
    thresholds(nbins, E, &em, 3, hi, lo);
    LutInfo li = build_lut(nbins, hi, lo, no_qband, lut);
    const int self_bin = host_bin(nbins, E, 0.0);

    // tables: pageable sources are staged by the driver before the call returns
    cudaError_t e = cudaMemcpyAsync(W + O_LUT, lut, sizeof(float4) * li.T, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(W + O_E, E, sizeof(double) * nbins, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(W + O_HI, hi, sizeof(float) * nbins, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(W + O_LO, lo, sizeof(float) * nbins, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(W + O_STEN, g.sten, sizeof(int) * g.nsten, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(W + O_STEND, g.stenD, sizeof(float4) * g.nsten, cudaMemcpyHostToDevice, st);
    // what must start at zero: histogram, work cursor, item count, error word, stats
    if (e == cudaSuccess) e = cudaMemsetAsync(W + O_HIST, 0, (SNB + 1) * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(W + O_MISC, 0, 8 * 8, st);
    if (e != cudaSuccess) return GBP_ERR_CUDA;

    int *misc_i = reinterpret_cast<int *>(W + O_MISC);
    unsigned long long *misc = reinterpret_cast<unsigned long long *>(W + O_MISC);
    MeshDev md;
    md.bf = g.bf;
    for (int d = 0; d < 3; d++) {
        md.n[d] = g.n[d];
        md.nb[d] = g.nb[d];
        md.c[d] = g.c[d];
        md.inv_c[d] = 1.0 / g.c[d]; md.inv_cf[d] = (float)(1.0 / g.c[d]);
        md.Lf[d] = f_down(g.L[d]);
        md.L[d] = g.L[d];
    }
    md.ncells = g.ncells;
    md.offsets = nullptr;
    md.nmocks = 1;
    float4 *pos32 = reinterpret_cast<float4 *>(W + O_POS32);
    int *start = reinterpret_cast<int *>(W + O_START);
    e = gbp_build_cells(xyz, 0, n, md, reinterpret_cast<int *>(W + O_CELLID),
                        reinterpret_cast<int *>(W + O_RANK), reinterpret_cast<int *>(W + O_COUNT),
                        start, reinterpret_cast<int *>(W + O_SCAN), pos32,
                        reinterpret_cast<int *>(W + O_ORIG), nullptr, 0, nullptr, nullptr,
                        misc_i + 2, st, nullptr);
    if (e != cudaSuccess) return GBP_ERR_CUDA;
    ItemPlan ip;
    ip.start1 = ip.start2 = start;
    ip.nkeys = g.nblocks;
    ip.ncm = (int)g.nblocks;
    ip.bf3 = g.bf * g.bf * g.bf;
    for (int d = 0; d < 3; d++) ip.n[d] = g.nb[d];
    ip.pbc = g.pbc;
    ip.sten = reinterpret_cast<const int *>(W + O_STEN);
    ip.stenD = reinterpret_cast<const float4 *>(W + O_STEND);
    ip.nsten = g.nsten;
    ip.jcap = GBP_JCAP_ITEM;
    // item capacity: every item holds >= 1 i-point and a group of >= 1 stencil
    // entry or >= GBP_JCAP_ITEM j-points, so chunks x groups stays within this
    e = gbp_build_items(ip, reinterpret_cast<int4 *>(W + O_ITEMS), (int)SITEMS, misc_i + 1,
                        misc_i + 3, reinterpret_cast<int *>(W + O_ITMP),
                        reinterpret_cast<int *>(W + O_SCAN), st, nullptr);
    if (e != cudaSuccess) return GBP_ERR_CUDA;

    CountArgs a;
    std::memset(&a, 0, sizeof(a));
    a.pos1 = a.pos2 = pos32;
    a.xyz1 = a.xyz2 = xyz;
    a.err = misc_i + 2;
    a.orig1 = a.orig2 = reinterpret_cast<const int *>(W + O_ORIG);
    a.start2 = start;
    a.items = reinterpret_cast<const int4 *>(W + O_ITEMS);
    a.nitems = misc_i + 1;
    a.counter = misc_i;
    a.sten = reinterpret_cast<const int *>(W + O_STEN);
    a.stenD = reinterpret_cast<const float4 *>(W + O_STEND);
    a.nsten = g.nsten;
    a.nself = g.nself;
    for (int d = 0; d < 3; d++) {
        a.n[d] = g.nb[d];
        a.L[d] = g.L[d];
    }
    a.bf3 = g.bf * g.bf * g.bf;
    a.pbc = g.pbc;
    AxisDev &ad = a.ax[0];
    ad.lut = reinterpret_cast<const float4 *>(W + O_LUT);
    ad.E = reinterpret_cast<const double *>(W + O_E);
    ad.hi = reinterpret_cast<const float *>(W + O_HI);
    ad.lo = reinterpret_cast<const float *>(W + O_LO);
    ad.nb = nbins;
    ad.T = li.T;
    ad.S = li.S;
    ad.B = li.B;
    ad.vlo = li.vlo;
    ad.vhi = li.vhi;
    a.hist_stride = nbins + 1;
    a.hist_copies = GBP_WARPS;  // as gbp_npairs_3d; MODE_3D keeps lane-private counts
    a.ncells_mock = (int)g.nblocks;
    a.flush_after = 1ull << 24;
    a.hist = reinterpret_cast<unsigned long long *>(W + O_HIST);
    a.nrecheck = misc + 2;
    a.top0 = std::min(hi[nbins - 1], 1.0e30f);
    a.self_bin = self_bin;
    SmemLayout L = gbp_smem_layout(MODE_3D, li.T, 0, nbins, 0, g.nsten, a.hist_copies, 0);
    size_t smem = (size_t)L.total;
    int occ = gbp_count_occupancy(MODE_3D, 1, smem);
    if (occ <= 0) return GBP_ERR_INVALID;
    e = gbp_launch_count(MODE_3D, 1, a, nsm * occ, smem, st);
    if (e != cudaSuccess) return GBP_ERR_CUDA;
    k_static_finalize<<<1, 32, 0, st>>>(a.hist, misc, nbins, self_bin, (long long)n,
                                        reinterpret_cast<long long *>(counts));
    return cudaGetLastError() == cudaSuccess ? GBP_OK : GBP_ERR_CUDA;
}
