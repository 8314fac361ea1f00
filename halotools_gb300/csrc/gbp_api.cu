// C-ABI of the gbpairs library: plans, argument checks, grid and stencil
// choice, edge thresholds, device workspace and the per-call pipeline
//   H2D positions -> cell lists (gbp_mesh.cu) -> work items -> count kernel
//   (gbp_count.cu) -> D2H differential histogram -> cumulative counts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/gbpairs.h"
#include "gbp_host.h"
#include "gbp_internal.cuh"

using namespace gbp;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct gbp_plan {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    int reach = 0;
    int block = 0;         // forced block factor of the two-level grid, 0 = automatic
    int nsm = 0;
    DevBuf work;           // device workspace, grow-only
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool graph_mode = false;          // capture each call into a CUDA graph and replay it
    bool autotune = false;            // time the feasible reaches on a new workload shape
    size_t item_cap = 0;              // work-item capacity learned from an overflow
    size_t first_item_cap = 0;        // gbp_plan_set_limits: room for the next call's items
    unsigned long long flush_after = 1ull << 24;  // gbp_plan_set_limits: early histogram flush
    std::vector<std::pair<std::string, int>> tuned;  // workload signature -> best reach
    cudaGraphExec_t gexec = nullptr;  // reused (updated in place) across calls
    gbp_stats stats;
    std::string err;
};

namespace {

int fail(gbp_plan *p, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (p) p->err = buf;
    return code;
}

#define CK(expr)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(plan, e_ == cudaErrorMemoryAllocation ? GBP_ERR_NOMEM : GBP_ERR_CUDA, \
                        "%s: %s", #expr, cudaGetErrorString(e_));                         \
    } while (0)

// ---------------- workspace ----------------
struct Carve {
    size_t off = 0;
    template <class T>
    size_t take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        size_t o = off;
        off += count * sizeof(T);
        return o;
    }
};

int ensure_work(gbp_plan *plan, size_t bytes) {
    if (plan->work.bytes >= bytes) return GBP_OK;
    if (plan->work.p) cudaFree(plan->work.p);
    plan->work.p = nullptr;
    plan->work.bytes = 0;
    size_t want = std::max(bytes, plan->work.bytes + plan->work.bytes / 4);
    CK(cudaMalloc(&plan->work.p, want));
    plan->work.bytes = want;
    return GBP_OK;
}

int ensure_pinned(gbp_plan *plan, size_t bytes) {
    if (plan->pinned_bytes >= bytes) return GBP_OK;
    if (plan->pinned) cudaFreeHost(plan->pinned);
    plan->pinned = nullptr;
    plan->pinned_bytes = 0;
    CK(cudaMallocHost(&plan->pinned, bytes));
    plan->pinned_bytes = bytes;
    return GBP_OK;
}

// one binning axis, vector-backed (up to GBP_NB_MAX edges)
struct AxisHost {
    int nb = 0;
    std::vector<double> E;
    std::vector<float> hi, lo;
    std::vector<float4> lut;
    int T = 0, S = 0, B = 0;
    float vlo = 0, vhi = 0;
    void set(const std::vector<double> &Ein, const ErrModel *em, int m) {
        nb = (int)Ein.size();
        E = Ein;
        hi.assign(nb, 0.f);
        lo.assign(nb, 0.f);
        thresholds(nb, E.data(), em, m, hi.data(), lo.data());
    }
    template <class QB>
    void make_lut(QB q) {
        lut.resize(GBP_LUT_MAX);
        LutInfo i = build_lut(nb, hi.data(), lo.data(), q, lut.data());
        T = i.T;
        S = i.S;
        B = i.B;
        vlo = i.vlo;
        vhi = i.vhi;
        lut.resize(T);
    }
};

struct SampleDev {
    const double *xyz = nullptr;
    int *cellid, *rank, *count, *start, *orig;
    float4 *pos32;
    float *w32 = nullptr;
    double *w64 = nullptr;
};

struct Call {
    int mode;
    int wf = 1;  // marking-function template for MODE_MARK
    int nmocks = 1;                  // batched auto-correlations of mocks (sample 1 only)
    std::vector<int64_t> offsets;    // nmocks+1 point offsets when nmocks > 1
    int xyz_f32 = 0;                 // sample 1 positions are float32
    std::vector<float> gt;           // adjoint: suffix sums of the upstream gradient (nb+1)
    int ntag = 0;                    // jackknife: tags 0..ntag-1 (N_samples + 1)
    std::vector<unsigned long long> htag;  // jackknife: (ntag, nb+1) pair ends by tag
    std::vector<unsigned> pobj;      // per-object: (n1, nb+1) differential counts, caller's order
    double *grad_out = nullptr;      // adjoint: dL/dw, caller's order, in `mem` memory
    // per-object neighbours: geometry, separation > 0, condition, output kind
    int ngeo = 0, nexcl0 = 0, ncond = 0, nout = 0;
    double ncpar[2] = {0, 0};
    int nceq[2] = {0, 0};
    std::vector<long long> poff;     // pair list: first slot per caller-order sample-1 point
    int64_t npairs = 0;              // pair list: total slots
    uint32_t *pairs_out = nullptr;   // pair list: (i1, i2) per slot, host memory
    const double *xyz1, *xyz2;
    int64_t n1, n2;
    bool autocorr;
    int mem;
    const double *w1 = nullptr, *w2 = nullptr;
    int nw = 0, wfunc = 0;
    AxisHost ax[2];
    int naxes;
    Geometry g;
};

template <class T>
T *at(void *base, size_t off) {
    return reinterpret_cast<T *>(static_cast<char *>(base) + off);
}

// The count kernels skip (i, i) in auto mode; the reference computes
// dx = (x - 0) - x = 0 for it, so it lands in the bins of v = 0.
void add_self_pairs(const Call &c, std::vector<unsigned long long> &h) {
    if (!c.autocorr) return;
    int a = host_bin(c.ax[0].nb, c.ax[0].E.data(), 0.0);
    if (a >= c.ax[0].nb) return;
    size_t idx = (size_t)a;
    size_t nh = (size_t)(c.ax[0].nb + 1);
    if (c.naxes > 1) {
        int b = host_bin(c.ax[1].nb, c.ax[1].E.data(), 0.0);
        if (b >= c.ax[1].nb) return;
        idx = (size_t)a * (c.ax[1].nb + 1) + b;
        nh *= (size_t)(c.ax[1].nb + 1);
    }
    for (int m = 0; m < c.nmocks; m++) {
        int64_t n = c.nmocks > 1 ? c.offsets[m + 1] - c.offsets[m] : c.n1;
        h[m * nh + idx] += (unsigned long long)n;
    }
}

// Runs the pipeline; fills hist_host with the differential histogram
// ((nb0+1) x (nb1+1) u64).
int run_call(gbp_plan *plan, Call &c, std::vector<unsigned long long> &hist_host,
             std::vector<double> *histd_host = nullptr) {
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    std::memset(&plan->stats, 0, sizeof(plan->stats));
    const int64_t ncells = c.g.ncells;
    const int nm = c.nmocks;
    const int64_t nkeys = ncells * nm;  // cell keys: mock * ncells + cell
    const int nb0 = c.ax[0].nb, nb1 = c.naxes > 1 ? c.ax[1].nb : 0;
    const int T0 = c.ax[0].T, T1 = c.naxes > 1 ? c.ax[1].T : 0;
    const int nsten = c.g.nsten;
    // MARKC: one (nb0 + 1) histogram per mark channel
    const size_t nhist = (size_t)(nb0 + 1) * (size_t)(c.naxes > 1 ? nb1 + 1 : 1) *
                         (size_t)(c.mode == MODE_MARKC ? c.nw : 1);
    const int nsamp = c.autocorr ? 1 : 2;
    const int64_t ns[2] = {c.n1, c.n2};

    // ---- carve the workspace ----
    Carve cv;
    size_t o_xyz[2] = {0, 0}, o_cellid[2], o_rank[2], o_count[2], o_start[2], o_orig[2],
           o_pos32[2], o_w32[2] = {0, 0}, o_w64[2] = {0, 0}, o_win[2] = {0, 0};
    // sorted FP64 weights: only the FP64 marking functions and the per-object
    // neighbour conditions read them; the FP32 kernels read the FP32 copy
    const bool need_w64 = c.mode == MODE_NEIGH ||
                          (c.wf == 0 && (c.mode == MODE_MARK || c.mode == MODE_XYZW ||
                                         c.mode == MODE_SMUW));
    for (int s = 0; s < nsamp; s++) {
        size_t n = (size_t)std::max<int64_t>(ns[s], 1);
        if (c.mem == GBP_MEM_HOST) o_xyz[s] = cv.take<double>(3 * n);
        o_cellid[s] = cv.take<int>(n);
        o_rank[s] = cv.take<int>(n);
        o_count[s] = cv.take<int>((size_t)nkeys + 1);
        o_start[s] = cv.take<int>((size_t)nkeys + 1);
        o_orig[s] = cv.take<int>(n);
        o_pos32[s] = cv.take<float4>(2 * n);
        if (c.nw > 0) {
            if (c.mem == GBP_MEM_HOST) o_win[s] = cv.take<double>(n * c.nw);
            o_w32[s] = cv.take<float>(n * c.nw);
            if (need_w64) o_w64[s] = cv.take<double>(n * c.nw);
        }
    }
    size_t scan_ints = gbp_scan_tmp_ints(nkeys + 1);
    size_t o_scan = cv.take<int>(scan_ints);
    // work items: i-chunks of GBP_TI times stencil groups of <= GBP_JCAP_ITEM
    // j-points; the builder flags an overflow and the call is repeated larger
    // the 16-channel adjoint holds one point per lane: items of 32
    const int item_ti = (c.mode == MODE_ADJC && c.nw > GBP_ADJ_CH) ? 32 : GBP_TI;
    size_t max_items = std::max<size_t>(
        plan->item_cap,
        2 * ((size_t)nkeys + (size_t)(c.n1 / item_ti)) +
            (size_t)nsten * (size_t)(c.n2 / GBP_JCAP_ITEM) + 65536);
    if (plan->first_item_cap) {
        max_items = plan->first_item_cap;  // once: an overflow sets item_cap for the retry
        plan->first_item_cap = 0;
    }
    size_t o_items = cv.take<int4>(max_items);
    size_t o_itmp = cv.take<int>(2 * ((size_t)nkeys + 2));
    size_t o_offs = cv.take<int64_t>((size_t)nm + 1);
    const bool adjc = c.mode == MODE_ADJC;  // several weight channels
    const bool adj = c.mode == MODE_ADJ || adjc;
    const size_t ngrad = (size_t)c.n1 * (size_t)(adjc ? c.nw : 1);  // dL/dw entries
    const size_t ngt = adj ? c.gt.size() : (size_t)nb0 + 1;         // gradient-table floats
    const bool pobj = c.mode == MODE_POBJ;
    const bool neigh = c.mode == MODE_NEIGH;
    const size_t npobj = pobj ? (size_t)c.n1 * (size_t)(nb0 + 1) : neigh ? (size_t)c.n1 : 0;
    const bool plist = neigh && c.nout == 2;
    size_t o_nthr = cv.take<float4>(neigh ? (size_t)std::max<int64_t>(c.n1, 1) : 1);
    size_t o_poff = cv.take<long long>(plist ? (size_t)c.n1 + 1 : 1);
    size_t o_pcur = cv.take<unsigned>(plist ? (size_t)std::max<int64_t>(c.n1, 1) : 1);
    size_t o_pairs = cv.take<unsigned>(plist ? 2 * (size_t)std::max<int64_t>(c.npairs, 1) : 1);
    size_t o_gt = cv.take<float>(std::max<size_t>(ngt, 1));
    size_t o_grad = cv.take<double>(adj && c.mem == GBP_MEM_HOST ? std::max<size_t>(ngrad, 1) : 1);
    size_t o_pobj = cv.take<unsigned>(npobj > 0 ? npobj : 1);
    size_t o_lut0 = cv.take<float4>(T0), o_lut1 = cv.take<float4>(std::max(T1, 1));
    size_t o_E0 = cv.take<double>(nb0), o_E1 = cv.take<double>(std::max(nb1, 1));
    size_t o_hi0 = cv.take<float>(nb0), o_lo0 = cv.take<float>(nb0);
    size_t o_hi1 = cv.take<float>(std::max(nb1, 1)), o_lo1 = cv.take<float>(std::max(nb1, 1));
    size_t o_sten = cv.take<int>(nsten), o_stenD = cv.take<float4>(nsten);
    size_t o_hist = cv.take<unsigned long long>(nhist * nm);
    size_t o_histd = cv.take<double>(nhist * nm);
    // jackknife: (tag, bin) pair ends over the 1-D or 2-D differential bins
    const size_t ntab = (size_t)c.ntag * (size_t)(nb0 + 1) * (size_t)(c.naxes > 1 ? nb1 + 1 : 1);
    size_t o_htag = cv.take<unsigned long long>(ntab > 0 ? ntab : 1);
    size_t o_misc = cv.take<unsigned long long>(8);  // counter, nitems, err, recheck, cand
    size_t total = cv.take<char>(0) + 256;
    int rc = ensure_work(plan, total);
    if (rc) return rc;
    void *W = plan->work.p;

    // ---- small tables through one pinned upload ----
    Carve hv;
    size_t h_lut0 = hv.take<float4>(T0), h_lut1 = hv.take<float4>(std::max(T1, 1));
    size_t h_E0 = hv.take<double>(nb0), h_E1 = hv.take<double>(std::max(nb1, 1));
    size_t h_hi0 = hv.take<float>(nb0), h_lo0 = hv.take<float>(nb0);
    size_t h_hi1 = hv.take<float>(std::max(nb1, 1)), h_lo1 = hv.take<float>(std::max(nb1, 1));
    size_t h_sten = hv.take<int>(nsten), h_stenD = hv.take<float4>(nsten);
    size_t h_offs = hv.take<int64_t>((size_t)nm + 1);
    size_t h_gt = hv.take<float>(std::max<size_t>(ngt, 1));
    size_t h_end = hv.take<char>(0);
    size_t h_hist = hv.take<unsigned long long>(nhist * nm);
    size_t h_histd = hv.take<double>(nhist * nm);
    size_t h_htag = hv.take<unsigned long long>(ntab > 0 ? ntab : 1);
    size_t h_misc = hv.take<unsigned long long>(8);
    rc = ensure_pinned(plan, hv.take<char>(0) + 256);
    if (rc) return rc;
    void *H = plan->pinned;
    std::memcpy(at<char>(H, h_lut0), c.ax[0].lut.data(), sizeof(float4) * T0);
    std::memcpy(at<char>(H, h_E0), c.ax[0].E.data(), sizeof(double) * nb0);
    std::memcpy(at<char>(H, h_hi0), c.ax[0].hi.data(), sizeof(float) * nb0);
    std::memcpy(at<char>(H, h_lo0), c.ax[0].lo.data(), sizeof(float) * nb0);
    if (c.naxes > 1) {
        std::memcpy(at<char>(H, h_lut1), c.ax[1].lut.data(), sizeof(float4) * T1);
        std::memcpy(at<char>(H, h_E1), c.ax[1].E.data(), sizeof(double) * nb1);
        std::memcpy(at<char>(H, h_hi1), c.ax[1].hi.data(), sizeof(float) * nb1);
        std::memcpy(at<char>(H, h_lo1), c.ax[1].lo.data(), sizeof(float) * nb1);
    }
    std::memcpy(at<char>(H, h_sten), c.g.sten, sizeof(int) * nsten);
    std::memcpy(at<char>(H, h_stenD), c.g.stenD, sizeof(float4) * nsten);
    if (nm > 1) std::memcpy(at<char>(H, h_offs), c.offsets.data(), sizeof(int64_t) * (nm + 1));
    if (adj) std::memcpy(at<char>(H, h_gt), c.gt.data(), sizeof(float) * ngt);

    int launches = 0;
    int64_t h2d = 0, d2h = 0;
    const bool graph = plan->graph_mode;
    // event records inside a capture must be external to be timed on replay
    auto rec = [&](cudaEvent_t ev) {
        return graph ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                     : cudaEventRecord(ev, st);
    };
    // every stream operation of the call, from the table uploads to the result
    // copies: run directly, or captured into one CUDA graph and replayed
    auto enqueue = [&]() -> int {
        CK(rec(plan->ev[0]));
        h2d += (int64_t)(sizeof(float4) * (T0 + T1) + sizeof(double) * (nb0 + nb1) +
                         sizeof(float) * 2 * (nb0 + nb1) + (sizeof(int) + sizeof(float4)) * nsten);
        CK(cudaMemcpyAsync(at<char>(W, o_lut0), at<char>(H, h_lut0), sizeof(float4) * T0, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(at<char>(W, o_E0), at<char>(H, h_E0), sizeof(double) * nb0, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(at<char>(W, o_hi0), at<char>(H, h_hi0), sizeof(float) * nb0, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(at<char>(W, o_lo0), at<char>(H, h_lo0), sizeof(float) * nb0, cudaMemcpyHostToDevice, st));
        if (c.naxes > 1) {
            CK(cudaMemcpyAsync(at<char>(W, o_lut1), at<char>(H, h_lut1), sizeof(float4) * T1, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(at<char>(W, o_E1), at<char>(H, h_E1), sizeof(double) * nb1, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(at<char>(W, o_hi1), at<char>(H, h_hi1), sizeof(float) * nb1, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(at<char>(W, o_lo1), at<char>(H, h_lo1), sizeof(float) * nb1, cudaMemcpyHostToDevice, st));
        }
        CK(cudaMemcpyAsync(at<char>(W, o_sten), at<char>(H, h_sten), sizeof(int) * nsten, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(at<char>(W, o_stenD), at<char>(H, h_stenD), sizeof(float4) * nsten, cudaMemcpyHostToDevice, st));
        if (adj) {
            CK(cudaMemcpyAsync(at<char>(W, o_gt), at<char>(H, h_gt), sizeof(float) * ngt, cudaMemcpyHostToDevice, st));
            h2d += (int64_t)(sizeof(float) * ngt);
        }
        if (nm > 1) {
            CK(cudaMemcpyAsync(at<char>(W, o_offs), at<char>(H, h_offs), sizeof(int64_t) * (nm + 1), cudaMemcpyHostToDevice, st));
            h2d += (int64_t)(sizeof(int64_t) * (nm + 1));
        }
        (void)h_end;

        // ---- positions and weights ----
        SampleDev sd[2];
        for (int s = 0; s < nsamp; s++) {
            const double *src = s == 0 ? c.xyz1 : c.xyz2;
            const double *wsrc = s == 0 ? c.w1 : c.w2;
            size_t n = (size_t)ns[s];
            const size_t esz = (s == 0 && c.xyz_f32) ? sizeof(float) : sizeof(double);
            if (c.mem == GBP_MEM_HOST) {
                sd[s].xyz = at<double>(W, o_xyz[s]);
                if (n) CK(cudaMemcpyAsync((void *)sd[s].xyz, src, 3 * n * esz, cudaMemcpyHostToDevice, st));
                h2d += (int64_t)(3 * n * esz);
            } else {
                sd[s].xyz = src;
            }
            sd[s].cellid = at<int>(W, o_cellid[s]);
            sd[s].rank = at<int>(W, o_rank[s]);
            sd[s].count = at<int>(W, o_count[s]);
            sd[s].start = at<int>(W, o_start[s]);
            sd[s].orig = at<int>(W, o_orig[s]);
            sd[s].pos32 = at<float4>(W, o_pos32[s]);
            if (c.nw > 0) {
                const double *wd = wsrc;
                if (c.mem == GBP_MEM_HOST) {
                    wd = at<double>(W, o_win[s]);
                    if (n) CK(cudaMemcpyAsync((void *)wd, wsrc, n * c.nw * sizeof(double), cudaMemcpyHostToDevice, st));
                    h2d += (int64_t)(n * c.nw * sizeof(double));
                }
                sd[s].w32 = at<float>(W, o_w32[s]);
                sd[s].w64 = need_w64 ? at<double>(W, o_w64[s]) : nullptr;
                wsrc = wd;
            }
            if (s == 0) c.w1 = wsrc; else c.w2 = wsrc;
        }
        unsigned long long *misc = at<unsigned long long>(W, o_misc);
        CK(cudaMemsetAsync(misc, 0, 8 * sizeof(unsigned long long), st));
        int *d_counter = reinterpret_cast<int *>(misc);
        int *d_nitems = reinterpret_cast<int *>(misc) + 1;
        int *d_err = reinterpret_cast<int *>(misc) + 2;
        unsigned long long *d_stat = misc + 2;  // [0] rechecks, [1] candidate pairs

        MeshDev md;
        md.bf = c.g.bf;
        for (int d = 0; d < 3; d++) {
            md.n[d] = c.g.n[d];
            md.nb[d] = c.g.nb[d];
            md.c[d] = c.g.c[d];
            md.inv_c[d] = 1.0 / c.g.c[d]; md.inv_cf[d] = (float)(1.0 / c.g.c[d]);
            md.Lf[d] = f_down(c.g.L[d]);
            md.L[d] = c.g.L[d];
        }
        md.ncells = ncells;
        md.offsets = nm > 1 ? at<int64_t>(W, o_offs) : nullptr;
        md.nmocks = nm;
        for (int s = 0; s < nsamp; s++) {
            const double *wsrc = s == 0 ? c.w1 : c.w2;
            cudaError_t e = gbp_build_cells(sd[s].xyz, s == 0 ? c.xyz_f32 : 0, ns[s], md, sd[s].cellid, sd[s].rank, sd[s].count,
                                            sd[s].start, at<int>(W, o_scan), sd[s].pos32,
                                            sd[s].orig, c.nw > 0 ? wsrc : nullptr, c.nw, sd[s].w32,
                                            sd[s].w64, d_err, st, &launches);
            CK(e);
        }
        ItemPlan ip;
        ip.start1 = sd[0].start;
        ip.start2 = (c.autocorr ? sd[0] : sd[1]).start;
        ip.nkeys = c.g.nblocks * nm;
        ip.ncm = (int)c.g.nblocks;
        ip.bf3 = c.g.bf * c.g.bf * c.g.bf;
        for (int d = 0; d < 3; d++) ip.n[d] = c.g.nb[d];
        ip.pbc = c.g.pbc;
        ip.sten = at<int>(W, o_sten);
        ip.stenD = at<float4>(W, o_stenD);
        ip.nsten = nsten;
        ip.jcap = GBP_JCAP_ITEM;
        ip.ti = item_ti;
        CK(gbp_build_items(ip, at<int4>(W, o_items), (int)std::min<size_t>(max_items, INT32_MAX),
                           d_nitems, reinterpret_cast<int *>(misc) + 3, at<int>(W, o_itmp),
                           at<int>(W, o_scan), st, &launches));
        CK(cudaMemsetAsync(at<char>(W, o_hist), 0, nm * nhist * sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(at<char>(W, o_histd), 0, nm * nhist * sizeof(double), st));
        if (ntab) CK(cudaMemsetAsync(at<char>(W, o_htag), 0, ntab * sizeof(unsigned long long), st));
        CK(rec(plan->ev[1]));

        const SampleDev &s2 = c.autocorr ? sd[0] : sd[1];
        CountArgs a;
        std::memset(&a, 0, sizeof(a));
        a.pos1 = sd[0].pos32;
        a.pos2 = s2.pos32;
        a.xyz1 = sd[0].xyz;
        a.xyz2 = s2.xyz;
        a.xyz1_f32 = c.xyz_f32;
        a.xyz2_f32 = c.autocorr ? c.xyz_f32 : 0;
        a.orig1 = sd[0].orig;
        a.orig2 = s2.orig;
        a.start2 = s2.start;
        a.items = at<int4>(W, o_items);
        a.nitems = d_nitems;
        a.counter = d_counter;
        a.flush_after = plan->flush_after;
        a.sten = at<int>(W, o_sten);
        a.stenD = at<float4>(W, o_stenD);
        a.nsten = nsten;
        a.nself = c.g.nself;
        for (int d = 0; d < 3; d++) {
            a.n[d] = c.g.nb[d];
            a.L[d] = c.g.L[d];
        }
        a.bf3 = c.g.bf * c.g.bf * c.g.bf;
        a.pbc = c.g.pbc;
        for (int x = 0; x < c.naxes; x++) {
            AxisDev &ad = a.ax[x];
            const AxisHost &ah = c.ax[x];
            ad.lut = at<float4>(W, x == 0 ? o_lut0 : o_lut1);
            ad.E = at<double>(W, x == 0 ? o_E0 : o_E1);
            ad.hi = at<float>(W, x == 0 ? o_hi0 : o_hi1);
            ad.lo = at<float>(W, x == 0 ? o_lo0 : o_lo1);
            ad.nb = ah.nb;
            ad.T = ah.T;
            ad.S = ah.S;
            ad.B = ah.B;
            ad.vlo = ah.vlo;
            ad.vhi = ah.vhi;
        }
        a.hist_stride = (int)nhist;
        a.ncells_mock = (int)c.g.nblocks;
        a.hist = at<unsigned long long>(W, o_hist);
        a.histd = at<double>(W, o_histd);
        a.htag = at<unsigned long long>(W, o_htag);
        a.ntag = c.ntag;
        a.nrecheck = d_stat;
        a.w1 = sd[0].w32;
        a.w2 = s2.w32;
        a.w64_1 = sd[0].w64;
        a.w64_2 = s2.w64;
        a.nw = c.nw;
        a.wfunc = c.wfunc;

        a.top0 = std::min(c.ax[0].hi[nb0 - 1], 1.0e30f);
        a.top1 = c.naxes > 1 ? std::min(c.ax[1].hi[nb1 - 1], 1.0e30f) : 0.f;
        a.self_bin = host_bin(nb0, c.ax[0].E.data(), 0.0);
        const bool jw = c.mode == MODE_JACKW || c.mode == MODE_JACKXYZW;
        const bool w2 = c.mode == MODE_XYZW || c.mode == MODE_SMUW || jw;
        if (w2) {
            // the flat (axis 0, axis 1) bin of separation 0, or -1 when outside
            const int sb1 = c.naxes > 1 ? host_bin(nb1, c.ax[1].E.data(), 0.0) : 0;
            const int ok = a.self_bin < nb0 && (c.naxes == 1 || sb1 < nb1);
            a.self_bin = ok ? a.self_bin * (c.naxes > 1 ? nb1 + 1 : 1) + sb1 : -1;
        }
        const int jwb = jw ? 4 * c.nw   // {w, tag} columns
                        : (c.mode == MODE_MARK || w2) ? (c.wf == 0 ? 8 * c.nw : 4)
                        : c.mode == MODE_MARKC ? 4 * gbp_markc_cols(c.nw)
                        : c.mode == MODE_ADJ   ? 4
                        : c.mode == MODE_ADJC  ? 4 * gbp_adjc_nch(c.nw)  // the kernel's fixed stride
                        : c.mode == MODE_POBJ  ? 4   // the gather kernel's fixed stride
                        : (c.mode == MODE_JACK || c.mode == MODE_JACKXYZ) ? 4
                        : neigh                ? 4   // the j-slots' sorted indices
                                               : 0;
        // 2-D and wide 1-D histograms: one shared copy per warp while they fit,
        // else the warps add straight into the global histogram
        int copies = GBP_WARPS;
        if (c.mode != MODE_3D && c.mode != MODE_MARK && c.mode != MODE_MARKC && c.mode != MODE_ADJ &&
            c.mode != MODE_JACK && c.mode != MODE_POBJ) {
            size_t one = (size_t)(nb0 + 1) * (size_t)(c.naxes > 1 ? nb1 + 1 : 1) * 4;
            if (one * GBP_WARPS > (96u << 10)) copies = 0;
        }
        if (c.mode == MODE_XYZW || c.mode == MODE_JACKW || c.mode == MODE_JACKXYZW)
            copies = 0;  // sums only: no integer counts
        a.hist_copies = copies;
        SmemLayout L = gbp_smem_layout(c.mode, T0, T1, nb0, nb1, nsten, copies, jwb, c.ntag);
        size_t smem = (size_t)L.total;
        if (smem > (size_t)(227u << 10))
            return fail(plan, GBP_ERR_INVALID, "too many bins for one shared-memory histogram (%zu B)", smem);
        a.gt = at<float>(W, o_gt);
        a.orig = sd[0].orig;
        a.grad = adj ? (c.mem == GBP_MEM_HOST ? at<double>(W, o_grad) : c.grad_out) : nullptr;
        a.pobj = at<unsigned>(W, o_pobj);
        a.err = d_err;
        if (neigh) {
            ErrModel em = err_model(c.g);
            a.nthr = at<float4>(W, o_nthr);
            a.nerr[0] = em.cmax;
            a.nerr[1] = em.K;
            a.nerr[2] = em.Lmax;
            a.ngeo = c.ngeo;
            a.nexcl0 = c.nexcl0;
            a.ncond = c.ncond;
            a.ncpar[0] = c.ncpar[0];
            a.ncpar[1] = c.ncpar[1];
            a.nceq[0] = c.nceq[0];
            a.nceq[1] = c.nceq[1];
            a.same = c.autocorr ? 1 : 0;
            if (plist) {
                a.poff = at<long long>(W, o_poff);
                a.pcur = at<unsigned>(W, o_pcur);
                a.pairs = at<unsigned>(W, o_pairs);
                CK(cudaMemcpyAsync((void *)a.poff, c.poff.data(), sizeof(long long) * (c.n1 + 1),
                                   cudaMemcpyHostToDevice, st));
                CK(cudaMemsetAsync(a.pcur, 0, sizeof(unsigned) * c.n1, st));
                h2d += (int64_t)(sizeof(long long) * (c.n1 + 1));
            }
        }
        int occ = adjc            ? gbp_adjoint_ch_occupancy(smem, c.nw)
                  : (adj || pobj) ? gbp_adjoint_occupancy(smem, pobj)
                  : neigh       ? gbp_neigh_occupancy(smem)
                                : gbp_count_occupancy(c.mode, c.wf, smem);
        if (occ <= 0) return fail(plan, GBP_ERR_INVALID, "count kernel does not fit (smem %zu B)", smem);
        int grid = plan->nsm * occ;
        if (adj) CK(cudaMemsetAsync(a.grad, 0, sizeof(double) * ngrad, st));
        if (pobj || neigh) CK(cudaMemsetAsync(a.pobj, 0, sizeof(unsigned) * npobj, st));
        if (adjc) CK(gbp_launch_adjoint_ch(a, grid, smem, st));
        else if (adj || pobj) CK(gbp_launch_adjoint(a, grid, smem, st, pobj));
        else if (neigh) CK(gbp_launch_neigh(a, (int)c.n1, c.nout, grid, smem, st));
        else CK(gbp_launch_count(c.mode, c.wf, a, grid, smem, st));
        if (adj && c.mem == GBP_MEM_HOST && c.n1 > 0) {
            CK(cudaMemcpyAsync(c.grad_out, a.grad, sizeof(double) * ngrad, cudaMemcpyDeviceToHost, st));
            d2h += (int64_t)(sizeof(double) * ngrad);
        }
        if (plist && c.npairs > 0) {
            CK(cudaMemcpyAsync(c.pairs_out, a.pairs, 2 * sizeof(unsigned) * (size_t)c.npairs,
                               cudaMemcpyDeviceToHost, st));
            d2h += (int64_t)(2 * sizeof(unsigned) * (size_t)c.npairs);
        }
        if ((pobj || (neigh && !plist)) && npobj) {
            // (the caller sized c.pobj; a pageable copy, the call syncs at the end anyway)
            CK(cudaMemcpyAsync(c.pobj.data(), a.pobj, sizeof(unsigned) * npobj,
                               cudaMemcpyDeviceToHost, st));
            d2h += (int64_t)(sizeof(unsigned) * npobj);
        }
        launches += neigh ? 2 : 1;  // (neighbours: the thresholds pre-pass too)
        CK(rec(plan->ev[2]));
        CK(cudaMemcpyAsync(at<char>(H, h_hist), a.hist, nm * nhist * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(at<char>(H, h_histd), a.histd, nm * nhist * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (ntab) {
            CK(cudaMemcpyAsync(at<char>(H, h_htag), a.htag, ntab * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st));
            d2h += (int64_t)(ntab * sizeof(unsigned long long));
        }
        CK(cudaMemcpyAsync(at<char>(H, h_misc), misc, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        CK(rec(plan->ev[3]));
        d2h += (int64_t)(nm * nhist * (sizeof(unsigned long long) + sizeof(double)) + 8 * sizeof(unsigned long long));
        return GBP_OK;
    };
    if (graph) {
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
        int erc = enqueue();
        cudaGraph_t gr = nullptr;
        cudaError_t ce = cudaStreamEndCapture(st, &gr);
        if (erc) {
            if (gr) cudaGraphDestroy(gr);
            return erc;
        }
        CK(ce);
        if (plan->gexec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(plan->gexec, gr, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(plan->gexec);
                plan->gexec = nullptr;
            }
        }
        if (!plan->gexec) {
            cudaError_t ie = cudaGraphInstantiate(&plan->gexec, gr, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(gr);
                CK(ie);
            }
        }
        cudaGraphDestroy(gr);
        CK(cudaGraphLaunch(plan->gexec, st));
    } else {
        int erc = enqueue();
        if (erc) return erc;
    }
    CK(cudaStreamSynchronize(st));

    const unsigned long long *hm = at<unsigned long long>(H, h_misc);
    int err_word = reinterpret_cast<const int *>(hm)[2];
    if (err_word & GBP_ERR_SMEM_LAYOUT)
        return fail(plan, GBP_ERR_CUDA, "internal: kernel shared-memory layout exceeds its launch");
    if (err_word & GBP_ERR_PAIR_SLOTS)
        return fail(plan, GBP_ERR_INVALID, "the pair list has more pairs than the given counts");
    if (err_word) return fail(plan, GBP_ERR_RANGE, "positions outside [0, period] or not finite");
    if (reinterpret_cast<const int *>(hm)[3]) {
        // more work items than the estimate: grow and repeat the call
        if (max_items >= (size_t)INT32_MAX / 2)
            return fail(plan, GBP_ERR_NOMEM, "too many work items");
        plan->item_cap = 2 * max_items;
        return run_call(plan, c, hist_host, histd_host);
    }
    hist_host.assign(at<unsigned long long>(H, h_hist), at<unsigned long long>(H, h_hist) + nm * nhist);
    if (c.mode != MODE_MARK && c.mode != MODE_MARKC && c.mode != MODE_XYZW && c.mode != MODE_NEIGH &&
        c.mode != MODE_JACKW && c.mode != MODE_JACKXYZW)
        add_self_pairs(c, hist_host);
    if (histd_host) histd_host->assign(at<double>(H, h_histd), at<double>(H, h_histd) + nm * nhist);
    if (ntab) c.htag.assign(at<unsigned long long>(H, h_htag), at<unsigned long long>(H, h_htag) + ntab);
    gbp_stats &S = plan->stats;
    S.recheck_pairs = (int64_t)hm[2];
    S.candidate_pairs = (int64_t)hm[3];
    for (int d = 0; d < 3; d++) S.cells[d] = c.g.n[d];
    S.reach = c.g.K;
    S.block = c.g.bf;
    S.stencil_cells = nsten;
    int nit = reinterpret_cast<const int *>(hm)[1];
    S.work_items = nit;
    cudaEventElapsedTime(&S.ms_build, plan->ev[0], plan->ev[1]);
    cudaEventElapsedTime(&S.ms_count, plan->ev[1], plan->ev[2]);
    cudaEventElapsedTime(&S.ms_total, plan->ev[0], plan->ev[3]);
    S.count_launches = 1;
    S.kernel_launches = launches;
    S.h2d_bytes = h2d;
    S.d2h_bytes = d2h;
    return GBP_OK;
}

int check_common(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                 const double *period3, int pbc, int mem) {
    if (!plan) return GBP_ERR_INVALID;
    if (n1 < 0 || n2 < 0) return fail(plan, GBP_ERR_INVALID, "negative point count");
    if ((n1 > 0 && !xyz1) || (n2 > 0 && !xyz2)) return fail(plan, GBP_ERR_INVALID, "null positions");
    if (n1 >= (1ll << 30) || n2 >= (1ll << 30)) return fail(plan, GBP_ERR_INVALID, "too many points (limit 2^30)");
    if (!period3) return fail(plan, GBP_ERR_INVALID, "null period");
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0) || !std::isfinite(period3[d]))
            return fail(plan, GBP_ERR_INVALID, "period must be finite and positive");
    if (pbc != 0 && pbc != 1) return fail(plan, GBP_ERR_INVALID, "pbc must be 0 or 1");
    if (mem != GBP_MEM_HOST && mem != GBP_MEM_DEVICE) return fail(plan, GBP_ERR_INVALID, "bad mem kind");
    return GBP_OK;
}

int check_search(gbp_plan *plan, const double search[3], const double period3[3]) {
    for (int d = 0; d < 3; d++) {
        // rectangular_mesh.py:376-417
        if (!(search[d] <= period3[d] / 3.0))
            return fail(plan, GBP_ERR_RANGE,
                        "search length %.6g cannot be larger than Lbox/3 (period %.6g)", search[d], period3[d]);
        if (!(search[d] > 0))
            return fail(plan, GBP_ERR_INVALID, "the largest bin edge must be positive");
    }
    return GBP_OK;
}



}  // namespace

// ======================= C ABI =======================
extern "C" {

int gbp_plan_create(int device, gbp_plan **out) {
    if (!out) return GBP_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return GBP_ERR_NODEVICE;
    if (device < 0 || device >= ndev) return GBP_ERR_INVALID;
    gbp_plan *plan = new gbp_plan();
    plan->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->own, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaEventCreate(&plan->ev[i]);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&plan->nsm, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        gbp_plan_destroy(plan);
        return GBP_ERR_CUDA;
    }
    plan->stream = plan->own;
    *out = plan;
    return GBP_OK;
}

int gbp_plan_destroy(gbp_plan *plan) {
    if (!plan) return GBP_OK;
    cudaSetDevice(plan->device);
    if (plan->stream) cudaStreamSynchronize(plan->stream);
    if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
    if (plan->work.p) cudaFree(plan->work.p);
    if (plan->pinned) cudaFreeHost(plan->pinned);
    for (int i = 0; i < 4; i++)
        if (plan->ev[i]) cudaEventDestroy(plan->ev[i]);
    if (plan->own) cudaStreamDestroy(plan->own);
    delete plan;
    return GBP_OK;
}

int gbp_plan_set_stream(gbp_plan *plan, void *s) {
    if (!plan) return GBP_ERR_INVALID;
    plan->stream = s ? static_cast<cudaStream_t>(s) : plan->own;
    return GBP_OK;
}

int gbp_plan_set_reach(gbp_plan *plan, int reach) {
    if (!plan || reach < 0 || reach > 4) return GBP_ERR_INVALID;
    plan->reach = reach;
    return GBP_OK;
}

int gbp_plan_set_block(gbp_plan *plan, int block) {
    if (!plan || block < 0 || block > 4) return GBP_ERR_INVALID;
    plan->block = block;
    return GBP_OK;
}

int gbp_grid_describe(const double *period3, int32_t pbc, const double *search3, int64_t n2,
                      int32_t kind, int32_t reach, int32_t block, int32_t *out) {
    if (!period3 || !search3 || !out || n2 < 0 || kind < 0 || kind > 2 || reach < 0 || reach > 4 ||
        block < 0 || block > 4)
        return GBP_ERR_INVALID;
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(search3[d] > 0.0) ||
            !(search3[d] * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // the choices of the entry points: npairs_3d (up to GBP_NB_LANE edges) and
    // npairs_s_mu take finer grids for dense samples, npairs_xy_z the default
    Geometry g;
    if (kind == 2) {
        choose_grid(g, period3, search3, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block);
    } else {
        choose_grid(g, period3, search3, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block,
                    GBP_DENSE_REACH2, true);
    }
    build_stencil(g, search3, kind == 2 ? 1 : 0, true);
    out[0] = g.K;
    out[1] = g.bf;
    for (int d = 0; d < 3; d++) out[2 + d] = g.n[d];
    out[5] = g.nsten;
    out[6] = g.DB;
    return GBP_OK;
}

int gbp_npairs_3d_thresholds(const double *period3, int32_t pbc, const double *rbins, int32_t nb,
                             int64_t n2, int32_t reach, int32_t block, float *hi, float *lo,
                             double *cell3) {
    if (!period3 || !rbins || !hi || !lo || !cell3 || nb < 2 || nb > GBP_NB_LANE || n2 < 0 ||
        reach < 0 || reach > 4 || block < 0 || block > 4)
        return GBP_ERR_INVALID;
    const double rmax = max_nan(rbins, nb);
    const double search[3] = {rmax, rmax, rmax};
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(rmax > 0.0) ||
            !(rmax * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // as gbp_npairs_3d: its grid, its error model, its edges and thresholds
    Geometry g;
    choose_grid(g, period3, search, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block,
                GBP_DENSE_REACH2, true);
    ErrModel em = err_model(g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    thresholds(nb, E.data(), &em, 3, hi, lo);
    for (int d = 0; d < 3; d++) cell3[d] = g.c[d];
    return GBP_OK;
}

int gbp_npairs_xy_z_thresholds(const double *period3, int32_t pbc, const double *rp_bins,
                               int32_t n_rp, const double *pi_bins, int32_t n_pi, int64_t n2,
                               int32_t reach, int32_t block, float *hi_rp, float *lo_rp,
                               float *hi_pi, float *lo_pi, double *cell3) {
    if (!period3 || !rp_bins || !pi_bins || !hi_rp || !lo_rp || !hi_pi || !lo_pi || !cell3 ||
        n_rp < 2 || n_pi < 2 || n_rp > GBP_NB_MAX || n_pi > GBP_NB_MAX || n2 < 0 || reach < 0 ||
        reach > 4 || block < 0 || block > 4)
        return GBP_ERR_INVALID;
    const double rpm = max_nan(rp_bins, n_rp), pim = max_nan(pi_bins, n_pi);
    const double search[3] = {rpm, rpm, pim};
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(search[d] > 0.0) ||
            !(search[d] * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // as setup_xyz: its grid, its error model, its edges and thresholds
    Geometry g;
    choose_grid(g, period3, search, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block);
    ErrModel em = err_model(g);
    std::vector<double> E0(n_rp), E1(n_pi);
    edges_top_walk(rp_bins, n_rp, E0.data());
    edges_top_walk(pi_bins, n_pi, E1.data());
    thresholds(n_rp, E0.data(), &em, 2, hi_rp, lo_rp);
    thresholds(n_pi, E1.data(), &em, 1, hi_pi, lo_pi);
    for (int d = 0; d < 3; d++) cell3[d] = g.c[d];
    return GBP_OK;
}

int gbp_npairs_3d_lut(const double *period3, int32_t pbc, const double *rbins, int32_t nb,
                      int64_t n2, int32_t reach, int32_t block, float *lut, int32_t *info,
                      float *vrange) {
    if (!period3 || !rbins || !lut || !info || !vrange || nb < 2 || nb > GBP_NB_LANE || n2 < 0 ||
        reach < 0 || reach > 4 || block < 0 || block > 4)
        return GBP_ERR_INVALID;
    const double rmax = max_nan(rbins, nb);
    const double search[3] = {rmax, rmax, rmax};
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(rmax > 0.0) ||
            !(rmax * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // as gbp_npairs_3d: its grid, thresholds and float-bit table
    Geometry g;
    choose_grid(g, period3, search, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block,
                GBP_DENSE_REACH2, true);
    ErrModel em = err_model(g);
    AxisHost ax;
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    ax.set(E, &em, 3);
    ax.make_lut(no_qband);
    std::memcpy(lut, ax.lut.data(), sizeof(float4) * ax.T);
    info[0] = ax.T;
    info[1] = ax.S;
    info[2] = ax.B;
    vrange[0] = ax.vlo;
    vrange[1] = ax.vhi;
    return GBP_OK;
}

int gbp_stencil_describe(const double *period3, int32_t pbc, const double *search3, int64_t n2,
                         int32_t kind, int32_t reach, int32_t block, int32_t autocorr,
                         int32_t *runs, int32_t *nruns) {
    if (!period3 || !search3 || !runs || !nruns || n2 < 0 || kind < 0 || kind > 2 || reach < 0 ||
        reach > 4 || block < 0 || block > 4)
        return GBP_ERR_INVALID;
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(search3[d] > 0.0) ||
            !(search3[d] * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // the grid and stencil of gbp_grid_describe
    Geometry g;
    if (kind == 2) {
        choose_grid(g, period3, search3, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block);
    } else {
        choose_grid(g, period3, search3, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block,
                    GBP_DENSE_REACH2, true);
    }
    build_stencil(g, search3, kind == 2 ? 1 : 0, autocorr != 0);
    for (int s = 0; s < g.nsten; s++) {
        const int w = g.sten[s];
        int span;
        std::memcpy(&span, &g.stenD[s].w, 4);
        runs[5 * s + 0] = (w & 0xff) - 64;
        runs[5 * s + 1] = ((w >> 8) & 0xff) - 64;
        runs[5 * s + 2] = ((w >> 16) & 0xff) - 64;
        runs[5 * s + 3] = (w >> 24) & 0xff;
        runs[5 * s + 4] = span;
    }
    *nruns = g.nsten;
    return GBP_OK;
}

int gbp_plan_set_graph(gbp_plan *plan, int enable) {
    if (!plan) return GBP_ERR_INVALID;
    plan->graph_mode = enable != 0;
    return GBP_OK;
}

int gbp_plan_set_autotune(gbp_plan *plan, int enable) {
    if (!plan) return GBP_ERR_INVALID;
    plan->autotune = enable != 0;
    return GBP_OK;
}

int gbp_plan_set_limits(gbp_plan *plan, int64_t first_item_cap, int64_t flush_after) {
    if (!plan || first_item_cap < 0 || first_item_cap > INT32_MAX / 2 || flush_after < 0)
        return GBP_ERR_INVALID;
    plan->first_item_cap = (size_t)first_item_cap;
    plan->item_cap = 0;
    plan->flush_after = flush_after ? (unsigned long long)flush_after : (1ull << 24);
    return GBP_OK;
}

const char *gbp_plan_last_error(const gbp_plan *plan) { return plan ? plan->err.c_str() : "null plan"; }

int gbp_plan_stats(const gbp_plan *plan, gbp_stats *st) {
    if (!plan || !st) return GBP_ERR_INVALID;
    *st = plan->stats;
    return GBP_OK;
}

int gbp_npairs_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                  const double *rbins, int32_t nb, const double *period3, int32_t pbc, int32_t mem,
                  int64_t *counts) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (!rbins || nb < 2 || nb > GBP_NB_MAX || !counts)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_MAX);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    Call c;
    c.mode = nb <= GBP_NB_LANE ? MODE_3D : MODE_3DS;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = (xyz1 == xyz2 && n1 == n2);
    c.mem = mem;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block,
                GBP_DENSE_REACH2, c.mode == MODE_3D);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    std::vector<unsigned long long> h;
    if (n1 == 0 || n2 == 0) {
        for (int k = 0; k < nb; k++) counts[k] = 0;
        return GBP_OK;
    }
    if ((rc = run_call(plan, c, h))) return rc;
    unsigned long long run = 0;
    for (int k = 0; k < nb; k++) {
        run += h[k];
        counts[k] = (int64_t)run;
    }
    return GBP_OK;
}

int gbp_batched_npairs_3d(gbp_plan *plan, const void *xyz, int32_t xyz_f32, const int64_t *offsets,
                          int32_t nmocks, const double *rbins, int32_t nb, const double *period3,
                          int32_t pbc, int32_t mem, int64_t *counts) {
    if (!plan) return GBP_ERR_INVALID;
    if (nmocks < 1 || !offsets) return fail(plan, GBP_ERR_INVALID, "nmocks must be >= 1 with offsets");
    if (offsets[0] != 0) return fail(plan, GBP_ERR_INVALID, "offsets[0] must be 0");
    for (int m = 0; m < nmocks; m++)
        if (offsets[m + 1] < offsets[m]) return fail(plan, GBP_ERR_INVALID, "offsets must be non-decreasing");
    const int64_t n = offsets[nmocks];
    int rc = check_common(plan, (const double *)xyz, n, (const double *)xyz, n, period3, pbc, mem);
    if (rc) return rc;
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || !counts)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    Call c;
    c.mode = MODE_3D;
    c.xyz1 = c.xyz2 = (const double *)xyz;
    c.n1 = c.n2 = n;
    c.autocorr = true;
    c.mem = mem;
    c.naxes = 1;
    c.nmocks = nmocks;
    c.xyz_f32 = xyz_f32 ? 1 : 0;
    c.offsets.assign(offsets, offsets + nmocks + 1);
    for (int k = 0; k < nmocks * nb; k++) counts[k] = 0;
    if (n == 0) return GBP_OK;
    // the grid follows the mean mock density
    const int64_t nmean = std::max<int64_t>(1, n / nmocks);
    auto plan_geometry = [&](int reach, double ppc, int bf) {
        choose_grid(c.g, period3, search, pbc, nmean, reach, MAX_CELLS_PER_DIM, ppc, bf);
        // cell keys of all mocks must fit an int
        while (c.g.ncells * nmocks >= (1ll << 31) - 1 && c.g.K > 1)
            choose_grid(c.g, period3, search, pbc, nmean, c.g.K - 1, MAX_CELLS_PER_DIM, ppc, bf);
        build_stencil(c.g, search, 0, true);
        ErrModel em = err_model(c.g);
        std::vector<double> E(nb);
        edges_top_walk(rbins, nb, E.data());
        c.ax[0].set(E, &em, 3);
        c.ax[0].make_lut(no_qband);
    };
    std::vector<unsigned long long> h;
    int reach = plan->reach;
    double ppc = 0.0;
    int bf = plan->block;
    if (plan->autotune && reach == 0 && bf == 0) {
        char sig[256];
        snprintf(sig, sizeof(sig), "b3d:%d:%lld:%d:%.17g:%.17g:%.17g:%.17g:%d", nmocks, (long long)n,
                 nb, rmax, period3[0], period3[1], period3[2], pbc);
        int found = -1;
        for (size_t t = 0; t < plan->tuned.size(); t++)
            if (plan->tuned[t].first == sig) found = plan->tuned[t].second;
        // candidates: (reach, points per cell of coarse reach-1 cells, block factor)
        constexpr int NCAND = 9;
        static const int RK[NCAND] = {1, 1, 1, 1, 1, 1, 2, 2, 3};
        static const double PPC[NCAND] = {0.0, 0.0, 0.0, -1.0, 32.0, 64.0, 0.0, 0.0, 0.0};
        static const int BF[NCAND] = {2, 3, 4, 1, 1, 1, 1, 2, 1};
        if (found < 0) {
            float best = 1e30f;
            int bi = 3;
            for (int q = 0; q < NCAND; q++) {
                plan_geometry(RK[q], PPC[q], BF[q]);
                if (c.g.K != RK[q] || c.g.bf != BF[q]) continue;  // not feasible
                if ((rc = run_call(plan, c, h))) return rc;
                if (plan->stats.ms_count + plan->stats.ms_build < best) {
                    best = plan->stats.ms_count + plan->stats.ms_build;
                    bi = q;
                }
            }
            plan->tuned.emplace_back(sig, bi);
            found = bi;
        }
        reach = RK[found];
        ppc = PPC[found];
        bf = BF[found];
    }
    plan_geometry(reach, ppc, bf);
    if (c.g.ncells * nmocks >= (1ll << 31) - 1)
        return fail(plan, GBP_ERR_INVALID, "too many mocks for one batched grid");
    if ((rc = run_call(plan, c, h))) return rc;
    const size_t nh = (size_t)nb + 1;
    for (int m = 0; m < nmocks; m++) {
        unsigned long long run = 0;
        for (int k = 0; k < nb; k++) {
            run += h[m * nh + k];
            counts[(size_t)m * nb + k] = (int64_t)run;
        }
    }
    return GBP_OK;
}

// (rp, pi) geometry shared by npairs_xy_z and marked_npairs_xy_z: grid, stencil,
// edges walked from the top (npairs_xy_z_engine.pyx:183-194) and their guard bands
static int setup_xyz(gbp_plan *plan, Call &c, const double *xyz1, int64_t n1, const double *xyz2,
                     int64_t n2, const double *rp_bins, int32_t n_rp, const double *pi_bins,
                     int32_t n_pi, const double *period3, int32_t pbc, int32_t mem, bool autocorr) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (!rp_bins || !pi_bins || n_rp < 2 || n_pi < 2 || n_rp > GBP_NB_MAX || n_pi > GBP_NB_MAX)
        return fail(plan, GBP_ERR_INVALID, "bin arrays must have 2..%d entries", GBP_NB_MAX);
    double rpm = max_nan(rp_bins, n_rp), pim = max_nan(pi_bins, n_pi);
    double search[3] = {rpm, rpm, pim};
    if ((rc = check_search(plan, search, period3))) return rc;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = autocorr;
    c.mem = mem;
    c.naxes = 2;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 1, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E0(n_rp), E1(n_pi);
    edges_top_walk(rp_bins, n_rp, E0.data());
    edges_top_walk(pi_bins, n_pi, E1.data());
    c.ax[0].set(E0, &em, 2);
    c.ax[1].set(E1, &em, 1);
    c.ax[0].make_lut(no_qband);
    c.ax[1].make_lut(no_qband);
    return GBP_OK;
}

// out[k][g] = sum of the differential bins a <= k, b <= g: running sums along g,
// then along k (no subtraction, so integer-valued sums stay exact)
extern "C++" {
template <class T, class H>
static void cumulate_2d(const H *h, int na, int nb, T *out) {
    const int st = nb + 1;
    for (int k = 0; k < na; k++) {
        T run = 0;
        for (int g = 0; g < nb; g++) {
            run += (T)h[(size_t)k * st + g];
            out[k * nb + g] = run + (k > 0 ? out[(k - 1) * nb + g] : (T)0);
        }
    }
}
}

int gbp_npairs_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                    const double *rp_bins, int32_t n_rp, const double *pi_bins, int32_t n_pi,
                    const double *period3, int32_t pbc, int32_t mem, int64_t *counts) {
    if (!counts) return fail(plan, GBP_ERR_INVALID, "null output");
    Call c;
    c.mode = MODE_XYZ;
    int rc = setup_xyz(plan, c, xyz1, n1, xyz2, n2, rp_bins, n_rp, pi_bins, n_pi, period3, pbc,
                       mem, xyz1 == xyz2 && n1 == n2);
    if (rc) return rc;
    if (n1 == 0 || n2 == 0) {
        for (int k = 0; k < n_rp * n_pi; k++) counts[k] = 0;
        return GBP_OK;
    }
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    cumulate_2d(h.data(), n_rp, n_pi, counts);
    return GBP_OK;
}

// marking-function ids: number of weights per point (marked_npairs_3d.py:281-326)
static const int WFUNC_NW[18] = {0, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 4, 4, 3, 3, 5, 5};
// f(a, b) == f(b, a): an auto-correlation may walk each unordered pair once
static bool wfunc_symmetric(int id) { return id <= 4 || id >= 12; }

int gbp_marked_npairs_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                           int64_t n2, const double *w1, const double *w2, int32_t nw,
                           int32_t wfunc_id, const double *rp_bins, int32_t n_rp,
                           const double *pi_bins, int32_t n_pi, const double *period3, int32_t pbc,
                           int32_t mem, double *out) {
    if (!out) return fail(plan, GBP_ERR_INVALID, "null output");
    if (wfunc_id < 1 || wfunc_id > 17)
        return fail(plan, GBP_ERR_INVALID, "weight_func_id %d is not recognized", wfunc_id);
    if (nw != WFUNC_NW[wfunc_id])
        return fail(plan, GBP_ERR_INVALID, "weight_func_id %d needs %d weights per point", wfunc_id,
                    WFUNC_NW[wfunc_id]);
    if ((n1 > 0 && !w1) || (n2 > 0 && !w2)) return fail(plan, GBP_ERR_INVALID, "null weights");
    Call c;
    c.mode = MODE_XYZW;
    c.wf = (wfunc_id == 1) ? 1 : (wfunc_id == 2) ? 2 : 0;
    c.w1 = w1;
    c.w2 = w2;
    c.nw = nw;
    c.wfunc = wfunc_id;
    int rc = setup_xyz(plan, c, xyz1, n1, xyz2, n2, rp_bins, n_rp, pi_bins, n_pi, period3, pbc,
                       mem, xyz1 == xyz2 && n1 == n2 && w1 == w2 && wfunc_symmetric(wfunc_id));
    if (rc) return rc;
    for (int k = 0; k < n_rp * n_pi; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    cumulate_2d(hd.data(), n_rp, n_pi, out);
    return GBP_OK;
}

// The (s, mu') grid, stencil and tables of a call: the differential bins of
// the strict walks (edges_smu), the s thresholds with the per-slot bound of q,
// and the tight FP32 bracket of each mu'^2 edge (the band of q is per pair)
static void smu_tables(Call &c, const double *period3, int32_t pbc, int64_t n2, int reach, int block,
                       const double *s_bins, int32_t n_s, const double *mu_prime, int32_t n_mu) {
    const double smax = max_nan(s_bins, n_s);
    const double search[3] = {smax, smax, smax};
    choose_grid(c.g, period3, search, pbc, n2, reach, MAX_CELLS_PER_DIM, 0.0, block,
                c.mode == MODE_SMU ? GBP_DENSE_REACH2 : 28.0, c.mode == MODE_SMU);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> Es(n_s), Em(n_mu), Eps(n_s), Epm(n_mu);
    for (int k = 0; k < n_s; k++) Es[k] = s_bins[k] * s_bins[k];
    for (int k = 0; k < n_mu; k++) Em[k] = mu_prime[k] * mu_prime[k];
    edges_smu(Es.data(), n_s, Eps.data());
    edges_smu(Em.data(), n_mu, Epm.data());
    c.ax[0].set(Eps, &em, 3);
    c.ax[1].set(Epm, nullptr, 0);
    // dxy / s^2 never exceeds 1 in FP64 (dxy <= fl(dz^2 + dxy)), so a top mu'^2
    // edge >= 1 is never crossed: no pair needs a recheck against it
    if (Epm[n_mu - 1] >= 1.0) c.ax[1].hi[n_mu - 1] = c.ax[1].lo[n_mu - 1] = INFINITY;
    // q = dxy/s^2 error bound for pairs with s^2 >= a (FP32 value), factor 2 margin
    double dtop = em.delta(smax * smax);
    double Lm = em.Lmax;
    ErrModel emc = em;
    c.ax[0].make_lut([&](float a) -> float {
        double s2lo = (double)a - 2.0 * emc.band((double)a, 3);
        if (!(s2lo > 0)) return 3.0e38f;
        double s = std::sqrt(s2lo);
        double qb = 9.0 * std::ldexp(1.0, -24) + 4.6 * dtop / s + 5.0 * dtop * dtop / (s * s) +
                    std::ldexp(1.0, -48) * Lm / s;
        return f_up(2.0 * qb);
    });
    c.ax[1].make_lut(no_qband);
}

// (s, mu') geometry shared by npairs_s_mu and weighted_npairs_s_mu: differential
// bins found by the strict walks of npairs_s_mu_engine.pyx:200-226, the FP32
// guard bands, and the per-slot error bound of q = dxy / s^2
static int setup_smu(gbp_plan *plan, Call &c, const double *xyz1, int64_t n1, const double *xyz2,
                     int64_t n2, const double *s_bins, int32_t n_s, const double *mu_prime,
                     int32_t n_mu, const double *period3, int32_t pbc, int32_t mem) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (!s_bins || !mu_prime || n_s < 2 || n_mu < 2 || n_s > GBP_NB_MAX || n_mu > GBP_NB_MAX)
        return fail(plan, GBP_ERR_INVALID, "bin arrays must have 2..%d entries", GBP_NB_MAX);
    double smax = max_nan(s_bins, n_s);
    double search[3] = {smax, smax, smax};
    if ((rc = check_search(plan, search, period3))) return rc;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = (xyz1 == xyz2 && n1 == n2 && c.w1 == c.w2);
    c.mem = mem;
    c.naxes = 2;
    smu_tables(c, period3, pbc, n2, plan->reach, plan->block, s_bins, n_s, mu_prime, n_mu);
    return GBP_OK;
}

int gbp_npairs_s_mu_tables(const double *period3, int32_t pbc, const double *s_bins, int32_t n_s,
                           const double *mu_prime, int32_t n_mu, int64_t n2, int32_t reach,
                           int32_t block, float *s_lut, float *s_hi, float *s_lo, float *q_lut,
                           float *q_hi, float *q_lo, int32_t *info, float *vrange, double *cell3) {
    if (!period3 || !s_bins || !mu_prime || !s_lut || !s_hi || !s_lo || !q_lut || !q_hi ||
        !q_lo || !info || !vrange || !cell3 || n_s < 2 || n_mu < 2 || n_s > GBP_NB_MAX ||
        n_mu > GBP_NB_MAX || n2 < 0 || reach < 0 || reach > 4 || block < 0 || block > 4)
        return GBP_ERR_INVALID;
    const double smax = max_nan(s_bins, n_s);
    for (int d = 0; d < 3; d++)
        if (!(period3[d] > 0.0) || !std::isfinite(period3[d]) || !(smax > 0.0) ||
            !(smax * 3.0 <= period3[d]))
            return GBP_ERR_RANGE;
    // the tables an npairs_s_mu auto-correlation builds (smu_tables)
    Call c;
    c.mode = MODE_SMU;
    c.autocorr = true;
    smu_tables(c, period3, pbc, n2, reach, block, s_bins, n_s, mu_prime, n_mu);
    std::memcpy(s_lut, c.ax[0].lut.data(), sizeof(float4) * c.ax[0].T);
    std::memcpy(q_lut, c.ax[1].lut.data(), sizeof(float4) * c.ax[1].T);
    for (int k = 0; k < n_s; k++) {
        s_hi[k] = c.ax[0].hi[k];
        s_lo[k] = c.ax[0].lo[k];
    }
    for (int k = 0; k < n_mu; k++) {
        q_hi[k] = c.ax[1].hi[k];
        q_lo[k] = c.ax[1].lo[k];
    }
    const int vals[6] = {c.ax[0].T, c.ax[0].S, c.ax[0].B, c.ax[1].T, c.ax[1].S, c.ax[1].B};
    for (int k = 0; k < 6; k++) info[k] = vals[k];
    vrange[0] = c.ax[0].vlo;
    vrange[1] = c.ax[0].vhi;
    vrange[2] = c.ax[1].vlo;
    vrange[3] = c.ax[1].vhi;
    for (int d = 0; d < 3; d++) cell3[d] = c.g.c[d];
    return GBP_OK;
}

int gbp_npairs_s_mu(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                    const double *s_bins, int32_t n_s, const double *mu_prime, int32_t n_mu,
                    const double *period3, int32_t pbc, int32_t mem, int64_t *counts) {
    if (!counts) return fail(plan, GBP_ERR_INVALID, "null output");
    Call c;
    c.mode = MODE_SMU;
    int rc = setup_smu(plan, c, xyz1, n1, xyz2, n2, s_bins, n_s, mu_prime, n_mu, period3, pbc, mem);
    if (rc) return rc;
    if (n1 == 0 || n2 == 0) {
        for (int k = 0; k < n_s * n_mu; k++) counts[k] = 0;
        return GBP_OK;
    }
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    // npairs_s_mu_engine.pyx:232-234
    cumulate_2d(h.data(), n_s, n_mu, counts);
    return GBP_OK;
}

int gbp_weighted_npairs_s_mu(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                             int64_t n2, const double *w1, const double *w2, const double *s_bins,
                             int32_t n_s, const double *mu_prime, int32_t n_mu,
                             const double *period3, int32_t pbc, int32_t mem, int64_t *counts,
                             double *wcounts) {
    if (!counts || !wcounts) return fail(plan, GBP_ERR_INVALID, "null output");
    if ((n1 > 0 && !w1) || (n2 > 0 && !w2)) return fail(plan, GBP_ERR_INVALID, "null weights");
    Call c;
    c.mode = MODE_SMUW;
    c.wf = 1;  // w1 * w2 (weighted_npairs_s_mu_engine.pyx:249)
    c.w1 = w1;
    c.w2 = w2;
    c.nw = 1;
    c.wfunc = 1;
    int rc = setup_smu(plan, c, xyz1, n1, xyz2, n2, s_bins, n_s, mu_prime, n_mu, period3, pbc, mem);
    if (rc) return rc;
    for (int k = 0; k < n_s * n_mu; k++) {
        counts[k] = 0;
        wcounts[k] = 0.0;
    }
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    // weighted_npairs_s_mu_engine.pyx:251-255: rectangle sums of the differential bins
    cumulate_2d(h.data(), n_s, n_mu, counts);
    cumulate_2d(hd.data(), n_s, n_mu, wcounts);
    return GBP_OK;
}

int gbp_marked_npairs_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                         int64_t n2, const double *w1, const double *w2, int32_t nw,
                         int32_t wfunc_id, const double *rbins, int32_t nb, const double *period3,
                         int32_t pbc, int32_t mem, double *out) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (wfunc_id < 1 || wfunc_id > 17) return fail(plan, GBP_ERR_INVALID, "weight_func_id %d is not recognized", wfunc_id);
    if (nw != WFUNC_NW[wfunc_id]) return fail(plan, GBP_ERR_INVALID, "weight_func_id %d needs %d weights per point", wfunc_id, WFUNC_NW[wfunc_id]);
    if ((n1 > 0 && !w1) || (n2 > 0 && !w2)) return fail(plan, GBP_ERR_INVALID, "null weights");
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || !out)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    // symmetric marking functions (f(a, b) == f(b, a)) may walk each unordered
    // pair once; the others walk every ordered pair
    const bool symmetric = wfunc_symmetric(wfunc_id);
    Call c;
    c.mode = MODE_MARK;
    c.wf = (wfunc_id == 1) ? 1 : (wfunc_id == 2) ? 2 : 0;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = (xyz1 == xyz2 && n1 == n2 && w1 == w2 && symmetric);
    c.mem = mem;
    c.w1 = w1;
    c.w2 = w2;
    c.nw = nw;
    c.wfunc = wfunc_id;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    for (int k = 0; k < nb; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    double run = 0.0;
    for (int k = 0; k < nb; k++) {
        run += hd[k];
        out[k] = run;
    }
    return GBP_OK;
}

int gbp_marked_npairs_3d_channels(gbp_plan *plan, const double *xyz1, int64_t n1,
                                  const double *xyz2, int64_t n2, const double *w1,
                                  const double *w2, int32_t nch, const double *rbins, int32_t nb,
                                  const double *period3, int32_t pbc, int32_t mem, double *out) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (nch < 1 || nch > 32) return fail(plan, GBP_ERR_INVALID, "nch must be 1..32, got %d", nch);
    if ((n1 > 0 && !w1) || (n2 > 0 && !w2)) return fail(plan, GBP_ERR_INVALID, "null weights");
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || !out)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    Call c;
    c.mode = MODE_MARKC;
    c.wf = 1;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    // the product is symmetric: an auto-correlation walks each unordered pair once
    c.autocorr = (xyz1 == xyz2 && n1 == n2 && w1 == w2);
    c.mem = mem;
    c.w1 = w1;
    c.w2 = w2;
    c.nw = nch;
    c.wfunc = 1;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    for (int k = 0; k < nch * nb; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    for (int ch = 0; ch < nch; ch++) {
        double run = 0.0;
        for (int k = 0; k < nb; k++) {
            run += hd[(size_t)ch * (nb + 1) + k];
            out[(size_t)ch * nb + k] = run;
        }
    }
    return GBP_OK;
}

int gbp_npairs_jackknife_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                            int64_t n2, const int32_t *jtags1, const int32_t *jtags2,
                            int32_t n_samples, const double *rbins, int32_t nb,
                            const double *period3, int32_t pbc, int32_t mem, double *out) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (mem != GBP_MEM_HOST)
        return fail(plan, GBP_ERR_INVALID, "jackknife counts take host positions and tags");
    if (n_samples < 1 || (n1 > 0 && !jtags1) || (n2 > 0 && !jtags2))
        return fail(plan, GBP_ERR_INVALID, "N_samples must be >= 1 with one tag per point");
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || !out)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    if ((int64_t)(n_samples + 1) * (nb + 1) * 8 > (48 << 10))
        return fail(plan, GBP_ERR_INVALID, "too many jackknife samples x bins for one table");
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    // tags go through the weight path as exact FP64 / FP32 integers
    const bool autocorr = (xyz1 == xyz2 && n1 == n2 && jtags1 == jtags2);
    std::vector<double> t1((size_t)n1), t2;
    for (int64_t i = 0; i < n1; i++) {
        if (jtags1[i] < 1 || jtags1[i] > n_samples)
            return fail(plan, GBP_ERR_INVALID, "jtags1 must be in [1, N_samples]");
        t1[(size_t)i] = (double)jtags1[i];
    }
    if (!autocorr) {
        t2.resize((size_t)n2);
        for (int64_t i = 0; i < n2; i++) {
            if (jtags2[i] < 1 || jtags2[i] > n_samples)
                return fail(plan, GBP_ERR_INVALID, "jtags2 must be in [1, N_samples]");
            t2[(size_t)i] = (double)jtags2[i];
        }
    }
    Call c;
    c.mode = MODE_JACK;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = autocorr;
    c.mem = mem;
    c.w1 = t1.data();
    c.w2 = autocorr ? t1.data() : t2.data();
    c.nw = 1;
    c.wf = 1;
    c.ntag = n_samples + 1;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    const int rows = n_samples + 1;
    for (int k = 0; k < rows * nb; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    std::vector<unsigned long long> &tab = c.htag;
    if (autocorr) {
        // (i, i): distance 0, both ends carry tag_i (the kernels skip it)
        const int sb = host_bin(nb, c.ax[0].E.data(), 0.0);
        if (sb < nb)
            for (int64_t i = 0; i < n1; i++) tab[(size_t)jtags1[i] * (nb + 1) + sb] += 2;
    }
    double cT = 0.0;
    std::vector<double> cQ((size_t)rows, 0.0);
    for (int k = 0; k < nb; k++) {
        cT += (double)h[k];
        out[k] = cT;
        for (int s = 1; s < rows; s++) {
            cQ[(size_t)s] += (double)tab[(size_t)s * (nb + 1) + k];
            out[(size_t)s * nb + k] = cT - 0.5 * cQ[(size_t)s];
        }
    }
    return GBP_OK;
}

int gbp_npairs_jackknife_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                              int64_t n2, const int32_t *jtags1, const int32_t *jtags2,
                              int32_t n_samples, const double *rp_bins, int32_t n_rp,
                              const double *pi_bins, int32_t n_pi, const double *period3,
                              int32_t pbc, int32_t mem, double *out) {
    if (!out) return fail(plan, GBP_ERR_INVALID, "null output");
    if (mem != GBP_MEM_HOST)
        return fail(plan, GBP_ERR_INVALID, "jackknife counts take host positions and tags");
    // tags travel packed as tag_i | tag_j << 16
    if (n_samples < 1 || n_samples > 32767 || (n1 > 0 && !jtags1) || (n2 > 0 && !jtags2))
        return fail(plan, GBP_ERR_INVALID, "N_samples must be 1..32767 with one tag per point");
    const bool autocorr = (xyz1 == xyz2 && n1 == n2 && jtags1 == jtags2);
    // tags go through the weight path as exact FP64 / FP32 integers
    std::vector<double> t1((size_t)n1), t2;
    for (int64_t i = 0; i < n1; i++) {
        if (jtags1[i] < 1 || jtags1[i] > n_samples)
            return fail(plan, GBP_ERR_INVALID, "jtags1 must be in [1, N_samples]");
        t1[(size_t)i] = (double)jtags1[i];
    }
    if (!autocorr) {
        t2.resize((size_t)n2);
        for (int64_t i = 0; i < n2; i++) {
            if (jtags2[i] < 1 || jtags2[i] > n_samples)
                return fail(plan, GBP_ERR_INVALID, "jtags2 must be in [1, N_samples]");
            t2[(size_t)i] = (double)jtags2[i];
        }
    }
    Call c;
    c.mode = MODE_JACKXYZ;
    c.w1 = t1.data();
    c.w2 = autocorr ? t1.data() : t2.data();
    c.nw = 1;
    c.wf = 1;
    c.ntag = n_samples + 1;
    int rc = setup_xyz(plan, c, xyz1, n1, xyz2, n2, rp_bins, n_rp, pi_bins, n_pi, period3, pbc,
                       mem, autocorr);
    if (rc) return rc;
    const int rows = n_samples + 1;
    const size_t plane = (size_t)n_rp * n_pi;
    for (size_t k = 0; k < rows * plane; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    std::vector<unsigned long long> &tab = c.htag;
    const size_t nbin = (size_t)(n_rp + 1) * (n_pi + 1);
    if (autocorr) {
        // (i, i): separation 0, both ends carry tag_i (the kernels skip it)
        const int a0 = host_bin(n_rp, c.ax[0].E.data(), 0.0);
        const int b0 = host_bin(n_pi, c.ax[1].E.data(), 0.0);
        if (a0 < n_rp && b0 < n_pi)
            for (int64_t i = 0; i < n1; i++)
                tab[(size_t)jtags1[i] * nbin + (size_t)a0 * (n_pi + 1) + b0] += 2;
    }
    // npairs_jackknife_xy_z_engine: row 0 all pairs, row s the pairs without
    // subsample s, one end in s counting one half: C - (ends in s) / 2
    std::vector<double> C(plane), Q(plane);
    cumulate_2d(h.data(), n_rp, n_pi, C.data());
    for (size_t k = 0; k < plane; k++) out[k] = C[k];
    for (int sidx = 1; sidx < rows; sidx++) {
        cumulate_2d(tab.data() + (size_t)sidx * nbin, n_rp, n_pi, Q.data());
        for (size_t k = 0; k < plane; k++) out[(size_t)sidx * plane + k] = C[k] - 0.5 * Q[k];
    }
    return GBP_OK;
}

// Weighted jackknife counts (npairs_jackknife_3d.py / npairs_jackknife_xy_z.py
// with weights; jweight of the engines): rows {w, tag} per point, C_w and the
// FP64 (tag, bin) table of w_i w_j per pair end, row s = C_w - Q_w(s) / 2.
static int jackknife_weighted(gbp_plan *plan, Call &c, const double *xyz1, int64_t n1,
                              const double *xyz2, int64_t n2, const double *w1, const double *w2,
                              const int32_t *jtags1, const int32_t *jtags2, int32_t n_samples,
                              std::vector<double> &r1, std::vector<double> &r2) {
    if (n_samples < 1 || n_samples > 32767 || (n1 > 0 && (!jtags1 || !w1)) ||
        (n2 > 0 && (!jtags2 || !w2)))
        return fail(plan, GBP_ERR_INVALID, "N_samples must be 1..32767 with one tag and weight per point");
    const bool autocorr = (xyz1 == xyz2 && n1 == n2 && jtags1 == jtags2 && w1 == w2);
    r1.assign(2 * (size_t)std::max<int64_t>(n1, 1), 0.0);
    for (int64_t i = 0; i < n1; i++) {
        if (jtags1[i] < 1 || jtags1[i] > n_samples)
            return fail(plan, GBP_ERR_INVALID, "jtags1 must be in [1, N_samples]");
        r1[2 * (size_t)i] = w1[i];
        r1[2 * (size_t)i + 1] = (double)jtags1[i];
    }
    if (!autocorr) {
        r2.assign(2 * (size_t)std::max<int64_t>(n2, 1), 0.0);
        for (int64_t i = 0; i < n2; i++) {
            if (jtags2[i] < 1 || jtags2[i] > n_samples)
                return fail(plan, GBP_ERR_INVALID, "jtags2 must be in [1, N_samples]");
            r2[2 * (size_t)i] = w2[i];
            r2[2 * (size_t)i + 1] = (double)jtags2[i];
        }
    }
    c.w1 = r1.data();
    c.w2 = autocorr ? r1.data() : r2.data();
    c.nw = 2;
    c.wf = 1;
    c.ntag = n_samples + 1;
    c.autocorr = autocorr;
    return GBP_OK;
}

int gbp_npairs_jackknife_3d_weighted(gbp_plan *plan, const double *xyz1, int64_t n1,
                                     const double *xyz2, int64_t n2, const double *w1,
                                     const double *w2, const int32_t *jtags1,
                                     const int32_t *jtags2, int32_t n_samples,
                                     const double *rbins, int32_t nb, const double *period3,
                                     int32_t pbc, int32_t mem, double *out) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (mem != GBP_MEM_HOST)
        return fail(plan, GBP_ERR_INVALID, "jackknife counts take host positions and tags");
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || !out)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    Call c;
    c.mode = MODE_JACKW;
    std::vector<double> r1, r2;
    if ((rc = jackknife_weighted(plan, c, xyz1, n1, xyz2, n2, w1, w2, jtags1, jtags2, n_samples,
                                 r1, r2)))
        return rc;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.mem = mem;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, c.autocorr);
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    const int rows = n_samples + 1;
    for (int k = 0; k < rows * nb; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    const double *tab = reinterpret_cast<const double *>(c.htag.data());
    double cT = 0.0;
    std::vector<double> cQ((size_t)rows, 0.0);
    for (int k = 0; k < nb; k++) {
        cT += hd[k];
        out[k] = cT;
        for (int sidx = 1; sidx < rows; sidx++) {
            cQ[(size_t)sidx] += tab[(size_t)sidx * (nb + 1) + k];
            out[(size_t)sidx * nb + k] = cT - 0.5 * cQ[(size_t)sidx];
        }
    }
    return GBP_OK;
}

int gbp_npairs_jackknife_xy_z_weighted(gbp_plan *plan, const double *xyz1, int64_t n1,
                                       const double *xyz2, int64_t n2, const double *w1,
                                       const double *w2, const int32_t *jtags1,
                                       const int32_t *jtags2, int32_t n_samples,
                                       const double *rp_bins, int32_t n_rp, const double *pi_bins,
                                       int32_t n_pi, const double *period3, int32_t pbc,
                                       int32_t mem, double *out) {
    if (!out) return fail(plan, GBP_ERR_INVALID, "null output");
    if (mem != GBP_MEM_HOST)
        return fail(plan, GBP_ERR_INVALID, "jackknife counts take host positions and tags");
    Call c;
    c.mode = MODE_JACKXYZW;
    std::vector<double> r1, r2;
    int rc = jackknife_weighted(plan, c, xyz1, n1, xyz2, n2, w1, w2, jtags1, jtags2, n_samples,
                                r1, r2);
    if (rc) return rc;
    if ((rc = setup_xyz(plan, c, xyz1, n1, xyz2, n2, rp_bins, n_rp, pi_bins, n_pi, period3, pbc,
                        mem, c.autocorr)))
        return rc;
    const int rows = n_samples + 1;
    const size_t plane = (size_t)n_rp * n_pi;
    for (size_t k = 0; k < rows * plane; k++) out[k] = 0.0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    std::vector<unsigned long long> h;
    std::vector<double> hd;
    if ((rc = run_call(plan, c, h, &hd))) return rc;
    const double *tab = reinterpret_cast<const double *>(c.htag.data());
    const size_t nbin = (size_t)(n_rp + 1) * (n_pi + 1);
    std::vector<double> C(plane), Q(plane);
    cumulate_2d(hd.data(), n_rp, n_pi, C.data());
    for (size_t k = 0; k < plane; k++) out[k] = C[k];
    for (int sidx = 1; sidx < rows; sidx++) {
        cumulate_2d(tab + (size_t)sidx * nbin, n_rp, n_pi, Q.data());
        for (size_t k = 0; k < plane; k++) out[(size_t)sidx * plane + k] = C[k] - 0.5 * Q[k];
    }
    return GBP_OK;
}

// ---------------- per-object neighbours ----------------
// Shared set-up of counts_in_cylinders, its pair list and the isolation
// functions: sample-1 FP64 rows {r or rp, pi, marks...}, sample-2 rows
// {0, 0, marks...}, the grid for the largest radius, the full stencil.
static int neigh_setup(gbp_plan *plan, Call &c, std::vector<double> &wa, std::vector<double> &wb,
                       const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                       const double *r, const double *pi, const double *period3, int32_t pbc,
                       const gbp_neigh_cond *cond) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, GBP_MEM_HOST);
    if (rc) return rc;
    if (n1 > 0 && !r) return fail(plan, GBP_ERR_INVALID, "null radii");
    const int kind = cond ? cond->kind : 0;
    const int nm = cond ? cond->nmarks : 0;
    if (kind < 0 || kind > 2 || nm < 0 || nm > 2 || (kind == 1 && nm != 1) ||
        (kind == 2 && (cond->func < 0 || cond->func > 6 || nm < 1)))
        return fail(plan, GBP_ERR_INVALID, "unknown neighbour condition");
    if (kind && ((n1 > 0 && !cond->marks1) || (n2 > 0 && !cond->marks2)))
        return fail(plan, GBP_ERR_INVALID, "null marks");
    double rmax = 0.0, pmax = 0.0;
    for (int64_t i = 0; i < n1; i++) {
        const double ri = r[i], pj = pi ? pi[i] : 0.0;
        if (!(ri >= 0.0 && ri < INFINITY) || !(pj >= 0.0 && pj < INFINITY))
            return fail(plan, GBP_ERR_INVALID, "radii must be finite and non-negative");
        rmax = std::max(rmax, ri);
        pmax = std::max(pmax, pj);
    }
    if (!pi) pmax = rmax;
    // a tiny positive search keeps the grid sane when every radius is 0
    double search[3] = {std::max(rmax, 1e-300), std::max(rmax, 1e-300), std::max(pmax, 1e-300)};
    if ((rc = check_search(plan, search, period3))) return rc;
    const int nw = 2 + nm;
    const bool same = xyz1 == xyz2 && n1 == n2 && (!kind || cond->marks1 == cond->marks2);
    wa.assign((size_t)std::max<int64_t>(n1, 1) * nw, 0.0);
    for (int64_t i = 0; i < n1; i++) {
        wa[(size_t)i * nw] = r[i];
        wa[(size_t)i * nw + 1] = pi ? pi[i] : 0.0;
        for (int k = 0; k < nm; k++) wa[(size_t)i * nw + 2 + k] = cond->marks1[(size_t)i * nm + k];
    }
    if (!same) {
        wb.assign((size_t)std::max<int64_t>(n2, 1) * nw, 0.0);
        for (int64_t j = 0; j < n2; j++)
            for (int k = 0; k < nm; k++) wb[(size_t)j * nw + 2 + k] = cond->marks2[(size_t)j * nm + k];
    }
    c.mode = MODE_NEIGH;
    c.xyz1 = xyz1;
    c.xyz2 = same ? xyz1 : xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = same;  // one sorted copy; the walk is a gather
    c.mem = GBP_MEM_HOST;
    c.w1 = wa.data();
    c.w2 = same ? wa.data() : wb.data();
    c.nw = nw;
    c.wf = 0;
    c.ngeo = pi ? 1 : 0;
    if (kind == 1) {
        c.ncond = 1;
        c.ncpar[0] = cond->lim[0];
        c.ncpar[1] = cond->lim[1];
        c.nceq[0] = cond->lower_inclusive ? 1 : 0;
        c.nceq[1] = cond->upper_inclusive ? 1 : 0;
    } else if (kind == 2) {
        c.ncond = 10 + cond->func;
    }
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, pi ? 1 : 0, false);  // full stencil: each row gathers its own
    // the pre-filter of the walk: one edge per axis at the largest radius squared
    ErrModel em = err_model(c.g);
    if (pi) {
        std::vector<double> E0(1, search[0] * search[0]), E1(1, search[2] * search[2]);
        c.naxes = 2;
        c.ax[0].set(E0, &em, 2);
        c.ax[1].set(E1, &em, 1);
        c.ax[0].make_lut(no_qband);
        c.ax[1].make_lut(no_qband);
    } else {
        std::vector<double> E0(1, search[0] * search[0]);
        c.naxes = 1;
        c.ax[0].set(E0, &em, 3);
        c.ax[0].make_lut(no_qband);
    }
    return GBP_OK;
}

int gbp_counts_in_cylinders(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                            int64_t n2, const double *rp, const double *pi, const double *period3,
                            int32_t pbc, const gbp_neigh_cond *cond, int64_t *counts) {
    if (!pi || (n1 > 0 && !counts)) return fail(plan, GBP_ERR_INVALID, "null argument");
    Call c;
    std::vector<double> wa, wb;
    int rc = neigh_setup(plan, c, wa, wb, xyz1, n1, xyz2, n2, rp, pi, period3, pbc, cond);
    if (rc) return rc;
    for (int64_t i = 0; i < n1; i++) counts[i] = 0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    c.nout = 0;
    c.pobj.assign((size_t)n1, 0u);
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    for (int64_t i = 0; i < n1; i++) counts[i] = (int64_t)c.pobj[(size_t)i];
    return GBP_OK;
}

int gbp_cylinder_pairs(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                       int64_t n2, const double *rp, const double *pi, const double *period3,
                       int32_t pbc, const gbp_neigh_cond *cond, const int64_t *counts,
                       uint32_t *pairs) {
    if (!pi || (n1 > 0 && !counts)) return fail(plan, GBP_ERR_INVALID, "null argument");
    if (n1 > (int64_t)UINT32_MAX || n2 > (int64_t)UINT32_MAX)
        return fail(plan, GBP_ERR_INVALID, "pair indexes are uint32: at most 2^32 - 1 points");
    Call c;
    std::vector<double> wa, wb;
    int rc = neigh_setup(plan, c, wa, wb, xyz1, n1, xyz2, n2, rp, pi, period3, pbc, cond);
    if (rc) return rc;
    c.poff.assign((size_t)n1 + 1, 0);
    int64_t tot = 0;
    for (int64_t i = 0; i < n1; i++) {
        if (counts[i] < 0) return fail(plan, GBP_ERR_INVALID, "negative count");
        c.poff[(size_t)i] = tot;
        tot += counts[i];
    }
    c.poff[(size_t)n1] = tot;
    if (tot == 0 || n2 == 0) return GBP_OK;
    if (!pairs) return fail(plan, GBP_ERR_INVALID, "null pair buffer");
    c.nout = 2;
    c.npairs = tot;
    c.pairs_out = pairs;
    std::vector<unsigned long long> h;
    return run_call(plan, c, h);
}

int gbp_isolation(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                  const double *r, const double *pi, const double *period3, int32_t pbc,
                  const gbp_neigh_cond *cond, uint8_t *is_isolated) {
    if (n1 > 0 && !is_isolated) return fail(plan, GBP_ERR_INVALID, "null output");
    if (cond && cond->kind == 1) return fail(plan, GBP_ERR_INVALID, "isolation takes marking functions");
    Call c;
    std::vector<double> wa, wb;
    int rc = neigh_setup(plan, c, wa, wb, xyz1, n1, xyz2, n2, r, pi, period3, pbc, cond);
    if (rc) return rc;
    for (int64_t i = 0; i < n1; i++) is_isolated[i] = 1;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    c.nout = 1;
    c.nexcl0 = 1;  // a neighbour sits at separation > 0
    c.pobj.assign((size_t)n1, 0u);
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    for (int64_t i = 0; i < n1; i++) is_isolated[i] = c.pobj[(size_t)i] ? 0 : 1;
    return GBP_OK;
}

int gbp_npairs_per_object_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                             int64_t n2, const double *rbins, int32_t nb, const double *period3,
                             int32_t pbc, int32_t mem, int64_t *counts) {
    int rc = check_common(plan, xyz1, n1, xyz2, n2, period3, pbc, mem);
    if (rc) return rc;
    if (!rbins || nb < 2 || nb > GBP_NB_LANE || (n1 > 0 && !counts))
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_LANE);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    for (int64_t k = 0; k < n1 * nb; k++) counts[k] = 0;
    if (n1 == 0 || n2 == 0) return GBP_OK;
    Call c;
    c.mode = MODE_POBJ;
    c.xyz1 = xyz1;
    c.xyz2 = xyz2;
    c.n1 = n1;
    c.n2 = n2;
    c.autocorr = (xyz1 == xyz2 && n1 == n2);  // one sorted copy; the walk is a gather
    c.mem = mem;
    c.naxes = 1;
    choose_grid(c.g, period3, search, pbc, n2, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, false);  // full stencil: each row gathers its own pairs
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    c.pobj.assign((size_t)n1 * (size_t)(nb + 1), 0u);
    std::vector<unsigned long long> h;
    if ((rc = run_call(plan, c, h))) return rc;
    // cumulative per row (npairs_per_object_3d_engine.pyx: walk from the top edge)
    for (int64_t i = 0; i < n1; i++) {
        const unsigned *r = c.pobj.data() + (size_t)i * (nb + 1);
        int64_t run = 0;
        for (int k = 0; k < nb; k++) {
            run += r[k];
            counts[(size_t)i * nb + k] = run;
        }
    }
    return GBP_OK;
}

int gbp_weighted_adjoint_3d(gbp_plan *plan, const double *xyz, int64_t n, const double *w,
                            const double *rbins, int32_t nb, const double *period3, int32_t pbc,
                            int32_t mem, const double *gbar, double *grad_w) {
    int rc = check_common(plan, xyz, n, xyz, n, period3, pbc, mem);
    if (rc) return rc;
    if ((n > 0 && (!w || !grad_w)) || !gbar) return fail(plan, GBP_ERR_INVALID, "null weights or gradients");
    if (!rbins || nb < 2 || nb > GBP_NB_MAX)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_MAX);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    if (n == 0) return GBP_OK;
    Call c;
    c.mode = MODE_ADJ;
    c.xyz1 = c.xyz2 = xyz;
    c.n1 = c.n2 = n;
    c.autocorr = true;  // one sorted copy ...
    c.mem = mem;
    c.w1 = c.w2 = w;
    c.nw = 1;
    c.wfunc = 1;
    c.naxes = 1;
    c.grad_out = grad_w;
    choose_grid(c.g, period3, search, pbc, n, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, false);  // the full stencil: a gather, no scatter to j
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    c.gt.assign(nb + 1, 0.f);
    double run = 0.0;
    for (int k = nb - 1; k >= 0; k--) {
        run += gbar[k];
        c.gt[k] = (float)run;
    }
    std::vector<unsigned long long> h;
    return run_call(plan, c, h);
}

int gbp_weighted_adjoint_3d_channels(gbp_plan *plan, const double *xyz, int64_t n,
                                     const double *w, int32_t nch, const double *rbins,
                                     int32_t nb, const double *period3, int32_t pbc, int32_t mem,
                                     const double *gbar, double *grad_w) {
    int rc = check_common(plan, xyz, n, xyz, n, period3, pbc, mem);
    if (rc) return rc;
    if (nch < 1 || nch > GBP_ADJ_CH_MAX)
        return fail(plan, GBP_ERR_INVALID, "nch must be 1..%d, got %d", GBP_ADJ_CH_MAX, nch);
    if ((n > 0 && (!w || !grad_w)) || !gbar) return fail(plan, GBP_ERR_INVALID, "null weights or gradients");
    if (!rbins || nb < 2 || nb > GBP_NB_MAX)
        return fail(plan, GBP_ERR_INVALID, "rbins must have 2..%d entries", GBP_NB_MAX);
    double rmax = max_nan(rbins, nb);
    double search[3] = {rmax, rmax, rmax};
    if ((rc = check_search(plan, search, period3))) return rc;
    if (n == 0) return GBP_OK;
    Call c;
    c.mode = MODE_ADJC;
    c.xyz1 = c.xyz2 = xyz;
    c.n1 = c.n2 = n;
    c.autocorr = true;  // one sorted copy; the walk is a gather
    c.mem = mem;
    c.w1 = c.w2 = w;
    c.nw = nch;
    c.wfunc = 1;
    c.naxes = 1;
    c.grad_out = grad_w;
    choose_grid(c.g, period3, search, pbc, n, plan->reach, MAX_CELLS_PER_DIM, 0.0, plan->block);
    build_stencil(c.g, search, 0, false);  // the full stencil: a gather, no scatter to j
    ErrModel em = err_model(c.g);
    std::vector<double> E(nb);
    edges_top_walk(rbins, nb, E.data());
    c.ax[0].set(E, &em, 3);
    c.ax[0].make_lut(no_qband);
    // per channel: G(bin b) = sum of the upstream gradient over cumulative bins >= b
    c.gt.assign((size_t)nch * (nb + 1), 0.f);
    for (int ch = 0; ch < nch; ch++) {
        double run = 0.0;
        for (int k = nb - 1; k >= 0; k--) {
            run += gbar[(size_t)ch * nb + k];
            c.gt[(size_t)ch * (nb + 1) + k] = (float)run;
        }
    }
    std::vector<unsigned long long> h;
    return run_call(plan, c, h);
}

static int zheng07_args(gbp_plan *plan, const double *theta, Zheng07 *th) {
    if (!theta) return fail(plan, GBP_ERR_INVALID, "null theta");
    th->logMmin = theta[0];
    th->sigma = theta[1];
    th->logM0 = theta[2];
    th->logM1 = theta[3];
    th->alpha = theta[4];
    if (!(th->sigma > 0)) return fail(plan, GBP_ERR_INVALID, "sigma_logM must be positive");
    th->M0 = std::pow(10.0, th->logM0);
    th->M1 = std::pow(10.0, th->logM1);
    th->inv_sigma = 1.0 / th->sigma;
    th->inv_M1 = 1.0 / th->M1;
    return GBP_OK;
}

// Zheng07 weights / VJP for nth parameter vectors at once: the derived constants
// of every vector on the device, then one launch over (halo, vector)
static int zheng07_batched_args(gbp_plan *plan, const double *thetas, int32_t nth,
                                std::vector<Zheng07F> &th) {
    if (!thetas || nth < 1) return fail(plan, GBP_ERR_INVALID, "no parameter vector");
    th.resize((size_t)nth);
    for (int m = 0; m < nth; m++) {
        Zheng07 t;
        int rc = zheng07_args(plan, thetas + 5 * (size_t)m, &t);
        if (rc) return rc;
        th[(size_t)m] = gbp_zheng07_f(t);
    }
    return GBP_OK;
}

int gbp_zheng07_weights_batched(gbp_plan *plan, const double *mass, int64_t n,
                                const double *thetas, int32_t nth, int32_t mem, double *W) {
    if (!plan) return GBP_ERR_INVALID;
    std::vector<Zheng07F> th;
    int rc = zheng07_batched_args(plan, thetas, nth, th);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!mass || !W))) return fail(plan, GBP_ERR_INVALID, "null arrays");
    if (n == 0) return GBP_OK;
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    Carve cv;
    size_t o_th = cv.take<Zheng07F>((size_t)nth);
    size_t o_lm = cv.take<float4>((size_t)n);
    size_t o_m = mem == GBP_MEM_HOST ? cv.take<double>((size_t)n) : 0;
    size_t o_w = mem == GBP_MEM_HOST ? cv.take<double>((size_t)n * nth) : 0;
    if ((rc = ensure_work(plan, cv.take<char>(0) + 256))) return rc;
    void *Wk = plan->work.p;
    CK(cudaMemcpyAsync(at<char>(Wk, o_th), th.data(), sizeof(Zheng07F) * nth, cudaMemcpyHostToDevice, st));
    const double *dm = mass;
    double *dw = W;
    if (mem == GBP_MEM_HOST) {
        dm = at<double>(Wk, o_m);
        dw = at<double>(Wk, o_w);
        CK(cudaMemcpyAsync((void *)dm, mass, n * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    CK(gbp_launch_zheng07_wb(dm, at<float4>(Wk, o_lm), n, at<Zheng07F>(Wk, o_th), nth, dw, st));
    if (mem == GBP_MEM_HOST)
        CK(cudaMemcpyAsync(W, dw, (size_t)n * nth * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GBP_OK;
}

int gbp_zheng07_vjp_batched(gbp_plan *plan, const double *mass, int64_t n, const double *thetas,
                            int32_t nth, const double *grad_W, int32_t mem, double *grad_theta) {
    if (!plan) return GBP_ERR_INVALID;
    std::vector<Zheng07F> th;
    int rc = zheng07_batched_args(plan, thetas, nth, th);
    if (rc) return rc;
    if (!grad_theta || n < 0 || (n > 0 && (!mass || !grad_W)))
        return fail(plan, GBP_ERR_INVALID, "null arrays");
    for (int k = 0; k < 5 * nth; k++) grad_theta[k] = 0.0;
    if (n == 0) return GBP_OK;
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    Carve cv;
    size_t o_th = cv.take<Zheng07F>((size_t)nth);
    size_t o_out = cv.take<double>(5 * (size_t)nth);
    size_t o_lm = cv.take<float4>((size_t)n);
    size_t o_m = mem == GBP_MEM_HOST ? cv.take<double>((size_t)n) : 0;
    size_t o_g = mem == GBP_MEM_HOST ? cv.take<double>((size_t)n * nth) : 0;
    if ((rc = ensure_work(plan, cv.take<char>(0) + 256))) return rc;
    void *Wk = plan->work.p;
    CK(cudaMemcpyAsync(at<char>(Wk, o_th), th.data(), sizeof(Zheng07F) * nth, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(at<char>(Wk, o_out), 0, sizeof(double) * 5 * nth, st));
    const double *dm = mass, *dg = grad_W;
    if (mem == GBP_MEM_HOST) {
        dm = at<double>(Wk, o_m);
        dg = at<double>(Wk, o_g);
        CK(cudaMemcpyAsync((void *)dm, mass, n * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync((void *)dg, grad_W, (size_t)n * nth * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    CK(gbp_launch_zheng07_vjpb(dm, at<float4>(Wk, o_lm), n, at<Zheng07F>(Wk, o_th), nth, dg,
                               at<double>(Wk, o_out), st));
    CK(cudaMemcpyAsync(grad_theta, at<double>(Wk, o_out), sizeof(double) * 5 * nth, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GBP_OK;
}

int gbp_hod_mocks(gbp_plan *plan, const double *halo_xyz, const double *mass, const double *conc,
                  const double *rvir, int64_t n_halo, const double *thetas, int32_t n_theta,
                  double lbox, uint64_t seed, int32_t mem, float *gal_xyz, int64_t cap,
                  int64_t *offsets) {
    if (!plan) return GBP_ERR_INVALID;
    if (mem != GBP_MEM_HOST && mem != GBP_MEM_DEVICE) return fail(plan, GBP_ERR_INVALID, "bad memory kind");
    if (n_halo < 0 || n_theta < 1 || !thetas || !offsets ||
        (n_halo > 0 && (!halo_xyz || !mass || !conc || !rvir)))
        return fail(plan, GBP_ERR_INVALID, "null arrays or no parameter vector");
    if (n_halo > (int64_t)UINT32_MAX) return fail(plan, GBP_ERR_INVALID, "at most 2^32 - 1 halos");
    if (!(lbox > 0.0 && lbox < INFINITY)) return fail(plan, GBP_ERR_INVALID, "box size must be positive and finite");
    for (int m = 0; m < n_theta; m++) {
        const double *t = thetas + 5 * (size_t)m;
        if (!(t[1] > 0.0) || !std::isfinite(t[0]) || !std::isfinite(t[2]) || !std::isfinite(t[3]) ||
            !std::isfinite(t[4]))
            return fail(plan, GBP_ERR_INVALID, "theta %d: sigma_logM must be > 0 and all finite", m);
    }
    for (int m = 0; m <= n_theta; m++) offsets[m] = 0;
    if (n_halo == 0) return GBP_OK;
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    const int64_t items = n_halo * (int64_t)n_theta;
    if (items >= (int64_t)INT32_MAX) return fail(plan, GBP_ERR_INVALID, "too many (theta, halo) pairs");
    const size_t tb = gbp_hod_theta_bytes();
    Carve cv;
    size_t o_in = mem == GBP_MEM_HOST ? cv.take<double>(6 * (size_t)n_halo) : 0;
    size_t o_logm = cv.take<double>((size_t)n_halo);
    size_t o_th = cv.take<char>(tb * n_theta);
    size_t o_cnt = cv.take<int>((size_t)items + 1);
    size_t o_off = cv.take<int>((size_t)items + 1);
    size_t o_scan = cv.take<int>(gbp_scan_tmp_ints(items + 1));
    size_t o_gal = mem == GBP_MEM_HOST && gal_xyz ? cv.take<float>(3 * (size_t)std::max<int64_t>(cap, 1)) : 0;
    int rc = ensure_work(plan, cv.take<char>(0) + 256);
    if (rc) return rc;
    void *W = plan->work.p;
    const double *dxyz = halo_xyz, *dm = mass, *dc = conc, *dr = rvir;
    if (mem == GBP_MEM_HOST) {
        double *in = at<double>(W, o_in);
        CK(cudaMemcpyAsync(in, halo_xyz, 3 * n_halo * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(in + 3 * n_halo, mass, n_halo * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(in + 4 * n_halo, conc, n_halo * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(in + 5 * n_halo, rvir, n_halo * sizeof(double), cudaMemcpyHostToDevice, st));
        dxyz = in;
        dm = in + 3 * n_halo;
        dc = in + 4 * n_halo;
        dr = in + 5 * n_halo;
    }
    std::vector<char> th(tb * n_theta);
    gbp_hod_thetas(thetas, n_theta, th.data());
    CK(cudaMemcpyAsync(at<char>(W, o_th), th.data(), th.size(), cudaMemcpyHostToDevice, st));
    int *cnt = at<int>(W, o_cnt), *off = at<int>(W, o_off);
    CK(cudaMemsetAsync(cnt + items, 0, sizeof(int), st));
    CK(gbp_hod_count(dm, at<double>(W, o_logm), n_halo, at<char>(W, o_th), n_theta, seed, cnt, st));
    CK(gbp_scan_exclusive(cnt, off, items, at<int>(W, o_scan), st, nullptr));
    // per-mock offsets: the scan at the first halo of each parameter vector
    std::vector<int> hoff((size_t)n_theta + 1);
    for (int m = 0; m <= n_theta; m++)
        CK(cudaMemcpyAsync(&hoff[(size_t)m], off + (int64_t)m * n_halo, sizeof(int),
                           cudaMemcpyDeviceToHost, st));
    // the total in int64 from the scan's parts: the int32 offsets are only valid
    // while it stays below 2^31 and no count is negative
    const int *parts = nullptr;
    int64_t nparts = 0;
    gbp_scan_parts(cnt, items, at<int>(W, o_scan), &parts, &nparts);
    std::vector<int> hparts((size_t)std::max<int64_t>(nparts, 1));
    if (nparts > 0)
        CK(cudaMemcpyAsync(hparts.data(), parts, (size_t)nparts * sizeof(int),
                           cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int64_t sum = 0;
    bool neg = false;
    for (int64_t k = 0; k < nparts; k++) {
        neg |= hparts[(size_t)k] < 0;
        sum += hparts[(size_t)k];
    }
    if (neg || sum >= (int64_t)INT32_MAX)
        return fail(plan, GBP_ERR_INVALID,
                    "the draws give %lld galaxies in all, beyond the 2^31 - 1 the offsets hold",
                    (long long)sum);
    for (int m = 0; m <= n_theta; m++) offsets[m] = hoff[(size_t)m];
    const int64_t total = offsets[n_theta];
    if (!gal_xyz || cap < total || total == 0) return GBP_OK;  // offsets only
    float *dg = mem == GBP_MEM_HOST ? at<float>(W, o_gal) : gal_xyz;
    CK(gbp_hod_write(dxyz, dm, at<double>(W, o_logm), dc, dr, n_halo, at<char>(W, o_th), n_theta,
                     seed, off, lbox, dg, st));
    if (mem == GBP_MEM_HOST)
        CK(cudaMemcpyAsync(gal_xyz, dg, 3 * total * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GBP_OK;
}

int gbp_zheng07_weights(gbp_plan *plan, const double *mass, int64_t n, const double *theta,
                        int32_t mem, double *w) {
    if (!plan) return GBP_ERR_INVALID;
    Zheng07 th;
    int rc = zheng07_args(plan, theta, &th);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!mass || !w))) return fail(plan, GBP_ERR_INVALID, "null arrays");
    if (n == 0) return GBP_OK;
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    const double *dm = mass;
    double *dw = w;
    if (mem == GBP_MEM_HOST) {
        if ((rc = ensure_work(plan, 2 * n * sizeof(double) + 256))) return rc;
        dm = static_cast<double *>(plan->work.p);
        dw = static_cast<double *>(plan->work.p) + n;
        CK(cudaMemcpyAsync((void *)dm, mass, n * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    CK(gbp_launch_zheng07_w(dm, n, th, dw, st));
    if (mem == GBP_MEM_HOST) CK(cudaMemcpyAsync(w, dw, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GBP_OK;
}

int gbp_zheng07_vjp(gbp_plan *plan, const double *mass, int64_t n, const double *theta,
                    const double *grad_w, int32_t mem, double *grad_theta) {
    if (!plan) return GBP_ERR_INVALID;
    Zheng07 th;
    int rc = zheng07_args(plan, theta, &th);
    if (rc) return rc;
    if (!grad_theta || n < 0 || (n > 0 && (!mass || !grad_w)))
        return fail(plan, GBP_ERR_INVALID, "null arrays");
    CK(cudaSetDevice(plan->device));
    cudaStream_t st = plan->stream;
    size_t need = (mem == GBP_MEM_HOST ? 2 * (size_t)n : 0) * sizeof(double) + 8 * sizeof(double) + 512;
    if ((rc = ensure_work(plan, need))) return rc;
    double *out = static_cast<double *>(plan->work.p);
    const double *dm = mass, *dg = grad_w;
    if (mem == GBP_MEM_HOST) {
        double *buf = out + 8;
        dm = buf;
        dg = buf + n;
        if (n) {
            CK(cudaMemcpyAsync((void *)dm, mass, n * sizeof(double), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync((void *)dg, grad_w, n * sizeof(double), cudaMemcpyHostToDevice, st));
        }
    }
    CK(gbp_launch_zheng07_vjp(dm, n, th, dg, out, st));
    CK(cudaMemcpyAsync(grad_theta, out, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GBP_OK;
}

int gbp_measure_fp32_peak(gbp_plan *plan, double *tflops) {
    if (!plan || !tflops) return GBP_ERR_INVALID;
    CK(cudaSetDevice(plan->device));
    float ms = 0;
    double flops = 0;
    CK(gbp_run_ffma_probe(plan->nsm, plan->stream, &ms, &flops));
    *tflops = ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
    return GBP_OK;
}

}  // extern "C"
