/*
 * gbpairs — GB300 (sm_103a) pair-counting engines behind a plain C ABI.
 *
 * Drop-in replacement for the engines behind halotools'
 * mock_observables.pair_counters front-ends.  Every entry point takes plain
 * pointers and sizes, writes into caller-owned output buffers, keeps no
 * pointer after it returns, and reports failure through an int status
 * (GBP_OK == 0); gbp_plan_last_error() gives the message.
 *
 * Positions are (N, 3) row-major float64.  For non-periodic counts the caller
 * passes positions already shifted into their enclosing box together with that
 * box as `period` and pbc = 0 (halotools mesh_helpers.py:17-64 does this shift
 * in the front-end before any engine runs).  `mem` says where the position,
 * weight and output arrays live: GBP_MEM_HOST (pageable or pinned host memory)
 * or GBP_MEM_DEVICE (device pointers on the plan's GPU).  Bin edges are always
 * host arrays.  Passing the same pointer (and count) for sample 2 as for
 * sample 1 selects the auto-correlation path, which visits each unordered
 * pair once and counts it for both orders, exactly as the reference counts
 * ordered pairs (npairs_3d.py:26-29).
 */
#ifndef GBPAIRS_H
#define GBPAIRS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBP_OK 0
#define GBP_ERR_INVALID (-1)   /* bad argument (null pointer, size, edge array) */
#define GBP_ERR_CUDA (-2)      /* CUDA runtime error (launch, copy, device) */
#define GBP_ERR_NOMEM (-3)     /* device or host allocation failed */
#define GBP_ERR_RANGE (-4)     /* search length exceeds period/3, or positions out of the box */
#define GBP_ERR_NODEVICE (-5)  /* no CUDA device / wrong architecture */

#define GBP_MEM_HOST 0
#define GBP_MEM_DEVICE 1

typedef struct gbp_plan gbp_plan;

/* Execution statistics of the most recent call on a plan. */
typedef struct {
    int64_t candidate_pairs;  /* pairs whose FP32 distance was evaluated */
    int64_t recheck_pairs;    /* pairs re-evaluated in FP64 near a bin edge */
    int64_t cells[3];         /* grid the call used */
    int32_t reach;            /* stencil reach in cells */
    int32_t stencil_cells;    /* cells in the (pruned) stencil */
    int64_t work_items;       /* (cell, point-chunk) items of the count kernel */
    float ms_build;           /* device time of the cell-list build */
    float ms_count;           /* device time of the pair-count kernel */
    float ms_total;           /* device time of the whole call incl. copies */
    int32_t count_launches;   /* launches of the pair-count kernel in the call */
    int32_t kernel_launches;  /* all kernel launches of the call */
    int64_t h2d_bytes;        /* host-to-device bytes copied by the call */
    int64_t d2h_bytes;        /* device-to-host bytes copied by the call */
    int32_t block;            /* fine cells per block edge of the two-level grid (1: plain cells) */
    int32_t reserved;
} gbp_stats;

/* Plan: a CUDA stream, cached device workspace and statistics. Not
 * thread-safe; distinct plans may be used from distinct host threads. */
int gbp_plan_create(int device, gbp_plan **plan);
int gbp_plan_destroy(gbp_plan *plan);
/* Use an existing cudaStream_t (NULL = the plan's own stream). */
int gbp_plan_set_stream(gbp_plan *plan, void *cuda_stream);
/* Force the stencil reach (1..4 cells per search length); 0 = automatic. */
int gbp_plan_set_reach(gbp_plan *plan, int reach);
/* Force the block factor of the two-level grid (1..4 fine cells per block
 * edge; 1 = plain cell list); 0 = automatic (blocks for sparse samples; for
 * dense npairs_3d and npairs_s_mu samples, reach 4 in blocks of 2). */
int gbp_plan_set_block(gbp_plan *plan, int block);
/* The cell grid a call would choose, computed on the host without a GPU (no
 * reference counterpart: the reference's mesh is RectangularDoubleMesh,
 * rectangular_mesh.py:228, which the GPU grid replaces).  kind: 0 npairs_3d
 * (up to 64 edges), 1 npairs_s_mu, 2 npairs_xy_z; search3: the largest
 * separation searched per dimension (each at most a third of the period);
 * n2: points of sample 2; reach, block: the plan's hints (0 = automatic).
 * out[0..6] = reach, block factor, fine cells per dimension (3), stencil runs,
 * block reach.  GBP_ERR_RANGE for a search longer than a third of the box. */
int gbp_grid_describe(const double *period3, int32_t pbc, const double *search3, int64_t n2,
                      int32_t kind, int32_t reach, int32_t block, int32_t *out);
/* The FP32 guard thresholds an npairs_3d call (up to 64 edges) compares its
 * FP32 squared separations with, computed on the host without a GPU (no
 * reference counterpart; for tests of the error bound).  The grid is the one
 * gbp_grid_describe gives for kind 0 with search = max(rbins); the squared
 * edges are walked from the top as npairs_3d_engine.pyx:178-182 does; then
 * v32 <= lo[k] proves v64 <= rbins[k]^2 and v32 > hi[k] proves v64 > rbins[k]^2
 * for the FP32 value v32 the count kernel forms from the grid's cell offsets.
 * cell3: the fine cell size per dimension. */
int gbp_npairs_3d_thresholds(const double *period3, int32_t pbc, const double *rbins, int32_t nb,
                             int64_t n2, int32_t reach, int32_t block, float *hi, float *lo,
                             double *cell3);
/* The same for npairs_xy_z (no reference counterpart): the grid of
 * gbp_grid_describe for kind 2, and the thresholds of the rp axis (v = dx^2 +
 * dy^2 against rp_bins^2) and of the pi axis (v = dz^2 against pi_bins^2), the
 * edges walked from the top as npairs_xy_z_engine.pyx:183-194 does. */
int gbp_npairs_xy_z_thresholds(const double *period3, int32_t pbc, const double *rp_bins,
                               int32_t n_rp, const double *pi_bins, int32_t n_pi, int64_t n2,
                               int32_t reach, int32_t block, float *hi_rp, float *lo_rp,
                               float *hi_pi, float *lo_pi, double *cell3);
/* The float-bit lookup table an npairs_3d call bins with (no reference
 * counterpart; for tests of the table): lut receives info[0] = T slots of 4
 * floats {first bin (int bits), upper threshold, lower threshold, unused}
 * (room for 1024 slots), info[1..2] = the right shift S and the first slot's
 * shifted bits B, vrange = the clamp range {vlo, vhi}.  A value v falls in slot
 * (bits(clamp(v)) >> S) - B; its bin is b0 + (v > upper), and the pair is
 * rechecked when lower < v <= upper. */
int gbp_npairs_3d_lut(const double *period3, int32_t pbc, const double *rbins, int32_t nb,
                      int64_t n2, int32_t reach, int32_t block, float *lut, int32_t *info,
                      float *vrange);
/* The stencil of the grid gbp_grid_describe gives (no reference counterpart;
 * for tests of its pruning): per run 5 ints {block offset x, y, z, first fine
 * cell, fine cells} into runs (room for 729 runs), their number into nruns.
 * A fine cell (lx, ly, lz) of a block is (lx * bf + ly) * bf + lz.  With
 * autocorr only the own block and the lexicographically positive block offsets
 * are listed (each unordered block pair once). */
int gbp_stencil_describe(const double *period3, int32_t pbc, const double *search3, int64_t n2,
                         int32_t kind, int32_t reach, int32_t block, int32_t autocorr,
                         int32_t *runs, int32_t *nruns);
/* The binning tables of an npairs_s_mu auto-correlation, computed on the host
 * without a GPU (no reference counterpart; for tests of the (s, mu') error
 * bounds).  s_lut / q_lut receive the float-bit tables of s^2 and of
 * q = mu'^2 = dxy / s^2 as gbp_npairs_3d_lut does (the s slots carry, in their
 * 4th float, the bound on the error of the FP32 quotient q for every s^2 of the
 * slot); s_hi / s_lo (n_s) and q_hi / q_lo (n_mu) the thresholds of the
 * differential edges that the strict walks of npairs_s_mu_engine.pyx:198-226
 * define; info = {T, S, B} of s, then of q; vrange = {vlo, vhi} of s, then of
 * q; cell3 the fine cell size per dimension. */
int gbp_npairs_s_mu_tables(const double *period3, int32_t pbc, const double *s_bins, int32_t n_s,
                           const double *mu_prime, int32_t n_mu, int64_t n2, int32_t reach,
                           int32_t block, float *s_lut, float *s_hi, float *s_lo, float *q_lut,
                           float *q_hi, float *q_lo, int32_t *info, float *vrange, double *cell3);
/* 1: capture each call's stream work into one CUDA graph (instantiated once,
 * updated in place on later calls) and launch that; 0: launch directly. */
int gbp_plan_set_graph(gbp_plan *plan, int enable);
/* 1: on the first call of a new workload shape, time every feasible reach and
 * keep the fastest for later calls of that shape; 0: density heuristic. */
int gbp_plan_set_autotune(gbp_plan *plan, int enable);
/* Capacity limits, for exercising rare paths on small inputs (no reference
 * counterpart).  first_item_cap > 0: the next call starts with room for that
 * many work items, so a denser workload overflows it and the call repeats with
 * room for its estimate (the path a large clustered sample takes); 0 = the
 * estimate.  flush_after > 0: a warp of the count kernel moves its 32-bit
 * histogram words to the 64-bit totals at the end of the first work item
 * after it has binned more than flush_after / 64 j-batches since its last
 * move (default 2^24, long before a word could wrap); 0 = default. */
int gbp_plan_set_limits(gbp_plan *plan, int64_t first_item_cap, int64_t flush_after);
const char *gbp_plan_last_error(const gbp_plan *plan);
int gbp_plan_stats(const gbp_plan *plan, gbp_stats *stats);

/*
 * Cumulative 3-D pair counts: counts[k] = #ordered pairs (i, j) whose FP64
 * squared separation satisfies the reference's walk from the top edge down,
 * i.e. dsq <= rbins[m]^2 for every m >= k.
 * Replaces npairs_3d_engine (cpairs/npairs_3d_engine.pyx:17-184) and the
 * mesh/Pool fan-out of npairs_3d (npairs_3d.py:112-150).
 */
int gbp_npairs_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                  int64_t n2, const double *rbins, int32_t nbins, const double *period3,
                  int32_t pbc, int32_t mem, int64_t *counts);

/*
 * Batched auto-correlation counts of many samples ("mocks", e.g. HOD
 * realisations on one halo catalogue) in one cell-list build and one
 * persistent count launch over a shared grid: counts[m][k] equals
 * gbp_npairs_3d of mock m alone.  Sample m is rows offsets[m] ..
 * offsets[m+1]-1 of xyz ((N, 3), float64, or float32 if xyz_f32 = 1, which
 * the reference upcasts exactly, npairs_3d_engine.pyx:58-63); offsets is a
 * host array of nmocks+1 non-decreasing entries from 0 to N.  No reference
 * counterpart as one call: it replaces nmocks calls of npairs_3d
 * (npairs_3d.py:20), e.g. the loop marked_tpcf.py:327-345 runs.
 */
int gbp_batched_npairs_3d(gbp_plan *plan, const void *xyz, int32_t xyz_f32, const int64_t *offsets,
                          int32_t nmocks, const double *rbins, int32_t nbins,
                          const double *period3, int32_t pbc, int32_t mem, int64_t *counts);

/*
 * Cumulative (r_p, pi) counts, row-major [n_rp][n_pi].
 * Replaces npairs_xy_z_engine (cpairs/npairs_xy_z_engine.pyx:17-196) and
 * npairs_xy_z (npairs_xy_z.py:124-163).
 */
int gbp_npairs_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                    int64_t n2, const double *rp_bins, int32_t n_rp, const double *pi_bins,
                    int32_t n_pi, const double *period3, int32_t pbc, int32_t mem,
                    int64_t *counts);

/*
 * Cumulative (s, mu') counts, row-major [n_s][n_mu], where mu_prime is
 * sort(sin(arccos(mu_bins))) as prepared by npairs_s_mu.py:174-175.
 * Replaces npairs_s_mu_engine (cpairs/npairs_s_mu_engine.pyx:18-236).
 */
int gbp_npairs_s_mu(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                    int64_t n2, const double *s_bins, int32_t n_s, const double *mu_prime,
                    int32_t n_mu, const double *period3, int32_t pbc, int32_t mem,
                    int64_t *counts);

/*
 * Cumulative weighted counts for marking function `wfunc_id` (1..17) with
 * `nw` weights per point, weights as (N, nw) row-major float64.
 * Replaces marked_npairs_3d_engine (marked_cpairs/marked_npairs_3d_engine.pyx:22-218).
 */
int gbp_marked_npairs_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                         int64_t n2, const double *w1, const double *w2, int32_t nw,
                         int32_t wfunc_id, const double *rbins, int32_t nbins,
                         const double *period3, int32_t pbc, int32_t mem, double *out);

/*
 * gbp_weighted_adjoint_3d for nch <= 16 weight channels at once (parameter
 * draws of an occupation model): w is (n, nch) row-major, gbar (nch, nbins),
 * grad_w (n, nch) with grad_w[m][c] = dL/dw_m of channel c for the forward
 * counts gbp_marked_npairs_3d_channels(x, x, w, w).  Each pair is binned once
 * for all channels (up to 8 channels: two i-points per lane; 9-16: one).
 */
int gbp_weighted_adjoint_3d_channels(gbp_plan *plan, const double *xyz, int64_t n,
                                     const double *w, int32_t nch, const double *rbins,
                                     int32_t nb, const double *period3, int32_t pbc, int32_t mem,
                                     const double *gbar, double *grad_w);

/*
 * gbp_zheng07_weights and gbp_zheng07_vjp for nth parameter vectors at once
 * (thetas (nth, 5)): W (n, nth) row-major, grad_W likewise, grad_theta (nth, 5)
 * on the host.  The occupations are evaluated in FP32 (the counting kernels
 * multiply weights in FP32) from hi + lo float splits of the FP64 log10 M and M;
 * the VJP terms are FP32, summed with compensation per lane and in FP64 across
 * lanes.
 */
int gbp_zheng07_weights_batched(gbp_plan *plan, const double *mass, int64_t n,
                                const double *thetas, int32_t nth, int32_t mem, double *W);
int gbp_zheng07_vjp_batched(gbp_plan *plan, const double *mass, int64_t n, const double *thetas,
                            int32_t nth, const double *grad_W, int32_t mem, double *grad_theta);

/*
 * Zheng07 HOD mocks on the GPU, one per parameter vector thetas[m] =
 * (logMmin, sigma_logM, logM0, logM1, alpha), (n_theta, 5) row-major: a
 * Bernoulli central with <Ncen> = (1 + erf((log10 M - logMmin) / sigma_logM)) / 2
 * at the halo centre and a Poisson number of satellites with <Nsat> =
 * ((M - 10^logM0) / 10^logM1)^alpha at NFW radii (concentration conc, radius
 * rvir) in isotropic directions, wrapped into [0, lbox) (zheng07_components.py:
 * 149-153, 455-470; population as hod_mock_factory.py:196-401 does it).  Draws
 * are Philox4x32-10 counters of (halo, m, draw) under `seed`, so a mock is fixed
 * by its inputs.  offsets[0..n_theta]: mock m is rows [offsets[m], offsets[m+1])
 * of gal_xyz, (offsets[n_theta], 3) float32.  With gal_xyz NULL or cap (rows)
 * below the total, only offsets are written: call again with a buffer of
 * offsets[n_theta] rows.  mem: all arrays on the host or all on the device
 * (offsets always on the host).  GBP_ERR_INVALID (offsets left 0) when the
 * draws give 2^31 - 1 galaxies or more in all.
 */
int gbp_hod_mocks(gbp_plan *plan, const double *halo_xyz, const double *mass, const double *conc,
                  const double *rvir, int64_t n_halo, const double *thetas, int32_t n_theta,
                  double lbox, uint64_t seed, int32_t mem, float *gal_xyz, int64_t cap,
                  int64_t *offsets);

/*
 * Condition a neighbour pair (i, j) must meet besides its separation.
 * kind 0: none.  kind 1: the mass fraction of counts_in_cylinders
 * (counts_in_cells/engines/conditions/conditions.pyx, MassFrac.func):
 * f = marks2[j] / marks1[i] (1 when both are 0, inf when only marks1[i] is)
 * within (lim[0], lim[1]), each bound inclusive when its flag is set; nmarks 1.
 * kind 2: marking function `func` 0..6 of the conditional isolation functions
 * (isolation_functions/engines/isolation_criteria_marking_functions.pyx) on
 * (n, nmarks) row-major FP64 marks, nmarks 1 or 2.  Marks in caller order.
 */
typedef struct {
    int32_t kind;
    int32_t func;
    const double *marks1;
    const double *marks2;
    int32_t nmarks;
    int32_t lower_inclusive;
    int32_t upper_inclusive;
    int32_t reserved;
    double lim[2];
} gbp_neigh_cond;

/*
 * counts[i] = number of sample-2 points j with dx^2 + dy^2 < rp[i]^2 and
 * dz^2 < pi[i]^2 (strict, FP64 in the reference's order, radii squared in
 * FP64) that meet `cond` (NULL: none).  Replaces counts_in_cylinders_engine
 * (counts_in_cells/engines/counts_in_cylinders_engine.pyx:255-281) and the
 * mesh and Pool fan-out of counts_in_cylinders (counts_in_cylinders.py:27-195);
 * the front-end subtracts the self match for its auto-correlation.  Host
 * memory; rp, pi per sample-1 point.
 */
int gbp_counts_in_cylinders(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                            int64_t n2, const double *rp, const double *pi,
                            const double *period3, int32_t pbc, const gbp_neigh_cond *cond,
                            int64_t *counts);

/*
 * The pairs behind gbp_counts_in_cylinders' counts (its return_indexes):
 * given those counts, writes (i1, i2) caller indices, 2 x sum(counts) uint32,
 * the pairs of point i in slots [sum(counts[:i]), sum(counts[:i+1])) in no
 * particular order.
 */
int gbp_cylinder_pairs(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                       int64_t n2, const double *rp, const double *pi, const double *period3,
                       int32_t pbc, const gbp_neigh_cond *cond, const int64_t *counts,
                       uint32_t *pairs);

/*
 * is_isolated[i] = 1 when no sample-2 point lies at separation > 0 inside
 * point i's sphere (pi == NULL: s^2 < r[i]^2) or cylinder (dx^2 + dy^2 <
 * r[i]^2 and dz^2 < pi[i]^2) while meeting `cond` (NULL, or kind 2).
 * Replaces spherical_isolation_engine, cylindrical_isolation_engine and their
 * marked forms (isolation_functions/engines/*_isolation_engine.pyx).
 */
int gbp_isolation(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                  const double *r, const double *pi, const double *period3, int32_t pbc,
                  const gbp_neigh_cond *cond, uint8_t *is_isolated);

/*
 * Jackknife (r_p, pi) pair counts, as npairs_jackknife_xy_z
 * (npairs_jackknife_xy_z.py:23-26, engine npairs_jackknife_xy_z_engine.pyx:231-281)
 * without weights: out[0][k][g] is the cumulative count, out[s][k][g]
 * (s = 1..n_samples) the count with subsample s removed, a pair with one end in
 * s counting one half.  jtags in [1, n_samples], n_samples <= 32767; positions
 * and tags in host memory; out is (n_samples + 1, n_rp, n_pi) FP64.
 */
int gbp_npairs_jackknife_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                              int64_t n2, const int32_t *jtags1, const int32_t *jtags2,
                              int32_t n_samples, const double *rp_bins, int32_t n_rp,
                              const double *pi_bins, int32_t n_pi, const double *period3,
                              int32_t pbc, int32_t mem, double *out);

/*
 * Weighted jackknife counts, as npairs_jackknife_3d / npairs_jackknife_xy_z with
 * weights (jweight in npairs_jackknife_3d_engine.pyx and
 * npairs_jackknife_xy_z_engine.pyx:250-281): row 0 sums w1_i w2_j over the
 * ordered pairs in each cumulative bin, row s leaves out the pairs with both
 * ends in subsample s and counts those with one end there at one half.  One FP64
 * weight and one tag per point; host memory; out (n_samples + 1, nbins) or
 * (n_samples + 1, n_rp, n_pi).  Sums in FP32 with an exact-error companion and an
 * FP64 (tag, bin) table: within 1e-6 relative of the FP64 reference for
 * non-negative weights.
 */
int gbp_npairs_jackknife_3d_weighted(gbp_plan *plan, const double *xyz1, int64_t n1,
                                     const double *xyz2, int64_t n2, const double *w1,
                                     const double *w2, const int32_t *jtags1,
                                     const int32_t *jtags2, int32_t n_samples,
                                     const double *rbins, int32_t nb, const double *period3,
                                     int32_t pbc, int32_t mem, double *out);
int gbp_npairs_jackknife_xy_z_weighted(gbp_plan *plan, const double *xyz1, int64_t n1,
                                       const double *xyz2, int64_t n2, const double *w1,
                                       const double *w2, const int32_t *jtags1,
                                       const int32_t *jtags2, int32_t n_samples,
                                       const double *rp_bins, int32_t n_rp, const double *pi_bins,
                                       int32_t n_pi, const double *period3, int32_t pbc,
                                       int32_t mem, double *out);

/*
 * Cumulative (r_p, pi) sums of marking function `wfunc_id` (1..17), row-major
 * [n_rp][n_pi]: out[k][g] adds wfunc(w1_i, w2_j) over ordered pairs with
 * dxy^2 <= rp_bins[k]^2 and dz^2 <= pi_bins[g]^2.  Weights (N, nw) row-major
 * FP64; nw as for gbp_marked_npairs_3d.  Replaces marked_npairs_xy_z_engine
 * (marked_cpairs/marked_npairs_xy_z_engine.pyx:23-229, pair loop :209-224) and
 * marked_npairs_xy_z (marked_npairs_xy_z.py:160-189).  Sums are FP32 with an
 * exact-error companion, moved to FP64 every few thousand pairs.
 */
int gbp_marked_npairs_xy_z(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                           int64_t n2, const double *w1, const double *w2, int32_t nw,
                           int32_t wfunc_id, const double *rp_bins, int32_t n_rp,
                           const double *pi_bins, int32_t n_pi, const double *period3,
                           int32_t pbc, int32_t mem, double *out);

/*
 * Cumulative (s, mu') counts and w1 * w2 sums, both row-major [n_s][n_mu], with
 * mu_prime = sort(sin(arccos(mu_bins))) (weighted_npairs_s_mu.py:192-193) and
 * one FP64 weight per point.  Replaces weighted_npairs_s_mu_engine
 * (cpairs/weighted_npairs_s_mu_engine.pyx:15-256) and weighted_npairs_s_mu
 * (weighted_npairs_s_mu.py:175-230).
 */
int gbp_weighted_npairs_s_mu(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                             int64_t n2, const double *w1, const double *w2,
                             const double *s_bins, int32_t n_s, const double *mu_prime,
                             int32_t n_mu, const double *period3, int32_t pbc, int32_t mem,
                             int64_t *counts, double *wcounts);

/*
 * Product-mark counts over nch channels in one pass (no single reference
 * counterpart): out[c][k] equals marked_npairs_3d(xyz1, xyz2, rbins, 1,
 * weights1=w1[:, c], weights2=w2[:, c]) (marked_npairs_3d.py:25,
 * marking_functions.pyx:36-43), e.g. the random-mark draws of marked_tpcf
 * (marked_tpcf.py:327-345) or the components of a vector mark. w1, w2: (n, nch)
 * row-major FP64; every pair is binned once and each channel's product is
 * accumulated in FP32 Kahan pairs. nch <= 32; out is (nch, nbins).
 */
int gbp_marked_npairs_3d_channels(gbp_plan *plan, const double *xyz1, int64_t n1,
                                  const double *xyz2, int64_t n2, const double *w1,
                                  const double *w2, int32_t nch, const double *rbins,
                                  int32_t nbins, const double *period3, int32_t pbc, int32_t mem,
                                  double *out);

/*
 * Jackknife pair counts, as npairs_jackknife_3d (npairs_jackknife_3d.py:29-31,
 * engine npairs_jackknife_3d_engine.pyx) without weights: out[0][k] is the
 * cumulative count, out[s][k] (s = 1..n_samples) the count with subsample s
 * removed, a pair with one end in s counting one half. jtags in [1, n_samples];
 * positions and tags in host memory; out is (n_samples + 1, nbins) FP64.
 */
int gbp_npairs_jackknife_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                            int64_t n2, const int32_t *jtags1, const int32_t *jtags2,
                            int32_t n_samples, const double *rbins, int32_t nbins,
                            const double *period3, int32_t pbc, int32_t mem, double *out);

/*
 * Per-object counts, as npairs_per_object_3d (npairs_per_object_3d.py:20-21,
 * engine npairs_per_object_3d_engine.pyx): counts[i][k] = number of points j of
 * sample 2 with (FP64, reference order) d_ij^2 <= rbins[k]^2, self pairs
 * included; counts is (n1, nbins) int64 in sample 1's order, host memory.
 */
int gbp_npairs_per_object_3d(gbp_plan *plan, const double *xyz1, int64_t n1, const double *xyz2,
                             int64_t n2, const double *rbins, int32_t nbins,
                             const double *period3, int32_t pbc, int32_t mem, int64_t *counts);

/*
 * Reverse pass of occupation-weighted counts, no reference counterpart
 * (halotools has no gradients).  For the forward
 * gbp_marked_npairs_3d(xyz, xyz, w, w, 1 weight, wfunc 1) =
 * C_k = sum_ij w_i w_j [d_ij <= r_k] and an upstream gradient gbar[k]
 * (host, nbins), writes grad_w[m] = dL/dw_m = sum_j w_j (G(d_mj) + G(d_jm)),
 * G(d) = sum_{k: d <= r_k} gbar[k], in the caller's order.  xyz (n, 3), w (n)
 * and grad_w (n) live in `mem` memory.
 */
int gbp_weighted_adjoint_3d(gbp_plan *plan, const double *xyz, int64_t n, const double *w,
                            const double *rbins, int32_t nbins, const double *period3,
                            int32_t pbc, int32_t mem, const double *gbar, double *grad_w);

/*
 * Zheng07 occupation weights w = <Ncen> + <Nsat> per halo mass M
 * (zheng07_components.py:149-153 and 455-470, satellites not modulated by the
 * central occupation), theta = (logMmin, sigma_logM, logM0, logM1, alpha)
 * (host array of 5), and the vector-Jacobian product
 * grad_theta = sum_m grad_w[m] dw_m/dtheta (host array of 5).
 */
int gbp_zheng07_weights(gbp_plan *plan, const double *mass, int64_t n, const double *theta,
                        int32_t mem, double *w);
int gbp_zheng07_vjp(gbp_plan *plan, const double *mass, int64_t n, const double *theta,
                    const double *grad_w, int32_t mem, double *grad_theta);

/*
 * Allocation-free npairs_3d.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory while they count (a process
 * whose device memory belongs to another framework's caching allocator, or a
 * latency-critical loop where cudaMalloc/cudaFree would synchronise the
 * device).  Same counts as gbp_npairs_3d for an auto-correlation
 * (sample 2 == sample 1), but every scratch buffer lives in one static
 * device array of GBP_STATIC_SCRATCH_BYTES that each GPU loading this
 * library holds until exit; the call allocates nothing, device or host.
 *   xyz     device pointer, (n, 3) row-major float64, 1 <= n <= GBP_STATIC_MAX_POINTS
 *   rbins   host array of 2..64 edges; period3 host array
 *   pbc     1: periodic box of sides period3; 0: no wrap, the points lie in
 *           the box [0, period3] (not shifted by their minimum as the
 *           period=None front-ends do); either way the largest edge must be
 *           at most period3 / 3
 *   counts  device pointer to n_bins int64, written by the last kernel of the
 *           call.  All counts are -1 (the call still returns GBP_OK, since
 *           it does not wait for its kernels) when a position lies outside
 *           [0, period3] or is not finite, or when the input needs more work
 *           items than the array holds (a sample far more clustered than
 *           GBP_STATIC_MAX_POINTS points spread over GBP_STATIC_MAX_CELLS
 *           cells can produce)
 *   stream  cudaStream_t (NULL = legacy default stream); the call does not
 *           synchronise it
 * Larger inputs return GBP_ERR_INVALID, and so does a stream that is being
 * captured (each call copies its bin tables from host memory).  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  The address is kept for the life of the
 * process: calls after a cudaDeviceReset are not supported.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised.
 */
#define GBP_STATIC_MAX_POINTS 131072
#define GBP_STATIC_MAX_CELLS 131072
#define GBP_STATIC_SCRATCH_BYTES (16u << 20)
int gbp_npairs_3d_static(const double *xyz, int64_t n, const double *rbins, int32_t nbins,
                         const double *period3, int32_t pbc, int64_t *counts, void *stream);

/*
 * Measurement utility with no counterpart in the reference: runs a dependent-
 * chain FFMA kernel on the plan's GPU and returns the FP32 FMA throughput in
 * TFLOP/s (2 flops per FFMA), the ceiling of the count kernels' FP32 pipe.
 */
int gbp_measure_fp32_peak(gbp_plan *plan, double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* GBPAIRS_H */
