/*
 * CPU restatement of halotools' pair-counting engines.
 *
 * TEST INFRASTRUCTURE: this is the oracle the CUDA path is checked against and
 * the CPU baseline that the benchmark times beside it.  It is never linked
 * into, or called by, the library's product path.
 *
 * It restates, in plain C, the reference's double mesh and its cell walks:
 *   - sample1_cell_size / sample2_cell_sizes / RectangularMesh
 *     (halotools mock_observables/pair_counters/rectangular_mesh.py:19-225)
 *   - npairs_3d_engine     (cpairs/npairs_3d_engine.pyx:103-184)
 *   - npairs_xy_z_engine   (cpairs/npairs_xy_z_engine.pyx:143-196)
 *   - npairs_s_mu_engine   (cpairs/npairs_s_mu_engine.pyx:150-236)
 *   - marked_npairs_3d_engine and the 17 marking functions
 *     (marked_cpairs/marked_npairs_3d_engine.pyx:150-218,
 *      marked_cpairs/marking_functions.pyx:21-218)
 * The outer cell1 loop is split into contiguous ranges over POSIX threads,
 * as the reference splits it over processes (mesh_helpers.py:183-221).
 *
 * Arithmetic: every squared distance is evaluated left to right and unfused,
 * ((dx*dx + dy*dy) + dz*dz) with dx = (x1 - shift) - x2, which is what the
 * reference's -Ofast build does on x86-64 (checked against its golden
 * vectors).  Build with -ffp-contract=off so no FMA is formed.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXCELLS_PER_DIM 50 /* rectangular_mesh.py:15-16 */

/* numpy's float floor_divide (npy_divmod), used by digitized_position. */
static double npy_floor_divide(double a, double b) {
    double mod = fmod(a, b);
    if (b == 0.0) return a / b;
    double div = (a - mod) / b;
    if (mod != 0.0) {
        if ((b < 0) != (mod < 0)) div -= 1.0;
    }
    double floordiv;
    if (div != 0.0) {
        floordiv = floor(div);
        if (div - floordiv > 0.5) floordiv += 1.0;
    } else {
        floordiv = copysign(0.0, a / b);
    }
    return floordiv;
}

/* rectangular_mesh.py:25-55 */
static double sample1_cell_size(double period, double search, double approx) {
    long ndivs = (long)floor(period / approx);
    if (ndivs < 1) ndivs = 1;
    if (ndivs > MAXCELLS_PER_DIM) ndivs = MAXCELLS_PER_DIM;
    long nsearch = (long)floor(period / search);
    if (nsearch < 1) nsearch = 1;
    if (nsearch < ndivs) ndivs = nsearch;
    if (ndivs < 3) ndivs = 3;
    return period / (double)ndivs;
}

/* rectangular_mesh.py:58-82; np.round rounds half to even, as nearbyint does */
static double sample2_cell_sizes(double period, double cell1, double approx) {
    long n1 = (long)nearbyint(period / cell1);
    long d = (long)nearbyint(cell1 / approx);
    if (d < 1) d = 1;
    if (d > MAXCELLS_PER_DIM) d = MAXCELLS_PER_DIM;
    long n2 = n1 * d;
    if (n2 > MAXCELLS_PER_DIM) {
        long per = MAXCELLS_PER_DIM / n1;
        n2 = per * n1;
    }
    return period / (double)n2;
}

typedef struct {
    int n[3];
    double cell[3];
    int64_t ncells;
    int64_t *start;   /* CSR offsets, ncells+1 */
    int64_t *order;   /* sorted position -> original index */
} mesh_t;

/* RectangularMesh.__init__ (rectangular_mesh.py:118-222); a stable counting
 * sort stands in for argsort, which changes only the order within a cell. */
static int mesh_build(mesh_t *m, const double *xyz, int64_t npts,
                      const double period[3], const double approx[3]) {
    for (int d = 0; d < 3; d++) {
        long nd = (long)nearbyint(period[d] / approx[d]);
        if (nd < 1) nd = 1;
        m->n[d] = (int)nd;
        m->cell[d] = period[d] / (double)nd;
    }
    m->ncells = (int64_t)m->n[0] * m->n[1] * m->n[2];
    m->start = (int64_t *)calloc((size_t)m->ncells + 1, sizeof(int64_t));
    m->order = (int64_t *)malloc((size_t)(npts > 0 ? npts : 1) * sizeof(int64_t));
    int64_t *cid = (int64_t *)malloc((size_t)(npts > 0 ? npts : 1) * sizeof(int64_t));
    if (!m->start || !m->order || !cid) { free(cid); return -1; }
    for (int64_t i = 0; i < npts; i++) {
        int64_t ip[3];
        for (int d = 0; d < 3; d++) {
            double q = floor(npy_floor_divide(xyz[3 * i + d], m->cell[d]));
            int64_t v = (int64_t)q;
            if (v >= m->n[d]) v = m->n[d] - 1;
            ip[d] = v;
        }
        int64_t c = ip[0] * ((int64_t)m->n[1] * m->n[2]) + ip[1] * m->n[2] + ip[2];
        /* ids outside [0, ncells) fall outside every CSR range, as with searchsorted */
        cid[i] = c;
        if (c >= 0 && c < m->ncells) m->start[c + 1]++;
    }
    for (int64_t c = 0; c < m->ncells; c++) m->start[c + 1] += m->start[c];
    int64_t *fill = (int64_t *)malloc((size_t)m->ncells * sizeof(int64_t) + 8);
    if (!fill) { free(cid); return -1; }
    memcpy(fill, m->start, (size_t)m->ncells * sizeof(int64_t));
    for (int64_t i = 0; i < npts; i++) {
        int64_t c = cid[i];
        if (c >= 0 && c < m->ncells) m->order[fill[c]++] = i;
    }
    free(fill);
    free(cid);
    return 0;
}

static void mesh_free(mesh_t *m) {
    free(m->start);
    free(m->order);
}

enum { K_3D = 0, K_XYZ = 1, K_SMU = 2, K_MARKED = 3, K_XYZ_MARKED = 4, K_SMU_WEIGHTED = 5,
       K_XYZ_JACK = 6, K_NEIGH = 7, K_3D_JACK = 8, K_WPOBJ = 9 };

typedef struct {
    int kind;
    mesh_t m1, m2;
    int steps[3], per[3];
    double period[3];
    int pbc;
    /* sorted SoA copies (npairs_3d_engine.pyx:58-63) */
    double *x1, *y1, *z1, *x2, *y2, *z2;
    double *w1, *w2;
    int nw, wfunc;
    int64_t *t1, *t2; /* jackknife tags, sorted like the positions */
    int nsamp;
    /* per-object neighbours: rows of w1 are {r or rp, pi, marks}, of w2 {0, 0, marks} */
    int geo, excl0, ckind, cfunc, ceq0, ceq1;
    double clim0, clim1;
    /* squared bin edges */
    const double *e1;
    int n1e;
    const double *e2;
    int n2e;
    double smax2, mumax2;
} walk_t;

typedef struct {
    const walk_t *w;
    int64_t c0, c1;
    int64_t *icounts;
    double *dcounts;
} job_t;

/* npairs_jackknife_xy_z_engine.pyx:250-281: weight of a pair in row j */
static double jweight(int64_t j, int64_t j1, int64_t j2, double w1, double w2) {
    if (j == 0) return w1 * w2;
    if (j1 == j2 && j1 == j) return 0.0;
    if (j1 != j && j2 != j) return w1 * w2;
    return 0.5 * (w1 * w2);
}

/* conditions.pyx MassFrac.func (counts_in_cylinders' "mass_frac") */
static int mass_frac_ok(const walk_t *w, double m1, double m2) {
    double f;
    if (m1 == 0.0) f = (m2 == 0.0) ? 1.0 : INFINITY;
    else f = m2 / m1;
    int t1 = w->ceq0 ? (w->clim0 <= f) : (w->clim0 < f);
    int t2 = w->ceq1 ? (f <= w->clim1) : (f < w->clim1);
    return t1 && t2;
}

/* isolation_criteria_marking_functions.pyx:30-136 */
static int iso_cond(int id, const double *a, const double *b) {
    switch (id) {
    case 0: return 1;
    case 1: return a[0] > b[0];
    case 2: return a[0] < b[0];
    case 3: return a[0] == b[0];
    case 4: return a[0] != b[0];
    case 5: return a[0] > (b[0] + a[1]);
    case 6: return a[0] < (b[0] + a[1]);
    default: return 0;
    }
}

/* marking_functions.pyx:21-218 (ids 1-17); id 0 is the custom hook, zero. */
static double wfunc_eval(int id, const double *a, const double *b) {
    switch (id) {
    case 1: return a[0] * b[0];
    case 2: return a[0] + b[0];
    case 3: return (a[0] == b[0]) ? a[1] * b[1] : 0.0;
    case 4: return (a[0] != b[0]) ? a[1] * b[1] : 0.0;
    case 5: return (b[0] > a[0]) ? a[1] * b[1] : 0.0;
    case 6: return (b[0] < a[0]) ? a[1] * b[1] : 0.0;
    case 7: return (b[0] > (a[0] + a[1])) ? b[1] : 0.0;
    case 8: return (b[0] < (a[0] + a[1])) ? b[1] : 0.0;
    case 9: return (fabs(a[0] - b[0]) < a[1]) ? b[1] : 0.0;
    case 10: return (fabs(a[0] - b[0]) > a[1]) ? b[1] : 0.0;
    case 11: return (b[0] > a[0] * a[1]) ? b[1] : 0.0;
    case 12: return a[0] * b[0] * (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
    case 13: {
        double d = (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
        return a[0] * b[0] * d * d;
    }
    case 14: return a[0] * b[0] * (a[1] * b[1] + a[2] * b[2]);
    case 15: {
        double d = (a[1] * b[1] + a[2] * b[2]);
        return a[0] * b[0] * d * d;
    }
    case 16:
        if (a[4] == b[4]) {
            double d = (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
            return a[0] * b[0] * d * d;
        }
        return 0.0;
    case 17:
        if (a[4] != b[4]) {
            double d = (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
            return a[0] * b[0] * d * d;
        }
        return 0.0;
    default: return 0.0;
    }
}

static void walk_range(const walk_t *w, int64_t c0, int64_t c1, int64_t *ic, double *dc) {
    const mesh_t *m1 = &w->m1, *m2 = &w->m2;
    const int n1y = m1->n[1], n1z = m1->n[2];
    const int n2x = m2->n[0], n2y = m2->n[1], n2z = m2->n[2];
    int64_t *diff = NULL;
    /* differential counts (and weighted sums), summed by the caller */
    if (w->kind == K_SMU || w->kind == K_SMU_WEIGHTED) diff = ic;
    for (int64_t icell1 = c0; icell1 < c1; icell1++) {
        int64_t if1 = m1->start[icell1], il1 = m1->start[icell1 + 1];
        int64_t Ni = il1 - if1;
        if (Ni <= 0) continue;
        int ix1 = (int)(icell1 / ((int64_t)n1y * n1z));
        int iy1 = (int)((icell1 - (int64_t)ix1 * n1y * n1z) / n1z);
        int iz1 = (int)(icell1 - (int64_t)ix1 * n1y * n1z - (int64_t)iy1 * n1z);
        int lx = ix1 * w->per[0] - w->steps[0], rx = (ix1 + 1) * w->per[0] + w->steps[0];
        int ly = iy1 * w->per[1] - w->steps[1], ry = (iy1 + 1) * w->per[1] + w->steps[1];
        int lz = iz1 * w->per[2] - w->steps[2], rz = (iz1 + 1) * w->per[2] + w->steps[2];
        for (int nx = lx; nx < rx; nx++) {
            double xs = nx < 0 ? -w->period[0] * w->pbc : (nx >= n2x ? w->period[0] * w->pbc : 0.0);
            int ix2 = ((nx % n2x) + n2x) % n2x;
            for (int ny = ly; ny < ry; ny++) {
                double ys = ny < 0 ? -w->period[1] * w->pbc : (ny >= n2y ? w->period[1] * w->pbc : 0.0);
                int iy2 = ((ny % n2y) + n2y) % n2y;
                for (int nz = lz; nz < rz; nz++) {
                    double zs = nz < 0 ? -w->period[2] * w->pbc : (nz >= n2z ? w->period[2] * w->pbc : 0.0);
                    int iz2 = ((nz % n2z) + n2z) % n2z;
                    int64_t icell2 = (int64_t)ix2 * n2y * n2z + (int64_t)iy2 * n2z + iz2;
                    int64_t if2 = m2->start[icell2], il2 = m2->start[icell2 + 1];
                    if (il2 <= if2) continue;
                    for (int64_t i = if1; i < il1; i++) {
                        double x1t = w->x1[i] - xs, y1t = w->y1[i] - ys, z1t = w->z1[i] - zs;
                        for (int64_t j = if2; j < il2; j++) {
                            double dx = x1t - w->x2[j];
                            double dy = y1t - w->y2[j];
                            double dz = z1t - w->z2[j];
                            if (w->kind == K_3D) {
                                double dsq = dx * dx + dy * dy + dz * dz;
                                int k = w->n1e - 1;
                                while (dsq <= w->e1[k]) {
                                    ic[k] += 1;
                                    k--;
                                    if (k < 0) break;
                                }
                            } else if (w->kind == K_MARKED) {
                                double dsq = dx * dx + dy * dy + dz * dz;
                                double wt = wfunc_eval(w->wfunc, w->w1 + i * w->nw, w->w2 + j * w->nw);
                                int k = w->n1e - 1;
                                while (dsq <= w->e1[k]) {
                                    dc[k] += wt;
                                    k--;
                                    if (k < 0) break;
                                }
                            } else if (w->kind == K_XYZ) {
                                double dxy = dx * dx + dy * dy;
                                double dzz = dz * dz;
                                int k = w->n1e - 1;
                                while (dxy <= w->e1[k]) {
                                    int g = w->n2e - 1;
                                    while (dzz <= w->e2[g]) {
                                        ic[(int64_t)k * w->n2e + g] += 1;
                                        g--;
                                        if (g < 0) break;
                                    }
                                    k--;
                                    if (k < 0) break;
                                }
                            } else if (w->kind == K_XYZ_MARKED) {
                                /* marked_npairs_xy_z_engine.pyx:209-224 (weight at :217, added at :222) */
                                double dxy = dx * dx + dy * dy;
                                double dzz = dz * dz;
                                double wt = wfunc_eval(w->wfunc, w->w1 + i * w->nw, w->w2 + j * w->nw);
                                int k = w->n1e - 1;
                                while (dxy <= w->e1[k]) {
                                    int g = w->n2e - 1;
                                    while (dzz <= w->e2[g]) {
                                        dc[(int64_t)k * w->n2e + g] += wt;
                                        g--;
                                        if (g < 0) break;
                                    }
                                    k--;
                                    if (k < 0) break;
                                }
                            } else if (w->kind == K_XYZ_JACK) {
                                /* npairs_jackknife_xy_z_engine.pyx:231-245 */
                                double dxy = dx * dx + dy * dy;
                                double dzz = dz * dz;
                                const int64_t plane = (int64_t)w->n1e * w->n2e;
                                for (int sidx = 0; sidx <= w->nsamp; sidx++) {
                                    int k = w->n1e - 1;
                                    while (dxy <= w->e1[k]) {
                                        int g = w->n2e - 1;
                                        while (dzz <= w->e2[g]) {
                                            dc[sidx * plane + (int64_t)k * w->n2e + g] +=
                                                jweight(sidx, w->t1[i], w->t2[j], w->w1[i], w->w2[j]);
                                            g--;
                                            if (g < 0) break;
                                        }
                                        k--;
                                        if (k < 0) break;
                                    }
                                }
                            } else if (w->kind == K_3D_JACK) {
                                /* npairs_jackknife_3d_engine.pyx: per row s, walk the
                                   cumulative bins from the top adding jweight */
                                double dsq = dx * dx + dy * dy + dz * dz;
                                for (int sidx = 0; sidx <= w->nsamp; sidx++) {
                                    int k = w->n1e - 1;
                                    while (dsq <= w->e1[k]) {
                                        dc[sidx * (int64_t)w->n1e + k] +=
                                            jweight(sidx, w->t1[i], w->t2[j], w->w1[i], w->w2[j]);
                                        k--;
                                        if (k < 0) break;
                                    }
                                }
                            } else if (w->kind == K_WPOBJ) {
                                /* per-point FP64 sums of the neighbours' weights by
                                   cumulative bin (no reference counterpart; the bin
                                   walk of npairs_3d_engine.pyx:173-182).  Rows are
                                   sorted sample-1 points: each thread owns its cells'
                                   rows of the one shared table. */
                                double dsq = dx * dx + dy * dy + dz * dz;
                                double *row = dc + i * (int64_t)w->n1e;
                                int k = w->n1e - 1;
                                while (dsq <= w->e1[k]) {
                                    row[k] += w->w2[j];
                                    k--;
                                    if (k < 0) break;
                                }
                            } else if (w->kind == K_NEIGH) {
                                /* counts_in_cylinders_engine.pyx:262-281,
                                   spherical_isolation_engine.pyx:190-199,
                                   cylindrical_isolation_engine.pyx:198-208 and the marked
                                   isolation engines: strict tests, radii squared in FP64 */
                                const double *a = w->w1 + i * w->nw, *b = w->w2 + j * w->nw;
                                const double r2 = a[0] * a[0];
                                int in;
                                if (w->geo == 0) {
                                    double dsq = dx * dx + dy * dy + dz * dz;
                                    in = dsq < r2;
                                    if (in && w->excl0) in = dsq > 0.0;
                                } else {
                                    double dxy = dx * dx + dy * dy;
                                    double dzz = dz * dz;
                                    in = (dxy < r2) && (dzz < a[1] * a[1]);
                                    if (in && w->excl0) in = (dzz + dxy) > 0.0;
                                }
                                if (in && w->ckind == 1) in = mass_frac_ok(w, a[2], b[2]);
                                if (in && w->ckind == 2) in = iso_cond(w->cfunc, a + 2, b + 2);
                                if (in) ic[i] += 1;
                            } else { /* K_SMU, K_SMU_WEIGHTED */
                                double dxy = dx * dx + dy * dy;
                                double dzz = dz * dz;
                                double s2 = dzz + dxy;
                                if (s2 > w->smax2) continue;
                                double mu2 = (s2 > 0.0) ? dxy / s2 : 0.0;
                                if (mu2 > w->mumax2) continue;
                                int k = w->n1e - 2;
                                while (k != -1) {
                                    if (s2 > w->e1[k]) break;
                                    k--;
                                }
                                int g = w->n2e - 2;
                                while (g != -1) {
                                    if (mu2 > w->e2[g]) break;
                                    g--;
                                }
                                diff[(int64_t)(k + 1) * w->n2e + (g + 1)] += 1;
                                /* weighted_npairs_s_mu_engine.pyx:249: w1 * w2 per pair */
                                if (w->kind == K_SMU_WEIGHTED)
                                    dc[(int64_t)(k + 1) * w->n2e + (g + 1)] += w->w1[i] * w->w2[j];
                            }
                        }
                    }
                }
            }
        }
    }
}

static void *walk_thread(void *arg) {
    job_t *j = (job_t *)arg;
    walk_range(j->w, j->c0, j->c1, j->icounts, j->dcounts);
    return NULL;
}

/*
 * Common driver.  xyz arrays are (N, 3) row-major float64.  period holds the
 * box lengths (the enclosing box when pbc == 0).  search[3] are the search
 * lengths, approx1/approx2 the approximate cell sizes.  Returns 0, or a
 * negative code: -1 allocation failure, -2 search longer than period/3.
 */
static int run_walk(int kind, const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                    const double *w1, const double *w2, int nw, int wfunc,
                    const int64_t *tags1, const int64_t *tags2, int nsamp,
                    const double *e1, int n1e, const double *e2, int n2e,
                    double smax2, double mumax2,
                    const double period[3], int pbc, const double search[3],
                    const double approx1[3], const double approx2[3], int nthreads,
                    int64_t *icounts, double *dcounts, const walk_t *nopt) {
    walk_t w;
    memset(&w, 0, sizeof(w));
    if (nopt) {
        /* per-object neighbours: geometry, separation > 0, condition */
        w.geo = nopt->geo; w.excl0 = nopt->excl0; w.ckind = nopt->ckind; w.cfunc = nopt->cfunc;
        w.ceq0 = nopt->ceq0; w.ceq1 = nopt->ceq1; w.clim0 = nopt->clim0; w.clim1 = nopt->clim1;
    }
    w.kind = kind;
    w.pbc = pbc;
    for (int d = 0; d < 3; d++) {
        w.period[d] = period[d];
        if (!(search[d] <= period[d] / 3.0)) return -2; /* rectangular_mesh.py:376-417 */
    }
    double c1[3], c2[3];
    for (int d = 0; d < 3; d++) c1[d] = sample1_cell_size(period[d], search[d], approx1[d]);
    if (mesh_build(&w.m1, xyz1, n1, period, c1) != 0) return -1;
    for (int d = 0; d < 3; d++) c2[d] = sample2_cell_sizes(period[d], w.m1.cell[d], approx2[d]);
    if (mesh_build(&w.m2, xyz2, n2, period, c2) != 0) { mesh_free(&w.m1); return -1; }
    for (int d = 0; d < 3; d++) {
        w.steps[d] = (int)ceil(search[d] / w.m2.cell[d]);
        w.per[d] = w.m2.n[d] / w.m1.n[d];
    }
    size_t s1 = (size_t)(n1 > 0 ? n1 : 1), s2 = (size_t)(n2 > 0 ? n2 : 1);
    double *buf = (double *)malloc(sizeof(double) * 3 * (s1 + s2));
    if (!buf) { mesh_free(&w.m1); mesh_free(&w.m2); return -1; }
    w.x1 = buf; w.y1 = buf + s1; w.z1 = buf + 2 * s1;
    w.x2 = buf + 3 * s1; w.y2 = w.x2 + s2; w.z2 = w.x2 + 2 * s2;
    for (int64_t k = 0; k < n1; k++) {
        int64_t i = w.m1.order[k];
        w.x1[k] = xyz1[3 * i]; w.y1[k] = xyz1[3 * i + 1]; w.z1[k] = xyz1[3 * i + 2];
    }
    for (int64_t k = 0; k < n2; k++) {
        int64_t i = w.m2.order[k];
        w.x2[k] = xyz2[3 * i]; w.y2[k] = xyz2[3 * i + 1]; w.z2[k] = xyz2[3 * i + 2];
    }
    double *wb = NULL;
    int64_t *tb = NULL;
    if (kind == K_XYZ_JACK || kind == K_3D_JACK) {
        tb = (int64_t *)malloc(sizeof(int64_t) * (s1 + s2));
        if (!tb) { free(buf); mesh_free(&w.m1); mesh_free(&w.m2); return -1; }
        w.t1 = tb; w.t2 = tb + s1;
        for (int64_t k = 0; k < n1; k++) w.t1[k] = tags1[w.m1.order[k]];
        for (int64_t k = 0; k < n2; k++) w.t2[k] = tags2[w.m2.order[k]];
        w.nsamp = nsamp;
    }
    if (kind == K_MARKED || kind == K_XYZ_MARKED || kind == K_SMU_WEIGHTED || kind == K_XYZ_JACK ||
        kind == K_NEIGH || kind == K_3D_JACK || kind == K_WPOBJ) {
        wb = (double *)malloc(sizeof(double) * (size_t)nw * (s1 + s2));
        if (!wb) { free(buf); mesh_free(&w.m1); mesh_free(&w.m2); return -1; }
        w.w1 = wb; w.w2 = wb + (size_t)nw * s1;
        for (int64_t k = 0; k < n1; k++)
            memcpy(w.w1 + k * nw, w1 + w.m1.order[k] * nw, sizeof(double) * nw);
        for (int64_t k = 0; k < n2; k++)
            memcpy(w.w2 + k * nw, w2 + w.m2.order[k] * nw, sizeof(double) * nw);
        w.nw = nw;
        w.wfunc = wfunc;
    }
    w.e1 = e1; w.n1e = n1e; w.e2 = e2; w.n2e = n2e;
    w.smax2 = smax2; w.mumax2 = mumax2;

    int64_t nout = (kind == K_3D || kind == K_MARKED) ? n1e : (int64_t)n1e * n2e;
    if (kind == K_XYZ_JACK) nout *= (int64_t)(nsamp + 1);
    if (kind == K_3D_JACK) nout = (int64_t)n1e * (nsamp + 1);
    if (kind == K_NEIGH) nout = n1 > 0 ? n1 : 1;  /* one count per sorted sample-1 point */
    double *wshared = NULL;  /* K_WPOBJ: one (n1, n1e) table of sorted rows, shared */
    if (kind == K_WPOBJ) {
        nout = 1;
        wshared = (double *)calloc(s1 * (size_t)n1e, sizeof(double));
        if (!wshared) { free(buf); free(wb); mesh_free(&w.m1); mesh_free(&w.m2); return -1; }
    }
    double *dsum = NULL;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > w.m1.ncells) nthreads = (int)w.m1.ncells;
    job_t *jobs = (job_t *)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int64_t *ipart = (int64_t *)calloc((size_t)nthreads * nout, sizeof(int64_t));
    double *dpart = (double *)calloc((size_t)nthreads * nout, sizeof(double));
    int rc = 0;
    if (!jobs || !th || !ipart || !dpart) { rc = -1; goto done; }
    /* contiguous cell1 ranges, as np.array_split (mesh_helpers.py:218-220) */
    {
        int64_t base = w.m1.ncells / nthreads, extra = w.m1.ncells % nthreads, c = 0;
        for (int t = 0; t < nthreads; t++) {
            int64_t len = base + (t < extra ? 1 : 0);
            jobs[t].w = &w;
            jobs[t].c0 = c;
            jobs[t].c1 = c + len;
            jobs[t].icounts = ipart + (size_t)t * nout;
            jobs[t].dcounts = wshared ? wshared : dpart + (size_t)t * nout;
            c += len;
        }
    }
    if (nthreads == 1) {
        walk_thread(&jobs[0]);
    } else {
        int started = 0;
        for (int t = 0; t < nthreads; t++) {
            if (pthread_create(&th[t], NULL, walk_thread, &jobs[t]) != 0) break;
            started++;
        }
        for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
        for (int t = started; t < nthreads; t++) walk_thread(&jobs[t]);
    }
    for (int64_t k = 0; k < nout; k++) {
        int64_t si = 0;
        double sd = 0.0;
        for (int t = 0; t < nthreads; t++) {
            si += ipart[(size_t)t * nout + k];
            sd += dpart[(size_t)t * nout + k];
        }
        if (icounts) icounts[k] = si;
        if (dcounts) dcounts[k] = sd;
    }
    if (kind == K_WPOBJ) {
        /* sorted rows -> the caller's order */
        for (int64_t k = 0; k < n1; k++)
            memcpy(dcounts + w.m1.order[k] * (int64_t)n1e, wshared + k * (int64_t)n1e,
                   sizeof(double) * (size_t)n1e);
    }
    if (kind == K_NEIGH && icounts) {
        /* per sorted point -> caller's order */
        int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)nout);
        if (!tmp) { rc = -1; goto done; }
        memcpy(tmp, icounts, sizeof(int64_t) * (size_t)nout);
        for (int64_t k = 0; k < n1; k++) icounts[w.m1.order[k]] = tmp[k];
        free(tmp);
    }
    if (kind == K_SMU_WEIGHTED && dcounts) {
        /* weighted_npairs_s_mu_engine.pyx:251-255: each cell sums its rectangle of the
           differential weighted counts */
        dsum = (double *)calloc((size_t)nout, sizeof(double));
        if (!dsum) { rc = -1; goto done; }
        for (int k = 0; k < n1e; k++)
            for (int g = 0; g < n2e; g++) {
                double v = 0.0;
                for (int a = 0; a <= k; a++)
                    for (int b = 0; b <= g; b++) v += dcounts[(int64_t)a * n2e + b];
                dsum[(int64_t)k * n2e + g] = v;
            }
        memcpy(dcounts, dsum, sizeof(double) * (size_t)nout);
    }
    if ((kind == K_SMU || kind == K_SMU_WEIGHTED) && icounts) {
        /* npairs_s_mu_engine.pyx:232-234: 2-D cumulative sum of the differential counts */
        for (int k = 0; k < n1e; k++)
            for (int g = 0; g < n2e; g++) {
                int64_t v = icounts[(int64_t)k * n2e + g];
                if (k > 0) v += icounts[(int64_t)(k - 1) * n2e + g];
                if (g > 0) v += icounts[(int64_t)k * n2e + g - 1];
                if (k > 0 && g > 0) v -= icounts[(int64_t)(k - 1) * n2e + g - 1];
                icounts[(int64_t)k * n2e + g] = v;
            }
    }
done:
    free(jobs); free(th); free(ipart); free(dpart); free(dsum); free(wshared);
    free(wb); free(tb); free(buf);
    mesh_free(&w.m1); mesh_free(&w.m2);
    return rc;
}

/* ---------------- public oracle entry points ---------------- */

/* npairs_3d_engine: counts[k] = #ordered pairs with dsq <= rbins[k]^2 (walked from the top) */
int orc_npairs_3d(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                  const double *rbins, int nb, const double period[3], int pbc,
                  const double approx1[3], const double approx2[3], int nthreads, int64_t *out) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    double rmax = rbins[0];
    for (int k = 0; k < nb; k++) { e[k] = rbins[k] * rbins[k]; if (rbins[k] > rmax) rmax = rbins[k]; }
    double search[3] = {rmax, rmax, rmax};
    int rc = run_walk(K_3D, xyz1, n1, xyz2, n2, NULL, NULL, 0, 0, NULL, NULL, 0, e, nb, NULL, 0, 0, 0,
                      period, pbc, search, approx1, approx2, nthreads, out, NULL, NULL);
    free(e);
    return rc;
}

int orc_npairs_xy_z(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                    const double *rp_bins, int nrp, const double *pi_bins, int npi,
                    const double period[3], int pbc, const double approx1[3],
                    const double approx2[3], int nthreads, int64_t *out) {
    double *e1 = (double *)malloc(sizeof(double) * (size_t)(nrp + npi));
    if (!e1) return -1;
    double *e2 = e1 + nrp;
    double rpmax = rp_bins[0], pimax = pi_bins[0];
    for (int k = 0; k < nrp; k++) { e1[k] = rp_bins[k] * rp_bins[k]; if (rp_bins[k] > rpmax) rpmax = rp_bins[k]; }
    for (int k = 0; k < npi; k++) { e2[k] = pi_bins[k] * pi_bins[k]; if (pi_bins[k] > pimax) pimax = pi_bins[k]; }
    double search[3] = {rpmax, rpmax, pimax};
    int rc = run_walk(K_XYZ, xyz1, n1, xyz2, n2, NULL, NULL, 0, 0, NULL, NULL, 0, e1, nrp, e2, npi, 0, 0,
                      period, pbc, search, approx1, approx2, nthreads, out, NULL, NULL);
    free(e1);
    return rc;
}

/* mu_prime = sort(sin(arccos(mu_bins))) is prepared by the caller (npairs_s_mu.py:174-175) */
int orc_npairs_s_mu(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                    const double *s_bins, int ns, const double *mu_prime, int nmu,
                    const double period[3], int pbc, const double approx1[3],
                    const double approx2[3], int nthreads, int64_t *out) {
    double *e1 = (double *)malloc(sizeof(double) * (size_t)(ns + nmu));
    if (!e1) return -1;
    double *e2 = e1 + ns;
    double smax = s_bins[0];
    for (int k = 0; k < ns; k++) { e1[k] = s_bins[k] * s_bins[k]; if (s_bins[k] > smax) smax = s_bins[k]; }
    for (int k = 0; k < nmu; k++) e2[k] = mu_prime[k] * mu_prime[k];
    /* np.max propagates NaN */
    double smax2 = e1[0], mumax2 = e2[0];
    for (int k = 0; k < ns; k++) { if (isnan(e1[k]) || isnan(smax2)) smax2 = NAN; else if (e1[k] > smax2) smax2 = e1[k]; }
    for (int k = 0; k < nmu; k++) { if (isnan(e2[k]) || isnan(mumax2)) mumax2 = NAN; else if (e2[k] > mumax2) mumax2 = e2[k]; }
    double search[3] = {smax, smax, smax};
    int rc = run_walk(K_SMU, xyz1, n1, xyz2, n2, NULL, NULL, 0, 0, NULL, NULL, 0, e1, ns, e2, nmu, smax2, mumax2,
                      period, pbc, search, approx1, approx2, nthreads, out, NULL, NULL);
    free(e1);
    return rc;
}

int orc_marked_npairs_3d(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                         const double *w1, const double *w2, int nw, int wfunc,
                         const double *rbins, int nb, const double period[3], int pbc,
                         const double approx1[3], const double approx2[3], int nthreads,
                         double *out) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    double rmax = rbins[0];
    for (int k = 0; k < nb; k++) { e[k] = rbins[k] * rbins[k]; if (rbins[k] > rmax) rmax = rbins[k]; }
    double search[3] = {rmax, rmax, rmax};
    int rc = run_walk(K_MARKED, xyz1, n1, xyz2, n2, w1, w2, nw, wfunc, NULL, NULL, 0, e, nb, NULL, 0, 0, 0,
                      period, pbc, search, approx1, approx2, nthreads, NULL, out, NULL);
    free(e);
    return rc;
}

/*
 * FP64 per-point neighbour weight sums, the oracle of the adjoint at full size
 * (halotools has no gradients): out[m][k] = sum over j of w2[j] for the
 * ordered pairs (m, j) with dsq <= rbins[k]^2, j = m included when the samples
 * are the same.  With sample 2 = sample 1 and weights w, C_k = sum_m w_m
 * out[m][k], dL/dw_m = 2 sum_k gbar_k out[m][k] and dC_k/dtheta =
 * 2 sum_m out[m][k] dw_m/dtheta.  out is (n1, nb), the caller's row order.
 */
int orc_weighted_per_object_3d(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                               const double *w2, const double *rbins, int nb,
                               const double period[3], int pbc, int nthreads, double *out) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    double rmax = rbins[0];
    for (int k = 0; k < nb; k++) { e[k] = rbins[k] * rbins[k]; if (rbins[k] > rmax) rmax = rbins[k]; }
    double search[3] = {rmax, rmax, rmax};
    int rc = run_walk(K_WPOBJ, xyz1, n1, xyz2, n2, w2, w2, 1, 1, NULL, NULL, 0, e, nb, NULL, 0, 0, 0,
                      period, pbc, search, search, search, nthreads, NULL, out, NULL);
    free(e);
    return rc;
}

/* marked_npairs_xy_z_engine: out[k][g] = sum of wfunc over ordered pairs with
   dxy <= rp[k]^2 and dz^2 <= pi[g]^2 (both walked from the top) */
int orc_marked_npairs_xy_z(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                           const double *w1, const double *w2, int nw, int wfunc,
                           const double *rp_bins, int nrp, const double *pi_bins, int npi,
                           const double period[3], int pbc, const double approx1[3],
                           const double approx2[3], int nthreads, double *out) {
    double *e1 = (double *)malloc(sizeof(double) * (size_t)(nrp + npi));
    if (!e1) return -1;
    double *e2 = e1 + nrp;
    double rpmax = rp_bins[0], pimax = pi_bins[0];
    for (int k = 0; k < nrp; k++) { e1[k] = rp_bins[k] * rp_bins[k]; if (rp_bins[k] > rpmax) rpmax = rp_bins[k]; }
    for (int k = 0; k < npi; k++) { e2[k] = pi_bins[k] * pi_bins[k]; if (pi_bins[k] > pimax) pimax = pi_bins[k]; }
    double search[3] = {rpmax, rpmax, pimax};
    int rc = run_walk(K_XYZ_MARKED, xyz1, n1, xyz2, n2, w1, w2, nw, wfunc, NULL, NULL, 0, e1, nrp, e2, npi, 0, 0,
                      period, pbc, search, approx1, approx2, nthreads, NULL, out, NULL);
    free(e1);
    return rc;
}

/* weighted_npairs_s_mu_engine: cumulative (s, mu') counts and w1 * w2 sums; mu_prime
   = sort(sin(arccos(mu_bins))) from the caller (weighted_npairs_s_mu.py:192-193) */
int orc_weighted_npairs_s_mu(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                             const double *w1, const double *w2, const double *s_bins, int ns,
                             const double *mu_prime, int nmu, const double period[3], int pbc,
                             const double approx1[3], const double approx2[3], int nthreads,
                             int64_t *counts, double *wcounts) {
    double *e1 = (double *)malloc(sizeof(double) * (size_t)(ns + nmu));
    if (!e1) return -1;
    double *e2 = e1 + ns;
    double smax = s_bins[0];
    for (int k = 0; k < ns; k++) { e1[k] = s_bins[k] * s_bins[k]; if (s_bins[k] > smax) smax = s_bins[k]; }
    for (int k = 0; k < nmu; k++) e2[k] = mu_prime[k] * mu_prime[k];
    double smax2 = e1[0], mumax2 = e2[0];
    for (int k = 0; k < ns; k++) { if (isnan(e1[k]) || isnan(smax2)) smax2 = NAN; else if (e1[k] > smax2) smax2 = e1[k]; }
    for (int k = 0; k < nmu; k++) { if (isnan(e2[k]) || isnan(mumax2)) mumax2 = NAN; else if (e2[k] > mumax2) mumax2 = e2[k]; }
    double search[3] = {smax, smax, smax};
    int rc = run_walk(K_SMU_WEIGHTED, xyz1, n1, xyz2, n2, w1, w2, 1, 0, NULL, NULL, 0, e1, ns, e2, nmu, smax2,
                      mumax2, period, pbc, search, approx1, approx2, nthreads, counts, wcounts, NULL);
    free(e1);
    return rc;
}

/* npairs_jackknife_xy_z_engine: out[s][k][g] = sum of jweight(s, ...) over ordered
   pairs with dxy <= rp[k]^2 and dz^2 <= pi[g]^2; w1, w2 one weight per point */
int orc_npairs_jackknife_xy_z(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                              const double *w1, const double *w2, const int64_t *tags1,
                              const int64_t *tags2, int nsamp, const double *rp_bins, int nrp,
                              const double *pi_bins, int npi, const double period[3], int pbc,
                              const double approx1[3], const double approx2[3], int nthreads,
                              double *out) {
    double *e1 = (double *)malloc(sizeof(double) * (size_t)(nrp + npi));
    if (!e1) return -1;
    double *e2 = e1 + nrp;
    double rpmax = rp_bins[0], pimax = pi_bins[0];
    for (int k = 0; k < nrp; k++) { e1[k] = rp_bins[k] * rp_bins[k]; if (rp_bins[k] > rpmax) rpmax = rp_bins[k]; }
    for (int k = 0; k < npi; k++) { e2[k] = pi_bins[k] * pi_bins[k]; if (pi_bins[k] > pimax) pimax = pi_bins[k]; }
    double search[3] = {rpmax, rpmax, pimax};
    int rc = run_walk(K_XYZ_JACK, xyz1, n1, xyz2, n2, w1, w2, 1, 0, tags1, tags2, nsamp, e1, nrp,
                      e2, npi, 0, 0, period, pbc, search, approx1, approx2, nthreads, NULL, out, NULL);
    free(e1);
    return rc;
}

/* npairs_jackknife_3d_engine: out[s][k] = sum of jweight(s, ...) over ordered pairs
   with dsq <= rbins[k]^2; w1, w2 one weight per point */
int orc_npairs_jackknife_3d(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                            const double *w1, const double *w2, const int64_t *tags1,
                            const int64_t *tags2, int nsamp, const double *rbins, int nb,
                            const double period[3], int pbc, const double approx1[3],
                            const double approx2[3], int nthreads, double *out) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    double rmax = rbins[0];
    for (int k = 0; k < nb; k++) { e[k] = rbins[k] * rbins[k]; if (rbins[k] > rmax) rmax = rbins[k]; }
    double search[3] = {rmax, rmax, rmax};
    int rc = run_walk(K_3D_JACK, xyz1, n1, xyz2, n2, w1, w2, 1, 0, tags1, tags2, nsamp, e, nb,
                      NULL, 0, 0, 0, period, pbc, search, approx1, approx2, nthreads, NULL, out,
                      NULL);
    free(e);
    return rc;
}

/* Per-object neighbours (counts_in_cylinders, the isolation functions): counts[i]
   = #sample-2 points in point i's sphere (pi == NULL) or cylinder meeting the
   condition (ckind 0 none, 1 mass fraction on marks column 0, 2 isolation marking
   function cfunc), separation > 0 when excl0.  marks (n, nmarks) row-major. */
int orc_neighbours(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                   const double *r, const double *pi, const double *marks1,
                   const double *marks2, int nmarks, int ckind, int cfunc, double lim0,
                   double lim1, int ceq0, int ceq1, int excl0, const double period[3], int pbc,
                   const double approx1[3], const double approx2[3], int nthreads,
                   int64_t *counts) {
    const int nw = 2 + nmarks;
    size_t s1 = (size_t)(n1 > 0 ? n1 : 1), s2 = (size_t)(n2 > 0 ? n2 : 1);
    double *wa = (double *)calloc(s1 * nw + s2 * nw, sizeof(double));
    if (!wa) return -1;
    double *wb = wa + s1 * nw;
    double rmax = 0.0, pmax = 0.0;
    for (int64_t i = 0; i < n1; i++) {
        wa[i * nw] = r[i];
        wa[i * nw + 1] = pi ? pi[i] : 0.0;
        for (int k = 0; k < nmarks; k++) wa[i * nw + 2 + k] = marks1[i * nmarks + k];
        if (r[i] > rmax) rmax = r[i];
        if (pi && pi[i] > pmax) pmax = pi[i];
    }
    for (int64_t j = 0; j < n2; j++)
        for (int k = 0; k < nmarks; k++) wb[j * nw + 2 + k] = marks2[j * nmarks + k];
    if (!pi) pmax = rmax;
    double search[3] = {rmax, rmax, pmax};
    walk_t opt;
    memset(&opt, 0, sizeof(opt));
    opt.geo = pi ? 1 : 0; opt.excl0 = excl0; opt.ckind = ckind; opt.cfunc = cfunc;
    opt.ceq0 = ceq0; opt.ceq1 = ceq1; opt.clim0 = lim0; opt.clim1 = lim1;
    double e = 0.0;
    int rc = run_walk(K_NEIGH, xyz1, n1, xyz2, n2, wa, wb, nw, 0, NULL, NULL, 0, &e, 1, NULL, 0,
                      0, 0, period, pbc, search, approx1, approx2, nthreads, counts, NULL, &opt);
    free(wa);
    return rc;
}

/*
 * Brute force over all N1*N2 ordered pairs, choosing per dimension the one
 * shift in {-L, 0, +L} that gives the smallest |dx| (for in-range pairs this
 * is the shift the cell walk uses), then the npairs_3d bin walk.  A second,
 * mesh-free oracle used to cross-check the cell walk on small inputs.
 */
static double shifted_delta(double a, double b, double L, int pbc) {
    double d0 = a - b;
    if (!pbc) return d0;
    double dp = (a - L) - b;   /* x2shift = +L */
    double dm = (a + L) - b;   /* x2shift = -L, x1 - (-L) */
    double best = d0;
    if (fabs(dp) < fabs(best)) best = dp;
    if (fabs(dm) < fabs(best)) best = dm;
    return best;
}

int orc_bf_npairs_3d(const double *xyz1, int64_t n1, const double *xyz2, int64_t n2,
                     const double *rbins, int nb, const double period[3], int pbc, int64_t *out) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    for (int k = 0; k < nb; k++) { e[k] = rbins[k] * rbins[k]; out[k] = 0; }
    for (int64_t i = 0; i < n1; i++)
        for (int64_t j = 0; j < n2; j++) {
            double dx = shifted_delta(xyz1[3 * i], xyz2[3 * j], period[0], pbc);
            double dy = shifted_delta(xyz1[3 * i + 1], xyz2[3 * j + 1], period[1], pbc);
            double dz = shifted_delta(xyz1[3 * i + 2], xyz2[3 * j + 2], period[2], pbc);
            double dsq = dx * dx + dy * dy + dz * dz;
            int k = nb - 1;
            while (dsq <= e[k]) { out[k]++; k--; if (k < 0) break; }
        }
    free(e);
    return 0;
}

/*
 * FP64 reference gradient of occupation-weighted counts (no reference
 * counterpart: halotools has no gradients).  For C_k = sum_ij w_i w_j
 * [d_ij <= r_k] and an upstream gradient gbar, grad[m] = dL/dw_m =
 * 2 sum_j w_j G(d_mj), G(d) = sum_{k: d <= r_k} gbar_k, by brute force over
 * all j with the reference's shift and FP64 operation order.  Threads split m.
 */
typedef struct {
    const double *xyz, *w, *e, *gbar;
    int64_t n, m0, m1;
    int nb, pbc;
    const double *period;
    double *grad;
} adj_job_t;

static void *adj_thread(void *arg) {
    adj_job_t *J = (adj_job_t *)arg;
    for (int64_t m = J->m0; m < J->m1; m++) {
        double acc = 0.0;
        for (int64_t j = 0; j < J->n; j++) {
            double dx = shifted_delta(J->xyz[3 * m], J->xyz[3 * j], J->period[0], J->pbc);
            double dy = shifted_delta(J->xyz[3 * m + 1], J->xyz[3 * j + 1], J->period[1], J->pbc);
            double dz = shifted_delta(J->xyz[3 * m + 2], J->xyz[3 * j + 2], J->period[2], J->pbc);
            double dsq = dx * dx + dy * dy + dz * dz;
            double G = 0.0;
            int k = J->nb - 1;
            while (dsq <= J->e[k]) { G += J->gbar[k]; k--; if (k < 0) break; }
            acc += J->w[j] * G;
        }
        J->grad[m] = 2.0 * acc;
    }
    return NULL;
}

int orc_weighted_adjoint_3d(const double *xyz, int64_t n, const double *w, const double *rbins,
                            int nb, const double period[3], int pbc, const double *gbar,
                            int nthreads, double *grad) {
    double *e = (double *)malloc(sizeof(double) * (size_t)nb);
    if (!e) return -1;
    for (int k = 0; k < nb; k++) e[k] = rbins[k] * rbins[k];
    if (nthreads < 1) nthreads = 1;
    adj_job_t *jobs = (adj_job_t *)calloc((size_t)nthreads, sizeof(adj_job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(e); free(jobs); free(th); return -1; }
    int64_t per = (n + nthreads - 1) / nthreads;
    char *running = (char *)calloc((size_t)nthreads, 1);
    if (!running) { free(e); free(jobs); free(th); return -1; }
    for (int t = 0; t < nthreads; t++) {
        adj_job_t J = {xyz, w, e, gbar, n, t * per, (t + 1) * per < n ? (t + 1) * per : n,
                       nb, pbc, period, grad};
        jobs[t] = J;
        if (jobs[t].m0 >= jobs[t].m1) continue;
        if (pthread_create(&th[t], NULL, adj_thread, &jobs[t]) == 0) running[t] = 1;
        else adj_thread(&jobs[t]);
    }
    for (int t = 0; t < nthreads; t++)
        if (running[t]) pthread_join(th[t], NULL);
    free(running);
    free(jobs); free(th); free(e);
    return 0;
}
