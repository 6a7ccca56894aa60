/* C restatement of the reference multigrid (vec3 / mat3, one rank).
 *
 * TEST INFRASTRUCTURE ONLY -- the oracle.  See stzmg_oracle.h.
 *
 * Each function names the reference code it restates (paths relative to the
 * reference checkout, mg_3d_template/ unless noted).  The reference keeps
 * per-point coefficient boxes whose bounds S (6 ints, region.hh:337-344) can
 * differ from point to point; this restatement keeps the same packed layout so
 * that box bounds can be compared exactly and coefficients entry by entry. */
#include "stzmg_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXLEV 16
#define BOUND_LOW (-1024) /* common.hh:41-42 */
#define BOUND_HIGH 1024

static char g_err[512];

static int fail(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return -1;
}

const char *so_last_error(void) { return g_err; }

/* Host threads of the sweeps, transfers and RAT (1: the serial restatement).
 * With P > 1 a level of o planes is split into min(P, o/8) z-slabs, each
 * swept lexicographically by its own thread with every value outside the slab
 * read from the copy taken at the start of the sweep: what the reference does
 * on P MPI ranks decomposed along z, whose ghost layers are refreshed once per
 * sweep (region.cc:1600, communicate region.cc:2759-2847). */
static int g_threads = 1;

void so_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int so_threads(void) {
#ifdef _OPENMP
    return g_threads;
#else
    return 1;
#endif
}

typedef struct {
    int m, n, o, xp, yp, zp;
    int npts;
    int *S;      /* 6 per point: box bounds relative to the point */
    long *aoff;  /* npts+1 offsets into A, in blocks */
    double *A;   /* 9 doubles per block, row-major mat3 */
    double *x;   /* 3 per point, natural order */
    double *r;
    double *xs;  /* snapshot used for lagged periodic ghosts */
} lev_t;

typedef struct {
    int nlev;
    lev_t L[MAXLEV];
    int v_down, v_up, bottom_sweeps;
    int grow;   /* 1: v_down+i / v_up+i-1 sweeps on level i (multigrid.cc:265,288); 0: constant */
    int nbot;
    double *lu;
    int *piv;
    double *work;
    long work_len;
} st_t;

static inline int wrap(int a, int m) { return ((a % m) + m) % m; }

static void *xcalloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

static void free_level(lev_t *L) {
    free(L->S); free(L->aoff); free(L->A); free(L->x); free(L->r); free(L->xs);
    memset(L, 0, sizeof *L);
}

static void alloc_fields(lev_t *L) {
    L->x = xcalloc((size_t)3 * L->npts, sizeof(double));
    L->r = xcalloc((size_t)3 * L->npts, sizeof(double));
    L->xs = xcalloc((size_t)3 * L->npts, sizeof(double));
}

static inline int box_size(const int *S) { return (S[1] - S[0]) * (S[3] - S[2]) * (S[5] - S[4]); }

/* shear_sim_3d::interior (src/shear_sim_3d.hh:378-383): a point with a full
 * 3x3x3 box unless it sits on a Dirichlet face. */
static inline int is_interior(const lev_t *L, int i, int j, int k) {
    return (L->xp || (i != 0 && i != L->m - 1)) && (L->yp || (j != 0 && j != L->n - 1)) &&
           (L->zp || (k != 0 && k != L->o - 1));
}

/* mat3 * vec3 in the reference's evaluation order (mat3.hh operator*(vec3)). */
static inline void matvec(const double *a, const double *v, double *out) {
    out[0] = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
    out[1] = a[3] * v[0] + a[4] * v[1] + a[5] * v[2];
    out[2] = a[6] * v[0] + a[7] * v[1] + a[8] * v[2];
}

/* mat3::inverse (mat3.hh) -- adjugate over the determinant. */
static inline void inverse3(const double *a, double *inv) {
    double a11 = a[0], a12 = a[1], a13 = a[2], a21 = a[3], a22 = a[4], a23 = a[5], a31 = a[6],
           a32 = a[7], a33 = a[8];
    double det = a11 * (a22 * a33 - a23 * a32) + a21 * (a13 * a32 - a12 * a33) + a31 * (a12 * a23 - a13 * a22);
    double idet = 1 / det;
    inv[0] = (a22 * a33 - a23 * a32) * idet; inv[1] = (a13 * a32 - a12 * a33) * idet;
    inv[2] = (a12 * a23 - a13 * a22) * idet; inv[3] = (a23 * a31 - a21 * a33) * idet;
    inv[4] = (a11 * a33 - a13 * a31) * idet; inv[5] = (a13 * a21 - a11 * a23) * idet;
    inv[6] = (a21 * a32 - a22 * a31) * idet; inv[7] = (a12 * a31 - a11 * a32) * idet;
    inv[8] = (a11 * a22 - a12 * a21) * idet;
}

/* Top level from the problem: region ctor region.hh:663-786 with the
 * interior/boundary boxes of shear_sim_3d.hh:262-273. */
static void build_fine(lev_t *L, const double *stencil, const double *fix, const double *pts) {
    int i, j, k;
    L->npts = L->m * L->n * L->o;
    L->S = xcalloc((size_t)6 * L->npts, sizeof(int));
    L->aoff = xcalloc((size_t)L->npts + 1, sizeof(long));
    long nb = 0;
    int p = 0;
    if (!pts) {
        /* one shared stencil: every interior point refers to the same 27
         * blocks and every Dirichlet point to the same fix block, as the
         * simulation's external_ptr does (src/shear_sim_3d.hh:388-402) */
        for (k = 0; k < L->o; k++)
            for (j = 0; j < L->n; j++)
                for (i = 0; i < L->m; i++, p++) {
                    int in = is_interior(L, i, j, k), *S = L->S + 6 * p;
                    S[0] = S[2] = S[4] = in ? -1 : 0;
                    S[1] = S[3] = S[5] = in ? 2 : 1;
                    L->aoff[p] = in ? 0 : 27;
                }
        L->aoff[L->npts] = 28;
        L->A = xcalloc((size_t)9 * 28, sizeof(double));
        memcpy(L->A, stencil, 243 * sizeof(double));
        memcpy(L->A + 243, fix, 9 * sizeof(double));
        alloc_fields(L);
        return;
    }
    for (k = 0; k < L->o; k++)
        for (j = 0; j < L->n; j++)
            for (i = 0; i < L->m; i++, p++) {
                int in = is_interior(L, i, j, k), *S = L->S + 6 * p;
                S[0] = S[2] = S[4] = in ? -1 : 0;
                S[1] = S[3] = S[5] = in ? 2 : 1;
                L->aoff[p] = nb;
                nb += in ? 27 : 1;
            }
    L->aoff[L->npts] = nb;
    L->A = xcalloc((size_t)9 * nb, sizeof(double));
    p = 0;
    for (k = 0; k < L->o; k++)
        for (j = 0; j < L->n; j++)
            for (i = 0; i < L->m; i++, p++) {
                double *dst = L->A + 9 * L->aoff[p];
                if (is_interior(L, i, j, k))
                    memcpy(dst, pts ? pts + 243 * (size_t)p : stencil, 243 * sizeof(double));
                else
                    memcpy(dst, pts ? pts + 243 * (size_t)p + 9 * 13 : fix, 9 * sizeof(double));
            }
    alloc_fields(L);
}

/* region::grid_map (region.cc:2587-2604): maps a parent box [lo,hi) in global
 * indices to the coarse box. */
static int grid_map(int *lo, int *hi, int ma, int prd) {
    if (prd) {
        if (*lo < -ma || *lo > ma - 1 || *hi < 1 || *hi > 2 * ma) return fail("S bound out of range [prd]");
        *lo = *lo < 0 ? (*lo - (ma & 1 ? 2 : 1)) / 2 : *lo >> 1;
        *hi = (*hi + ((ma & 1) && *hi > ma ? 1 : 2)) >> 1;
    } else {
        if (*lo < 0 || *lo > ma - 1 || *hi < 1 || *hi > ma) return fail("S bound out of range [non-prd]");
        *lo = (!(ma & 1) && *lo == ma - 1 ? *lo + 1 : *lo) >> 1;
        *hi = (*hi + 2) >> 1;
    }
    return 0;
}

/* region::igrid_map (region.cc:2618-2647): parent index range [lo,hi) that
 * coarse index i draws from, cropped to [blo,bhi); returns the parent index
 * that coincides with i. */
static int igrid_map(int *lo, int *hi, int blo, int bhi, int i, int ma, int prd, int *err) {
    int j;
    if (prd) {
        j = i * 2;
        if (ma & 1) {
            int llo, hhi;
            if (j < 0) { j += 1; llo = -ma; hhi = 0; }
            else if (j >= ma) { j -= 1; llo = ma; hhi = 2 * ma; }
            else { llo = 0; hhi = ma; }
            *lo = j == llo ? llo : j - 1;
            *hi = j == hhi - 1 ? hhi : j + 2;
        } else { *lo = j - 1; *hi = j + 2; }
    } else {
        if (i < 0 || i >= (ma + 2) >> 1) { *err = fail("grid index out of range [non-prd]"); return 0; }
        j = i << 1;
        if (ma & 1) { *lo = j == 0 ? 0 : j - 1; *hi = j == ma - 1 ? ma : j + 2; }
        else {
            if (j == ma) { *lo = ma - 1; *hi = ma; j = ma - 1; }
            else { *lo = j == 0 ? 0 : j - 1; *hi = j == ma - 2 ? ma - 1 : j + 2; }
        }
    }
    if (*lo < blo) *lo = blo;
    if (*hi > bhi) *hi = bhi;
    return j;
}

/* Coarse parents of fine index f in one dimension, in unwrapped coarse
 * indices, and the interpolation weight shared by them.  This is the set of
 * coarse points that rt_scan_row and the interpolate, restrict and rat_fill
 * routines (region.cc:1971-2471) attach fine point f to: even f coincides with coarse
 * f/2; odd f sits between (f-1)/2 and (f+1)/2, except the last point of an
 * even non-periodic dimension, which coincides with the last coarse point
 * (the "xs/ys/zs" masks 4/32/256). */
static inline int parents1d(int f, int mf, int prd, int *c, int *collapse) {
    *collapse = 0;
    if ((f & 1) == 0) { c[0] = f >> 1; return 1; }
    if (!prd && !(mf & 1) && f == mf - 1) { c[0] = (f >> 1) + 1; *collapse = 1; return 1; }
    c[0] = f >> 1;
    c[1] = (f >> 1) + 1;
    return 2;
}

/* Box union b_ex (region.cc:2665-2698). */
static inline void box_extend(int *S, int lo0, int hi0, int lo1, int hi1, int lo2, int hi2) {
    if (lo0 < S[0]) S[0] = lo0;
    if (hi0 > S[1]) S[1] = hi0;
    if (lo1 < S[2]) S[2] = lo1;
    if (hi1 > S[3]) S[3] = hi1;
    if (lo2 < S[4]) S[4] = lo2;
    if (hi2 > S[5]) S[5] = hi2;
}

/* Coarse box of the RAT row of fine point (fi,fj,fk): Sbound + b_red
 * (region.cc:2472-2480, 2654-2660). Returns fine box in fb[6] and coarse box
 * in cb[6], global unwrapped indices. */
static int fine_and_coarse_box(const lev_t *P, int fi, int fj, int fk, int *fb, int *cb) {
    const int *S = P->S + 6 * (fi + P->m * (fj + P->n * fk));
    fb[0] = fi + S[0]; fb[1] = fi + S[1];
    fb[2] = fj + S[2]; fb[3] = fj + S[3];
    fb[4] = fk + S[4]; fb[5] = fk + S[5];
    memcpy(cb, fb, 6 * sizeof(int));
    if (grid_map(cb, cb + 1, P->m, P->xp)) return -1;
    if (grid_map(cb + 2, cb + 3, P->n, P->yp)) return -1;
    if (grid_map(cb + 4, cb + 5, P->o, P->zp)) return -1;
    return 0;
}

static int level_slabs(const lev_t *L);
static int scatter_threads(const lev_t *C);

/* Coarse level bounds: region ctor region.cc:853-959 and fill_rat_bounds
 * region.cc:1848-1905 (strip communication replaced by wrapping the target
 * index; box union is order independent). */
static int bounds_plane(lev_t *C, const lev_t *P, int ck) {
    int cj, ci, sx, sy, sz;
        for (cj = 0; cj < C->n; cj++)
            for (ci = 0; ci < C->m; ci++)
                for (sz = 0; sz < 2; sz++)
                    for (sy = 0; sy < 2; sy++)
                        for (sx = 0; sx < 2; sx++) {
                            int fi = 2 * ci + sx, fj = 2 * cj + sy, fk = 2 * ck + sz;
                            if (fi >= P->m || fj >= P->n || fk >= P->o) continue;
                            int fb[6], cb[6], px[2], py[2], pz[2], cx, cy, cz;
                            if (fine_and_coarse_box(P, fi, fj, fk, fb, cb)) return -1;
                            int nx = parents1d(fi, P->m, P->xp, px, &cx);
                            int ny = parents1d(fj, P->n, P->yp, py, &cy);
                            int nz = parents1d(fk, P->o, P->zp, pz, &cz);
                            for (int a = 0; a < nz; a++)
                                for (int b = 0; b < ny; b++)
                                    for (int c = 0; c < nx; c++) {
                                        int ti = px[c], tj = py[b], tk = pz[a];
                                        int wi = wrap(ti, C->m), wj = wrap(tj, C->n), wk = wrap(tk, C->o);
                                        if (!C->xp && wi != ti) return fail("non-periodic wrap (x)");
                                        if (!C->yp && wj != tj) return fail("non-periodic wrap (y)");
                                        if (!C->zp && wk != tk) return fail("non-periodic wrap (z)");
                                        int *S = C->S + 6 * (wi + C->m * (wj + C->n * wk));
                                        box_extend(S, cb[0] - ti, cb[1] - ti, cb[2] - tj, cb[3] - tj,
                                                   cb[4] - tk, cb[5] - tk);
                                    }
                        }
    return 0;
}

static int build_coarse_bounds(lev_t *C, const lev_t *P) {
    C->npts = C->m * C->n * C->o;
    C->S = xcalloc((size_t)6 * C->npts, sizeof(int));
    for (int p = 0; p < C->npts; p++) {
        int *S = C->S + 6 * p;
        S[0] = 0; S[1] = 1; S[2] = 0; S[3] = 1; S[4] = 0; S[5] = 1;
    }
    /* a box union does not depend on the order of its updates */
    const int T = scatter_threads(C);
    int bad = 0;
    for (int par = 0; par < (T == 1 ? 1 : 2); par++) {
#pragma omp parallel for num_threads(T) schedule(static) if (T > 1)
        for (int ck = (T == 1 ? 0 : par); ck < C->o; ck += (T == 1 ? 1 : 2))
            if (bounds_plane(C, P, ck)) {
#pragma omp atomic write
                bad = 1;
            }
    }
    if (bad) return -1;
    C->aoff = xcalloc((size_t)C->npts + 1, sizeof(long));
    long nb = 0;
    for (int p = 0; p < C->npts; p++) {
        C->aoff[p] = nb;
        nb += box_size(C->S + 6 * p);
    }
    C->aoff[C->npts] = nb;
    C->A = xcalloc((size_t)9 * nb, sizeof(double));
    alloc_fields(C);
    return 0;
}

/* Coarse coefficients: compute_rats region.cc:1911-1966 with rat_fill_full /
 * rat_fill_partial (2369-2466), A_red (2485-2538), A_mul/A_sca (region.hh:627-633)
 * and A_add (2545-2578).  Fine points are visited in the same cell/sub-point
 * order as rt_scan_grid; contributions to wrapped targets are added directly
 * (the reference routes them through strip buffers, which only changes the
 * order of the floating-point additions). */
static int rat_plane(lev_t *C, const lev_t *P, int ck, double **work, long *work_len) {
    int cj, ci, sx, sy, sz, err = 0;
        for (cj = 0; cj < C->n; cj++)
            for (ci = 0; ci < C->m; ci++)
                for (sz = 0; sz < 2; sz++)
                    for (sy = 0; sy < 2; sy++)
                        for (sx = 0; sx < 2; sx++) {
                            int fi = 2 * ci + sx, fj = 2 * cj + sy, fk = 2 * ck + sz;
                            if (fi >= P->m || fj >= P->n || fk >= P->o) continue;
                            int fb[6], cb[6];
                            if (fine_and_coarse_box(P, fi, fj, fk, fb, cb)) return -1;
                            int nJ = (cb[1] - cb[0]) * (cb[3] - cb[2]) * (cb[5] - cb[4]);
                            if (*work_len < 9L * nJ) {
                                free(*work);
                                *work_len = 9L * nJ;
                                *work = xcalloc((size_t)*work_len, sizeof(double));
                            }
                            double *At = *work;
                            const double *Apar = P->A + 9 * P->aoff[fi + P->m * (fj + P->n * fk)];
                            int t0 = fb[1] - fb[0], t1 = fb[3] - fb[2];
                            /* A_red */
                            int idx = 0, vi, vj, vk, li, ui, lj, uj, lk, uk;
                            for (vk = cb[4]; vk < cb[5]; vk++) {
                                int c_k = igrid_map(&lk, &uk, fb[4], fb[5], vk, P->o, P->zp, &err);
                                for (vj = cb[2]; vj < cb[3]; vj++) {
                                    int c_j = igrid_map(&lj, &uj, fb[2], fb[3], vj, P->n, P->yp, &err);
                                    for (vi = cb[0]; vi < cb[1]; vi++, idx++) {
                                        int c_i = igrid_map(&li, &ui, fb[0], fb[1], vi, P->m, P->xp, &err);
                                        if (err) return -1;
                                        double *a = At + 9 * idx;
                                        for (int e = 0; e < 9; e++) a[e] = 0;
                                        for (int kk = lk; kk < uk; kk++) {
                                            double kfac = kk == c_k ? 1 : 0.5;
                                            for (int jj = lj; jj < uj; jj++) {
                                                double jkfac = jj == c_j ? kfac : 0.5 * kfac;
                                                for (int ii = li; ii < ui; ii++) {
                                                    const double *blk = Apar + 9 * (((kk - fb[4]) * t1 + (jj - fb[2])) * t0 + (ii - fb[0]));
                                                    double w = ii == c_i ? jkfac : 0.5 * jkfac;
                                                    for (int e = 0; e < 9; e++) a[e] += (0.125 * blk[e]) * w;
                                                }
                                            }
                                        }
                                    }
                                }
                            }
                            /* A_mul / A_sca: weight of this fine point in its parents */
                            int px[2], py[2], pz[2], cx, cy, cz;
                            int nx = parents1d(fi, P->m, P->xp, px, &cx);
                            int ny = parents1d(fj, P->n, P->yp, py, &cy);
                            int nz = parents1d(fk, P->o, P->zp, pz, &cz);
                            double fac = (nx == 2 ? 0.5 : 1) * (ny == 2 ? 0.5 : 1) * (nz == 2 ? 0.5 : 1);
                            if (fac != 1)
                                for (int e = 0; e < 9 * nJ; e++) At[e] *= fac;
                            /* A_add into every parent */
                            for (int a = 0; a < nz; a++)
                                for (int b = 0; b < ny; b++)
                                    for (int c = 0; c < nx; c++) {
                                        int ti = px[c], tj = py[b], tk = pz[a];
                                        int w = wrap(ti, C->m) + C->m * (wrap(tj, C->n) + C->n * wrap(tk, C->o));
                                        const int *S = C->S + 6 * w;
                                        double *Ap = C->A + 9 * C->aoff[w];
                                        int T0 = S[1] - S[0], T1 = S[3] - S[2];
                                        const double *src = At;
                                        for (vk = cb[4]; vk < cb[5]; vk++)
                                            for (vj = cb[2]; vj < cb[3]; vj++)
                                                for (vi = cb[0]; vi < cb[1]; vi++, src += 9) {
                                                    int oi = vi - ti - S[0], oj = vj - tj - S[2], ok = vk - tk - S[4];
                                                    if (oi < 0 || oi >= T0 || oj < 0 || oj >= T1 || ok < 0 || ok >= S[5] - S[4])
                                                        return fail("RAT contribution outside the target box");
                                                    double *d = Ap + 9 * ((ok * T1 + oj) * T0 + oi);
                                                    for (int e = 0; e < 9; e++) d[e] += src[e];
                                                }
                                    }
                        }
    return 0;
}

static int build_coarse_coeffs(st_t *s, lev_t *C, const lev_t *P) {
    const int T = scatter_threads(C);
    if (T == 1) {
        for (int ck = 0; ck < C->o; ck++)
            if (rat_plane(C, P, ck, &s->work, &s->work_len)) return -1;
        return 0;
    }
    int bad = 0;
    for (int par = 0; par < 2; par++) {
#pragma omp parallel num_threads(T)
        {
            double *work = NULL;
            long work_len = 0;
#pragma omp for schedule(static)
            for (int ck = par; ck < C->o; ck += 2)
                if (rat_plane(C, P, ck, &work, &work_len)) {
#pragma omp atomic write
                    bad = 1;
                }
            free(work);
        }
    }
    return bad ? -1 : 0;
}

/* Value of x at an unwrapped neighbour index: a periodic index outside the
 * grid reads the wrapped value from `ghost` (the lagged snapshot in a
 * Gauss-Seidel sweep, the current array elsewhere). */
static inline const double *nbr(const lev_t *L, const double *cur, const double *ghost, int i, int j,
                                int k) {
    int out = (i < 0 || i >= L->m || j < 0 || j >= L->n || k < 0 || k >= L->o);
    if (out) {
        i = wrap(i, L->m); j = wrap(j, L->n); k = wrap(k, L->o);
        return ghost + 3 * (i + (size_t)L->m * (j + (size_t)L->n * k));
    }
    return cur + 3 * (i + (size_t)L->m * (j + (size_t)L->n * k));
}

/* One point update of region::gauss_seidel (region.cc:1557-1762):
 * x_c = inv(A_c) (r - sum_{q != c} A_q x_q), box order, centre skipped.
 * Planes outside [k0, k1) (another sub-domain's, or a periodic image) are
 * read from `ghost`; the whole grid is one sub-domain on one thread. */
static void gs_point(lev_t *L, int i, int j, int k, int k0, int k1, const double *ghost) {
    int p = i + L->m * (j + L->n * k);
    const int *S = L->S + 6 * p;
    const double *Ap = L->A + 9 * L->aoff[p], *Ac = NULL;
    double Ax[3] = {0, 0, 0}, t[3];
    for (int dk = S[4]; dk < S[5]; dk++) {
        const int kk = k + dk;
        const double *src = (kk >= k0 && kk < k1) ? L->x : ghost;
        for (int dj = S[2]; dj < S[3]; dj++)
            for (int di = S[0]; di < S[1]; di++, Ap += 9) {
                if (di == 0 && dj == 0 && dk == 0) { Ac = Ap; continue; }
                matvec(Ap, nbr(L, src, ghost, i + di, j + dj, kk), t);
                Ax[0] += t[0]; Ax[1] += t[1]; Ax[2] += t[2];
            }
    }
    double inv[9], d[3], *x = L->x + 3 * (size_t)p;
    const double *r = L->r + 3 * (size_t)p;
    inverse3(Ac, inv);
    d[0] = r[0] - Ax[0]; d[1] = r[1] - Ax[1]; d[2] = r[2] - Ax[2];
    matvec(inv, d, x);
}

/* z-slabs of a level: min(threads, o/8), at least 1 (small levels stay on
 * fewer threads, as the reference gathers coarse levels onto fewer ranks,
 * multigrid.cc:47-103). */
static int level_slabs(const lev_t *L) {
    int P = so_threads(), cap = L->o / 8;
    if (P > cap) P = cap;
    return P < 1 ? 1 : P;
}

/* Lexicographic sweep with ghosts lagged to the start of the sweep
 * (communicate() once at region.cc:1600); with several slabs each is swept
 * by one thread and reads the others' planes from the same snapshot. */
static void gs_lex(lev_t *L) {
    const int P = level_slabs(L);
    const size_t plane = (size_t)3 * L->m * L->n;
    if (P == 1) {
        memcpy(L->xs, L->x, sizeof(double) * 3 * (size_t)L->npts);
        for (int k = 0; k < L->o; k++)
            for (int j = 0; j < L->n; j++)
                for (int i = 0; i < L->m; i++) gs_point(L, i, j, k, 0, L->o, L->xs);
        return;
    }
#pragma omp parallel for num_threads(P) schedule(static)
    for (int k = 0; k < L->o; k++) memcpy(L->xs + plane * k, L->x + plane * k, sizeof(double) * plane);
#pragma omp parallel for num_threads(P) schedule(static, 1)
    for (int sl = 0; sl < P; sl++) {
        const int k0 = (int)((long)sl * L->o / P), k1 = (int)((long)(sl + 1) * L->o / P);
        for (int k = k0; k < k1; k++)
            for (int j = 0; j < L->n; j++)
                for (int i = 0; i < L->m; i++) gs_point(L, i, j, k, k0, k1, L->xs);
    }
}

/* 8-colour sweep: colour q = (i&1) + 2(j&1) + 4(k&1), q = 0..7; within a
 * colour every point reads the current values of the other colours. */
static void gs_mc8(lev_t *L) {
    for (int q = 0; q < 8; q++)
        for (int k = (q >> 2) & 1; k < L->o; k += 2)
            for (int j = (q >> 1) & 1; j < L->n; j += 2)
                for (int i = q & 1; i < L->m; i += 2) gs_point(L, i, j, k, 0, L->o, L->x);
}

static void gs_sweep(lev_t *L, int smoother) {
    if (smoother == 1) gs_mc8(L);
    else gs_lex(L);
}

/* region::residual (region.cc:1008-1055): r0 - A x over the full box. */
static void residual_point(const lev_t *L, int i, int j, int k, double *out) {
    int p = i + L->m * (j + L->n * k);
    const int *S = L->S + 6 * p;
    const double *Ap = L->A + 9 * L->aoff[p];
    double Ax[3] = {0, 0, 0}, t[3];
    for (int dk = S[4]; dk < S[5]; dk++)
        for (int dj = S[2]; dj < S[3]; dj++)
            for (int di = S[0]; di < S[1]; di++, Ap += 9) {
                matvec(Ap, nbr(L, L->x, L->x, i + di, j + dj, k + dk), t);
                Ax[0] += t[0]; Ax[1] += t[1]; Ax[2] += t[2];
            }
    const double *r = L->r + 3 * (size_t)p;
    out[0] = r[0] - Ax[0]; out[1] = r[1] - Ax[1]; out[2] = r[2] - Ax[2];
}

/* region::restriction (region.cc:1766-1812) with restrict_full/partial
 * (2129-2271): coarse r = sum over fine points of (1/8) P^T residual, the
 * weight of each fine point being 1/8 times its interpolation weight; then
 * multigrid::restriction clears the coarse x (multigrid.cc:444). */
static void restrict_plane(lev_t *C, const lev_t *P, int ck) {
    for (int cj = 0; cj < C->n; cj++)
        for (int ci = 0; ci < C->m; ci++)
            for (int sz = 0; sz < 2; sz++)
                for (int sy = 0; sy < 2; sy++)
                    for (int sx = 0; sx < 2; sx++) {
                        int fi = 2 * ci + sx, fj = 2 * cj + sy, fk = 2 * ck + sz;
                        if (fi >= P->m || fj >= P->n || fk >= P->o) continue;
                        double res[3];
                        residual_point(P, fi, fj, fk, res);
                        int px[2], py[2], pz[2], cx, cy, cz;
                        int nx = parents1d(fi, P->m, P->xp, px, &cx);
                        int ny = parents1d(fj, P->n, P->yp, py, &cy);
                        int nz = parents1d(fk, P->o, P->zp, pz, &cz);
                        if (sx == 0 && sy == 1 && sz == 1) {
                            /* restrict_partial, mask 145 (region.cc:2236-2243): the
                             * split of this sub-point between the two y parents is
                             * decided by the cell's x-collapse flag xs, not by ys. */
                            int xs = !P->xp && !(P->m & 1) && ci == C->m - 2;
                            if (xs) { py[0] = cj + 1; ny = 1; }
                            else { py[0] = cj; py[1] = cj + 1; ny = 2; }
                        }
                        double w = 0.125 * (nx == 2 ? 0.5 : 1) * (ny == 2 ? 0.5 : 1) * (nz == 2 ? 0.5 : 1);
                        double rd[3] = {w * res[0], w * res[1], w * res[2]};
                        for (int a = 0; a < nz; a++)
                            for (int b = 0; b < ny; b++)
                                for (int c = 0; c < nx; c++) {
                                    double *t = C->r + 3 * (wrap(px[c], C->m) + (size_t)C->m * (wrap(py[b], C->n) + (size_t)C->n * wrap(pz[a], C->o)));
                                    t[0] += rd[0]; t[1] += rd[1]; t[2] += rd[2];
                                }
                    }
}

/* Threads for a scatter over the coarse planes ck of a level: the fine points
 * under coarse plane ck add into coarse planes ck and ck + 1 only, so planes
 * of one parity run in parallel and the two parities one after the other
 * (1: serial, in the reference's order; also when a periodic z of odd extent
 * would let the last plane's updates wrap onto plane 0). */
static int scatter_threads(const lev_t *C) {
    int P = level_slabs(C);
    return (C->zp && (C->o & 1)) ? 1 : P;
}

static void restriction(lev_t *C, const lev_t *P) {
    memset(C->r, 0, sizeof(double) * 3 * (size_t)C->npts);
    const int T = scatter_threads(C);
    if (T == 1) {
        for (int ck = 0; ck < C->o; ck++) restrict_plane(C, P, ck);
    } else {
        for (int par = 0; par < 2; par++) {
#pragma omp parallel for num_threads(T) schedule(static)
            for (int ck = par; ck < C->o; ck += 2) restrict_plane(C, P, ck);
        }
    }
    memset(C->x, 0, sizeof(double) * 3 * (size_t)C->npts);
}

/* region::interpolation (region.cc:1816-1843) with interpolate_full/partial
 * (2061-2121): fine x += P x_coarse (weights 1, 1/2, 1/4, 1/8). */
static void interpolation(const lev_t *C, lev_t *P) {
    const int T = level_slabs(P);
#pragma omp parallel for num_threads(T) schedule(static) if (T > 1)
    for (int fk = 0; fk < P->o; fk++)
        for (int fj = 0; fj < P->n; fj++)
            for (int fi = 0; fi < P->m; fi++) {
                int px[2], py[2], pz[2], cx, cy, cz;
                int nx = parents1d(fi, P->m, P->xp, px, &cx);
                int ny = parents1d(fj, P->n, P->yp, py, &cy);
                int nz = parents1d(fk, P->o, P->zp, pz, &cz);
                double s[3] = {0, 0, 0};
                for (int a = 0; a < nz; a++)
                    for (int b = 0; b < ny; b++)
                        for (int c = 0; c < nx; c++) {
                            const double *v = C->x + 3 * (wrap(px[c], C->m) + (size_t)C->m * (wrap(py[b], C->n) + (size_t)C->n * wrap(pz[a], C->o)));
                            s[0] += v[0]; s[1] += v[1]; s[2] += v[2];
                        }
                double w = (nx == 2 ? 0.5 : 1) * (ny == 2 ? 0.5 : 1) * (nz == 2 ? 0.5 : 1);
                double *x = P->x + 3 * (fi + (size_t)P->m * (fj + (size_t)P->n * fk));
                x[0] += w * s[0]; x[1] += w * s[1]; x[2] += w * s[2];
            }
}

/* Dense LU with partial pivoting of the bottom level (the direct bottom solve
 * the product offers in place of solve_exact's 24 sweeps, region.cc:812-815;
 * aliased periodic entries are summed). */
static int build_bottom_lu(st_t *s) {
    lev_t *L = &s->L[s->nlev - 1];
    int N = 3 * L->npts;
    free(s->lu); free(s->piv);
    s->nbot = N;
    s->lu = xcalloc((size_t)N * N, sizeof(double));
    s->piv = xcalloc((size_t)N, sizeof(int));
    double *a = s->lu;
    for (int k = 0; k < L->o; k++)
        for (int j = 0; j < L->n; j++)
            for (int i = 0; i < L->m; i++) {
                int p = i + L->m * (j + L->n * k);
                const int *S = L->S + 6 * p;
                const double *Ap = L->A + 9 * L->aoff[p];
                for (int dk = S[4]; dk < S[5]; dk++)
                    for (int dj = S[2]; dj < S[3]; dj++)
                        for (int di = S[0]; di < S[1]; di++, Ap += 9) {
                            int ii = wrap(i + di, L->m), jj = wrap(j + dj, L->n), kk = wrap(k + dk, L->o);
                            int q = ii + L->m * (jj + L->n * kk);
                            for (int r = 0; r < 3; r++)
                                for (int c = 0; c < 3; c++) a[(size_t)(3 * p + r) * N + 3 * q + c] += Ap[3 * r + c];
                        }
            }
    for (int c = 0; c < N; c++) {
        int pv = c;
        double best = fabs(a[(size_t)c * N + c]);
        for (int r = c + 1; r < N; r++)
            if (fabs(a[(size_t)r * N + c]) > best) { best = fabs(a[(size_t)r * N + c]); pv = r; }
        if (best == 0) return fail("bottom-level matrix is singular");
        s->piv[c] = pv;
        if (pv != c)
            for (int q = 0; q < N; q++) {
                double t = a[(size_t)c * N + q]; a[(size_t)c * N + q] = a[(size_t)pv * N + q]; a[(size_t)pv * N + q] = t;
            }
        double inv = 1.0 / a[(size_t)c * N + c];
        for (int r = c + 1; r < N; r++) {
            double f = a[(size_t)r * N + c] * inv;
            a[(size_t)r * N + c] = f;
            if (f != 0)
                for (int q = c + 1; q < N; q++) a[(size_t)r * N + q] -= f * a[(size_t)c * N + q];
        }
    }
    return 0;
}

static int direct_bottom(st_t *s) {
    lev_t *L = &s->L[s->nlev - 1];
    if (!s->lu && build_bottom_lu(s)) return -1;
    int N = s->nbot;
    double *b = L->x;   /* solve in place: x <- A^-1 r */
    memcpy(b, L->r, sizeof(double) * N);
    const double *a = s->lu;
    for (int c = 0; c < N; c++) {
        int pv = s->piv[c];
        if (pv != c) { double t = b[c]; b[c] = b[pv]; b[pv] = t; }
        for (int r = c + 1; r < N; r++) b[r] -= a[(size_t)r * N + c] * b[c];
    }
    for (int r = N - 1; r >= 0; r--) {
        double t = b[r];
        for (int q = r + 1; q < N; q++) t -= a[(size_t)r * N + q] * b[q];
        b[r] = t / a[(size_t)r * N + r];
    }
    return 0;
}

/* multigrid::v_cycle (multigrid.cc:253-297). */
static int vcycle(st_t *s, int smoother, int bottom) {
    int L = s->nlev, i, l;
    for (i = 0; i < L - 1; i++) {
        for (l = 0; l < s->v_down + (s->grow ? i : 0); l++) gs_sweep(&s->L[i], smoother);
        restriction(&s->L[i + 1], &s->L[i]);
    }
    if (bottom == 1) {
        if (direct_bottom(s)) return -1;
    } else {
        for (l = 0; l < s->bottom_sweeps; l++) gs_sweep(&s->L[L - 1], smoother);
    }
    for (i = L - 1; i > 0; i--) {
        interpolation(&s->L[i], &s->L[i - 1]);
        for (l = 0; l < s->v_up + (s->grow ? i - 1 : 0); l++) gs_sweep(&s->L[i - 1], smoother);
    }
    return 0;
}

static double residual_sq_serial(const lev_t *L, double *out);

/* With several threads: per-plane sums, added in plane order. */
static double residual_sq(const lev_t *L, double *out) {
    const int T = level_slabs(L);
    if (T == 1) return residual_sq_serial(L, out);
    double *part = xcalloc((size_t)L->o, sizeof(double));
#pragma omp parallel for num_threads(T) schedule(static)
    for (int k = 0; k < L->o; k++) {
        double sum = 0, r[3];
        for (int j = 0; j < L->n; j++)
            for (int i = 0; i < L->m; i++) {
                residual_point(L, i, j, k, r);
                if (out) {
                    size_t p = i + (size_t)L->m * (j + (size_t)L->n * k);
                    out[3 * p] = r[0]; out[3 * p + 1] = r[1]; out[3 * p + 2] = r[2];
                }
                sum += r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            }
        part[k] = sum;
    }
    double sum = 0;
    for (int k = 0; k < L->o; k++) sum += part[k];
    free(part);
    return sum;
}

static double residual_sq_serial(const lev_t *L, double *out) {
    double sum = 0, r[3];
    for (int k = 0; k < L->o; k++)
        for (int j = 0; j < L->n; j++)
            for (int i = 0; i < L->m; i++) {
                residual_point(L, i, j, k, r);
                if (out) {
                    size_t p = i + (size_t)L->m * (j + (size_t)L->n * k);
                    out[3 * p] = r[0]; out[3 * p + 1] = r[1]; out[3 * p + 2] = r[2];
                }
                sum += r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            }
    return sum;
}

static st_t *H(void *h) { return (st_t *)h; }

static int check_level(st_t *s, int l) {
    if (!s || l < 0 || l >= s->nlev) return fail("level %d out of range", l);
    return 0;
}

int so_create(int m, int n, int o, int xp, int yp, int zp, const double *stencil,
              const double *fix, const double *pts, int max_coarse, void **out) {
    *out = NULL;
    if (m < 1 || n < 1 || o < 1) return fail("bad grid size");
    if (!pts && (!stencil || !fix)) return fail("need a stencil and fix block, or per-point stencils");
    st_t *s = xcalloc(1, sizeof(st_t));
    s->v_down = 2; s->v_up = 2; s->bottom_sweeps = 24;   /* multigrid.hh:123, common.hh:57 */
    s->grow = 1;
    lev_t *F = &s->L[0];
    F->m = m; F->n = n; F->o = o; F->xp = xp != 0; F->yp = yp != 0; F->zp = zp != 0;
    build_fine(F, stencil, fix, pts);
    s->nlev = 1;
    /* multigrid::setup_hierarchy (multigrid.cc:19-132): coarsen while total() > threshold */
    while ((long)s->L[s->nlev - 1].m * s->L[s->nlev - 1].n * s->L[s->nlev - 1].o > max_coarse) {
        lev_t *P = &s->L[s->nlev - 1], *C = &s->L[s->nlev];
        int mc = (P->m + (P->xp ? 1 : 2)) >> 1, nc = (P->n + (P->yp ? 1 : 2)) >> 1,
            oc = (P->o + (P->zp ? 1 : 2)) >> 1;
        if (mc == P->m && nc == P->n && oc == P->o) break;
        if (s->nlev == MAXLEV) { so_destroy(s); return fail("too many levels"); }
        C->m = mc; C->n = nc; C->o = oc; C->xp = P->xp; C->yp = P->yp; C->zp = P->zp;
        if (build_coarse_bounds(C, P)) { s->nlev++; so_destroy(s); return -1; }
        s->nlev++;
    }
    for (int l = 1; l < s->nlev; l++)
        if (build_coarse_coeffs(s, &s->L[l], &s->L[l - 1])) { so_destroy(s); return -1; }
    *out = s;
    return 0;
}

void so_destroy(void *h) {
    st_t *s = H(h);
    if (!s) return;
    for (int l = 0; l < MAXLEV; l++) free_level(&s->L[l]);
    free(s->lu); free(s->piv); free(s->work);
    free(s);
}

int so_num_levels(void *h) { return H(h)->nlev; }

int so_level_dims(void *h, int l, int *dims) {
    if (check_level(H(h), l)) return -1;
    lev_t *L = &H(h)->L[l];
    dims[0] = L->m; dims[1] = L->n; dims[2] = L->o;
    return 0;
}

int so_level_S(void *h, int l, int *S) {
    if (check_level(H(h), l)) return -1;
    lev_t *L = &H(h)->L[l];
    memcpy(S, L->S, sizeof(int) * 6 * (size_t)L->npts);
    return 0;
}

int so_level_A(void *h, int l, double *A27) {
    if (check_level(H(h), l)) return -1;
    lev_t *L = &H(h)->L[l];
    memset(A27, 0, sizeof(double) * 243 * (size_t)L->npts);
    for (int p = 0; p < L->npts; p++) {
        const int *S = L->S + 6 * p;
        if (S[0] < -1 || S[1] > 2 || S[2] < -1 || S[3] > 2 || S[4] < -1 || S[5] > 2)
            return fail("stencil box reaches beyond one point");
        const double *Ap = L->A + 9 * L->aoff[p];
        for (int dk = S[4]; dk < S[5]; dk++)
            for (int dj = S[2]; dj < S[3]; dj++)
                for (int di = S[0]; di < S[1]; di++, Ap += 9)
                    memcpy(A27 + 243 * (size_t)p + 9 * ((di + 1) + 3 * (dj + 1) + 9 * (dk + 1)), Ap,
                           9 * sizeof(double));
    }
    return 0;
}

int so_set_field(void *h, int l, int which, const double *v) {
    if (check_level(H(h), l)) return -1;
    lev_t *L = &H(h)->L[l];
    memcpy(which == 0 ? L->x : L->r, v, sizeof(double) * 3 * (size_t)L->npts);
    return 0;
}

int so_get_field(void *h, int l, int which, double *v) {
    if (check_level(H(h), l)) return -1;
    lev_t *L = &H(h)->L[l];
    memcpy(v, which == 0 ? L->x : L->r, sizeof(double) * 3 * (size_t)L->npts);
    return 0;
}

int so_gauss_seidel(void *h, int l, int sweeps, int smoother) {
    if (check_level(H(h), l)) return -1;
    for (int i = 0; i < sweeps; i++) gs_sweep(&H(h)->L[l], smoother);
    return 0;
}

int so_restriction(void *h, int l) {
    if (check_level(H(h), l) || l < 1) return l < 1 ? fail("restriction target must be coarse") : -1;
    restriction(&H(h)->L[l], &H(h)->L[l - 1]);
    return 0;
}

int so_interpolation(void *h, int l) {
    if (check_level(H(h), l) || l < 1) return l < 1 ? fail("interpolation source must be coarse") : -1;
    interpolation(&H(h)->L[l], &H(h)->L[l - 1]);
    return 0;
}

int so_vcycle(void *h, int smoother, int bottom) { return vcycle(H(h), smoother, bottom); }

int so_residual(void *h, int l, double *out, double *sq) {
    if (check_level(H(h), l)) return -1;
    double s = residual_sq(&H(h)->L[l], out);
    if (sq) *sq = s;
    return 0;
}

int so_solve(void *h, double tol, int max_cycles, int smoother, int bottom, int *cycles,
             double *hist) {
    st_t *s = H(h);
    lev_t *F = &s->L[0];
    double bsq = 0;
    for (long p = 0; p < 3L * F->npts; p++) bsq += F->r[p] * F->r[p];
    double bn = sqrt(bsq);
    if (bn == 0) bn = 1;
    int c = 0;
    double rel = sqrt(residual_sq(F, NULL)) / bn;
    while (rel > tol && c < max_cycles) {
        if (vcycle(s, smoother, bottom)) return -1;
        rel = sqrt(residual_sq(F, NULL)) / bn;
        if (hist) hist[c] = rel;
        c++;
    }
    *cycles = c;
    return 0;
}

int so_set_cycle(void *h, int v_down, int v_up, int bottom_sweeps, int grow) {
    H(h)->v_down = v_down;
    H(h)->v_up = v_up;
    H(h)->bottom_sweeps = bottom_sweeps;
    H(h)->grow = grow;
    return 0;
}
