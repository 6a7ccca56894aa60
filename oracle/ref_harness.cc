// CPU oracle harness around the UNMODIFIED reference multigrid library.
//
// Test infrastructure only: this file is compiled together with the reference
// sources where they lie (mg_3d_template/region.cc, multigrid.cc,
// geometry.cc, common.cc, buffer.cc) and the single-rank MPI shim in
// oracle/mpi_shim, into oracle/_ref/libstzref.so.  Python tests load it with
// ctypes to pin the C restatement (oracle/stzmg_oracle.c) and to generate the
// golden fixtures.  Nothing in the product links it.
//
// The problem class below implements the reference's duck-typed problem
// contract (region.hh:663-786: range_xd..range_zu, internal, mem_size,
// external_ptr, fill_entries, x_field, r_field) in the same two ways the
// reference's own problem classes do:
//   * a shared 27-block stencil for interior points and a `fix` block for
//     Dirichlet rows, returned through external_ptr (shear_sim_3d.hh:388-402,
//     manu_ps_vec.hh);
//   * per-point 27-block stencils stored inside the region through
//     internal()/mem_size()/fill_entries().
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpi.h"
#include "vec3.hh"
#include "mat3.hh"

// Free-function hooks that region.cc expects before inclusion
// (same roles as manu_ps_vec.cc:15-17 / src/shear_sim_3d.cpp:3200-3205).
inline mat3 mg3d_inverse(mat3 a) { double det; return a.inverse(det); }
inline double mg3d_mod_sq(mat3 a) { return a.modsq(); }
inline float mg3d_float(mat3 a) { return static_cast<float>(a.mod()); }

#include "region.cc"
#include "multigrid.cc"

template class region<vec3, mat3>;
template class multigrid<vec3, mat3>;

namespace {

std::string g_err;

struct stz_problem {
    int m, n, o;
    bool xp, yp, zp;
    mat3 stencil[27];
    mat3 fix[1];
    const double *pts;      // per-point 27x9 stencils in natural order, or null
    const double *xin;      // initial guess, 3 doubles per point, or null (zero)
    const double *rin;      // right-hand side, 3 doubles per point, or null (zero)

    inline bool interior(int i, int j, int k) {
        return (xp || (i != 0 && i != m - 1)) && (yp || (j != 0 && j != n - 1)) &&
               (zp || (k != 0 && k != o - 1));
    }
    inline int range_xd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    inline int range_xu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    inline int range_yd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    inline int range_yu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    inline int range_zd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    inline int range_zu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    inline bool internal(int, int, int) { return pts != nullptr; }
    inline int mem_size(int i, int j, int k) { return interior(i, j, k) ? 27 : 1; }
    inline mat3 *external_ptr(int i, int j, int k) { return interior(i, j, k) ? stencil : fix; }
    void fill_entries(int i, int j, int k, mat3 *&en) {
        const double *src = pts + 243 * ((size_t)i + (size_t)m * (j + (size_t)n * k));
        if (interior(i, j, k)) {
            for (int b = 0; b < 27; b++, en++) std::memcpy(&en->a11, src + 9 * b, 9 * sizeof(double));
        } else {
            std::memcpy(&en->a11, src + 9 * 13, 9 * sizeof(double));
            en++;
        }
    }
    inline vec3 x_field(int i, int j, int k, int, int, int) {
        if (!xin) return vec3(0.);
        const double *p = xin + 3 * ((size_t)i + (size_t)m * (j + (size_t)n * k));
        return vec3(p[0], p[1], p[2]);
    }
    inline vec3 r_field(int i, int j, int k, int, int, int) {
        if (!rin) return vec3(0.);
        const double *p = rin + 3 * ((size_t)i + (size_t)m * (j + (size_t)n * k));
        return vec3(p[0], p[1], p[2]);
    }
};

struct handle {
    stz_problem prob;
    std::vector<double> pts_copy;
    geometry *gm = nullptr;
    comm_buffer com;
    multigrid<vec3, mat3> *mg = nullptr;
    // dense LU of the bottom level (direct bottom solve of this harness)
    int nbot = 0;
    std::vector<double> lu;
    std::vector<int> piv;
    ~handle() {
        delete mg;
        if (gm) delete gm;
    }
};

inline int wrap(int a, int m) { return ((a % m) + m) % m; }

// Dense LU with partial pivoting (row-major n x n), in place.
void lu_factor(std::vector<double> &a, std::vector<int> &piv, int n) {
    piv.resize(n);
    for (int c = 0; c < n; c++) {
        int p = c;
        double best = std::fabs(a[(size_t)c * n + c]);
        for (int r = c + 1; r < n; r++) {
            double v = std::fabs(a[(size_t)r * n + c]);
            if (v > best) { best = v; p = r; }
        }
        if (best == 0) throw std::runtime_error("bottom-level matrix is singular");
        piv[c] = p;
        if (p != c)
            for (int q = 0; q < n; q++) std::swap(a[(size_t)c * n + q], a[(size_t)p * n + q]);
        double inv = 1.0 / a[(size_t)c * n + c];
        for (int r = c + 1; r < n; r++) {
            double f = a[(size_t)r * n + c] * inv;
            a[(size_t)r * n + c] = f;
            if (f != 0)
                for (int q = c + 1; q < n; q++) a[(size_t)r * n + q] -= f * a[(size_t)c * n + q];
        }
    }
}

void lu_solve(const std::vector<double> &a, const std::vector<int> &piv, int n, double *b) {
    for (int c = 0; c < n; c++) {
        if (piv[c] != c) std::swap(b[c], b[piv[c]]);
        for (int r = c + 1; r < n; r++) b[r] -= a[(size_t)r * n + c] * b[c];
    }
    for (int r = n - 1; r >= 0; r--) {
        double s = b[r];
        for (int q = r + 1; q < n; q++) s -= a[(size_t)r * n + q] * b[q];
        b[r] = s / a[(size_t)r * n + r];
    }
}

region<vec3, mat3> *level(handle *h, int l) {
    if (l < 0 || l >= h->mg->nlevels) throw std::runtime_error("level out of range");
    return h->mg->reg[l];
}

void build_bottom_lu(handle *h) {
    region<vec3, mat3> *r = level(h, h->mg->nlevels - 1);
    int N = r->smno, n3 = 3 * N;
    h->nbot = n3;
    h->lu.assign((size_t)n3 * n3, 0.0);
    for (int k = 0; k < r->so; k++)
        for (int j = 0; j < r->sn; j++)
            for (int i = 0; i < r->sm; i++) {
                int p = i + r->sm * (j + r->sn * k);
                int *Sp = r->S + 6 * p;
                mat3 *Ap = r->A[p];
                for (int dk = Sp[4]; dk < Sp[5]; dk++)
                    for (int dj = Sp[2]; dj < Sp[3]; dj++)
                        for (int di = Sp[0]; di < Sp[1]; di++, Ap++) {
                            int ii = i + di, jj = j + dj, kk = k + dk;
                            ii = r->x_prd ? wrap(ii, r->m) : ii;
                            jj = r->y_prd ? wrap(jj, r->n) : jj;
                            kk = r->z_prd ? wrap(kk, r->o) : kk;
                            if (ii < 0 || ii >= r->m || jj < 0 || jj >= r->n || kk < 0 || kk >= r->o)
                                throw std::runtime_error("bottom stencil leaves the grid");
                            int q = ii + r->sm * (jj + r->sn * kk);
                            const double *b = &Ap->a11;
                            for (int a = 0; a < 3; a++)
                                for (int c = 0; c < 3; c++)
                                    h->lu[(size_t)(3 * p + a) * n3 + 3 * q + c] += b[3 * a + c];
                        }
            }
    lu_factor(h->lu, h->piv, n3);
}

void direct_bottom(handle *h) {
    region<vec3, mat3> *r = level(h, h->mg->nlevels - 1);
    if (h->nbot == 0) build_bottom_lu(h);
    std::vector<double> b(h->nbot);
    for (int p = 0; p < r->smno; p++) {
        b[3 * p] = r->r0[p].x; b[3 * p + 1] = r->r0[p].y; b[3 * p + 2] = r->r0[p].z;
    }
    lu_solve(h->lu, h->piv, h->nbot, b.data());
    for (int k = 0; k < r->so; k++)
        for (int j = 0; j < r->sn; j++)
            for (int i = 0; i < r->sm; i++) {
                int p = i + r->sm * (j + r->sn * k);
                r->x0[i + r->mg * (j + r->ng * k)] = vec3(b[3 * p], b[3 * p + 1], b[3 * p + 2]);
            }
}

// V-cycle of multigrid::v_cycle (multigrid.cc:253-297) with a dense direct
// solve in place of solve_exact at the bottom.
void vcycle_direct(handle *h) {
    multigrid<vec3, mat3> &mg = *h->mg;
    int L = mg.mlevels;
    for (int i = 0; i < L - 1; i++) {
        for (int l = 0; l < mg.v_down + i; l++) mg.gauss_seidel(i);
        mg.restriction(i + 1);
    }
    direct_bottom(h);
    for (int i = L - 1; i > 0; i--) {
        mg.interpolation(i);
        for (int l = 0; l < mg.v_up + i - 1; l++) mg.gauss_seidel(i - 1);
    }
}

double true_res_sq(handle *h, int l, double *out) {
    region<vec3, mat3> *r = level(h, l);
    r->communicate();
    double s = 0;
    for (int k = 0; k < r->so; k++)
        for (int j = 0; j < r->sn; j++)
            for (int i = 0; i < r->sm; i++) {
                vec3 v = r->residual(i, j, k);
                if (out) {
                    size_t p = i + (size_t)r->sm * (j + (size_t)r->sn * k);
                    out[3 * p] = v.x; out[3 * p + 1] = v.y; out[3 * p + 2] = v.z;
                }
                s += v.x * v.x + v.y * v.y + v.z * v.z;
            }
    return s;
}

#define GUARD_BEGIN try {
#define GUARD_END                              \
    }                                          \
    catch (const std::exception &e) {          \
        g_err = e.what();                      \
        stz_shim_reset();                      \
        return -1;                             \
    }                                          \
    return 0;

}  // namespace

extern "C" {

const char *sr_last_error(void) { return g_err.c_str(); }

// Builds the reference hierarchy (multigrid.hh:126-153, setup_hierarchy
// multigrid.cc:19-132, which coarsens while total()>1024), optionally extends
// it with further coarse regions (region ctor region.cc:853-959) while the
// coarsest level has more than max_coarse points, then runs setup_matrices
// (fill_entries + compute_rats, multigrid.hh:194-198).
int sr_create(int m, int n, int o, int xp, int yp, int zp, const double *stencil,
              const double *fix, const double *pts, int max_coarse, void **out) {
    GUARD_BEGIN
    handle *h = new handle();
    *out = nullptr;
    try {
        stz_problem &p = h->prob;
        p.m = m; p.n = n; p.o = o; p.xp = xp; p.yp = yp; p.zp = zp;
        for (int b = 0; b < 27; b++) {
            if (stencil) std::memcpy(&p.stencil[b].a11, stencil + 9 * b, 72);
            else p.stencil[b] = mat3(0.);
        }
        if (fix) std::memcpy(&p.fix[0].a11, fix, 72); else p.fix[0] = mat3(1.);
        if (pts) {
            h->pts_copy.assign(pts, pts + (size_t)243 * m * n * o);
            p.pts = h->pts_copy.data();
        } else p.pts = nullptr;
        p.xin = p.rin = nullptr;
        h->gm = new geometry(m, n, o, xp != 0, yp != 0, zp != 0);
        h->mg = new multigrid<vec3, mat3>(p, *h->gm, h->com);
        multigrid<vec3, mat3> &mg = *h->mg;
        if (max_coarse > 1024) throw std::runtime_error("max_coarse above the reference's 1024");
        while (mg.reg[mg.nlevels - 1]->total() > max_coarse) {
            region<vec3, mat3> *last = mg.reg[mg.nlevels - 1];
            int mc = (last->m + (xp ? 1 : 2)) >> 1, nc = (last->n + (yp ? 1 : 2)) >> 1,
                oc = (last->o + (zp ? 1 : 2)) >> 1;
            if (mc == last->m && nc == last->n && oc == last->o) break;
            if (mg.nlevels == mg_max_levels) throw std::runtime_error("too many levels");
            mg.reg[mg.nlevels] = new region<vec3, mat3>(last, h->com);
            mg.geo[mg.nlevels] = NULL;
            mg.nlevels++;
            mg.mlevels = mg.nlevels;
        }
        mg.setup_matrices(p);
    } catch (...) {
        delete h;
        throw;
    }
    *out = h;
    GUARD_END
}

void sr_destroy(void *hp) { delete (handle *)hp; }

int sr_num_levels(void *hp) { return ((handle *)hp)->mg->nlevels; }

int sr_level_dims(void *hp, int l, int *dims) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    dims[0] = r->m; dims[1] = r->n; dims[2] = r->o;
    GUARD_END
}

// Box bounds S (region.hh:337-344), 6 ints per point, natural order.
int sr_level_S(void *hp, int l, int *S) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    std::memcpy(S, r->S, sizeof(int) * 6 * (size_t)r->smno);
    GUARD_END
}

// Coefficients expanded to a 3x3x3 box per point: block b = (dx+1)+3(dy+1)+9(dz+1)
// (the stencil index of shear_sim_3d.cpp:224), 9 doubles row-major per block,
// zero outside the point's box S.  Fails if a box reaches further than 1.
int sr_level_A(void *hp, int l, double *out) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    std::memset(out, 0, sizeof(double) * 243 * (size_t)r->smno);
    for (int p = 0; p < r->smno; p++) {
        int *Sp = r->S + 6 * p;
        if (Sp[0] < -1 || Sp[1] > 2 || Sp[2] < -1 || Sp[3] > 2 || Sp[4] < -1 || Sp[5] > 2)
            throw std::runtime_error("stencil box reaches beyond one point");
        mat3 *Ap = r->A[p];
        for (int dk = Sp[4]; dk < Sp[5]; dk++)
            for (int dj = Sp[2]; dj < Sp[3]; dj++)
                for (int di = Sp[0]; di < Sp[1]; di++, Ap++) {
                    int b = (di + 1) + 3 * (dj + 1) + 9 * (dk + 1);
                    std::memcpy(out + 243 * (size_t)p + 9 * b, &Ap->a11, 72);
                }
    }
    GUARD_END
}

// which = 0: solution x (x0, ghost-padded), 1: source r0.  3 doubles per point.
int sr_set_field(void *hp, int l, int which, const double *v) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    for (int k = 0; k < r->so; k++)
        for (int j = 0; j < r->sn; j++)
            for (int i = 0; i < r->sm; i++) {
                size_t p = i + (size_t)r->sm * (j + (size_t)r->sn * k);
                vec3 val(v[3 * p], v[3 * p + 1], v[3 * p + 2]);
                if (which == 0) r->x0[i + r->mg * (j + r->ng * k)] = val;
                else r->r0[p] = val;
            }
    GUARD_END
}

int sr_get_field(void *hp, int l, int which, double *v) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    for (int k = 0; k < r->so; k++)
        for (int j = 0; j < r->sn; j++)
            for (int i = 0; i < r->sm; i++) {
                size_t p = i + (size_t)r->sm * (j + (size_t)r->sn * k);
                vec3 val = which == 0 ? r->x0[i + r->mg * (j + r->ng * k)] : r->r0[p];
                v[3 * p] = val.x; v[3 * p + 1] = val.y; v[3 * p + 2] = val.z;
            }
    GUARD_END
}

int sr_gauss_seidel(void *hp, int l, int sweeps) {
    GUARD_BEGIN
    handle *h = (handle *)hp;
    level(h, l);
    for (int s = 0; s < sweeps; s++) h->mg->gauss_seidel(l);
    GUARD_END
}

// multigrid::restriction(l): coarse r at level l from the fine residual at
// level l-1, and the coarse x cleared (multigrid.cc:436-449).
int sr_restriction(void *hp, int l) {
    GUARD_BEGIN
    handle *h = (handle *)hp;
    if (l < 1) throw std::runtime_error("restriction target must be a coarse level");
    level(h, l);
    h->mg->restriction(l);
    GUARD_END
}

// multigrid::interpolation(l): level l-1 x += P x(level l) (multigrid.cc:418-430).
int sr_interpolation(void *hp, int l) {
    GUARD_BEGIN
    handle *h = (handle *)hp;
    if (l < 1) throw std::runtime_error("interpolation source must be a coarse level");
    level(h, l);
    h->mg->interpolation(l);
    GUARD_END
}

// bottom = 0: multigrid::v_cycle as shipped (solve_exact = 24 GS sweeps,
// region.cc:812-815); bottom = 1: same cycle with a dense direct bottom solve.
int sr_vcycle(void *hp, int bottom) {
    GUARD_BEGIN
    handle *h = (handle *)hp;
    if (bottom == 0) h->mg->v_cycle();
    else vcycle_direct(h);
    GUARD_END
}

// Residual r0 - A x0 of every point at level l (region::residual, region.cc:1008-1055),
// after a halo refresh; returns sum |r|^2 in *sq.
int sr_residual(void *hp, int l, double *out, double *sq) {
    GUARD_BEGIN
    double s = true_res_sq((handle *)hp, l, out);
    if (sq) *sq = s;
    GUARD_END
}

// region::l2_error_all (region.cc:3030-3057) exactly as shipped: for V=vec3
// this is the sum of |r|^4.
int sr_l2_error_all(void *hp, int l, double *out) {
    GUARD_BEGIN
    *out = level((handle *)hp, l)->l2_error_all();
    GUARD_END
}

// V-cycles until the true relative residual |b-Ax|/|b| <= tol (or max_cycles);
// hist receives the relative residual after each cycle.
int sr_solve(void *hp, double tol, int max_cycles, int bottom, int *cycles, double *hist) {
    GUARD_BEGIN
    handle *h = (handle *)hp;
    region<vec3, mat3> *r = level(h, 0);
    double bsq = 0;
    for (int p = 0; p < r->smno; p++) bsq += r->r0[p].x * r->r0[p].x + r->r0[p].y * r->r0[p].y + r->r0[p].z * r->r0[p].z;
    double bn = std::sqrt(bsq);
    int c = 0;
    double rel = std::sqrt(true_res_sq(h, 0, nullptr)) / (bn > 0 ? bn : 1.0);
    while (rel > tol && c < max_cycles) {
        if (bottom == 0) h->mg->v_cycle();
        else vcycle_direct(h);
        rel = std::sqrt(true_res_sq(h, 0, nullptr)) / (bn > 0 ? bn : 1.0);
        if (hist) hist[c] = rel;
        c++;
    }
    *cycles = c;
    GUARD_END
}

// region::output_x / output_r / output_residual of level l (region.cc:3062-3120):
// the z-slice k written by output_internal (region.cc:3135-3202) to filename.
// which: 0 x, 1 r, 2 residual.
int sr_output_slice(void *hp, int l, int which, int k, double ax, double bx, double ay, double by,
                    const char *filename) {
    GUARD_BEGIN
    region<vec3, mat3> *r = level((handle *)hp, l);
    if (which == 0) r->output_x(ax, bx, ay, by, filename, k);
    else if (which == 1) r->output_r(ax, bx, ay, by, filename, k);
    else r->output_residual(ax, bx, ay, by, filename, k);
    GUARD_END
}

}  // extern "C"
