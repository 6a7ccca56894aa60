// Adjoint of the projection solve u = A(mu, lam)^{-1} b for a scalar loss L(u).
//
// With w = A^{-T} dL/du:  dL/db = w  and  dL/dtheta = -w^T (dA/dtheta) u.
//
// Structure used: the top-level operator is A = [A_II A_ID; 0 F] over
// interior (I) and Dirichlet (D) nodes, with F the per-node fix blocks
// (shear_sim_3d.hh:45-55, range_* = single node on the plates) and A_II
// symmetric (the elasticity stencil of set_up_stencil_base,
// shear_sim_3d.cpp:215-331, and its variable-coefficient form).  Then
//   A^T w = g  <=>  A_II w_I = g_I  and  F^T w_D = g_D - A_ID^T w_I,
// so w_I is the ordinary multigrid solve of A y = g' with g'_D = 0 (which
// gives y_D = 0 and A_II y_I = g_I), and w_D follows node by node.  These
// kernels work on natural-order vec3 fields (3 doubles per node,
// node i + m*(j + n*k)); mu and lam are the solver's colour-blocked copies.
#include <cuda_runtime.h>

#include "launch.h"
#include "ops.cuh"

namespace stzmg {

namespace {

__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Neighbour of (i,j,k) at offset (di,dj,dk), -1 when it leaves a
// non-periodic grid.
__device__ __forceinline__ long long nbr_nat(const Geom &g, int i, int j, int k, int di, int dj, int dk) {
    int a = i + di, b = j + dj, c = k + dk;
    if (a < 0 || a >= g.m) {
        if (!g.xp) return -1;
        a = wrapi(a, g.m);
    }
    if (b < 0 || b >= g.n) {
        if (!g.yp) return -1;
        b = wrapi(b, g.n);
    }
    if (c < 0 || c >= g.o) {
        if (!g.zp) return -1;
        c = wrapi(c, g.o);
    }
    return (long long)a + (long long)g.m * ((long long)b + (long long)g.n * c);
}

__device__ __forceinline__ void nat_coords(const Geom &g, long long p, int &i, int &j, int &k) {
    i = (int)(p % g.m);
    const long long t = p / g.m;
    j = (int)(t % g.n);
    k = (int)(t / g.n);
}

// Block (row-major 3x3) of interior row (i,j,k) of the Lame operator towards
// the neighbour at offset d; the same coefficients as lame_row (ops.cuh).
__device__ void lame_block(const LameOp<double> &op, const Geom &g, int i, int j, int k, const int d[3],
                           double *blk) {
#pragma unroll
    for (int e = 0; e < 9; e++) blk[e] = 0.0;
    const int nz = (d[0] != 0) + (d[1] != 0) + (d[2] != 0);
    auto coef_at = [&](int di, int dj, int dk, double &mu, double &lam) {
        const int a = wrapi(i + di, g.m), b = wrapi(j + dj, g.n), c = wrapi(k + dk, g.o);
        const int s = slot(g, a, b, c);
        mu = op.mu[s];
        lam = op.lam[s];
    };
    if (nz == 1) {
        const int ax = d[0] ? 0 : (d[1] ? 1 : 2);
        double mu0, lam0, mu1, lam1;
        coef_at(0, 0, 0, mu0, lam0);
        coef_at(d[0], d[1], d[2], mu1, lam1);
        const double mu_f = 0.5 * (mu0 + mu1), lam_f = 0.5 * (lam0 + lam1);
        for (int c = 0; c < 3; c++) blk[4 * c] = -op.dt * ((c == ax ? (lam_f + 2.0 * mu_f) : mu_f) * op.ih2[ax]);
    } else if (nz == 2) {
        const int r = d[0] ? 0 : 1, c = d[2] ? 2 : 1;
        const int sr = d[r], sc = d[c];
        int er[3] = {0, 0, 0}, ec[3] = {0, 0, 0};
        er[r] = sr;
        ec[c] = sc;
        double mu_r, lam_r, mu_c, lam_c;
        coef_at(er[0], er[1], er[2], mu_r, lam_r);
        coef_at(ec[0], ec[1], ec[2], mu_c, lam_c);
        const double ie = op.iedge[r + c - 1], sgn = (double)(sr * sc);
        blk[3 * r + c] = -op.dt * ((sgn * (lam_r + mu_c)) * ie);
        blk[3 * c + r] = -op.dt * ((sgn * (lam_c + mu_r)) * ie);
    }
}

// dst = src with the rows of Dirichlet nodes set to zero.
__global__ void mask_dirichlet_kernel(Geom g, const double *__restrict__ src, double *__restrict__ dst) {
    const long long npts = (long long)g.m * g.n * g.o;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        nat_coords(g, p, i, j, k);
        const bool in = is_interior(g, i, j, k);
        for (int c = 0; c < 3; c++) dst[3 * p + c] = in ? src[3 * p + c] : 0.0;
    }
}

// w_D = F^{-T} (g_D - sum over interior rows p next to D of A[p, D]^T w_p).
// Reads w only at interior nodes and writes only Dirichlet nodes.
template <int KIND>
__global__ void adjoint_dirichlet_kernel(Geom g, const __grid_constant__ ConstOp<double> cop, LameOp<double> lop,
                                         const double *__restrict__ gv, double *__restrict__ w) {
    const long long npts = (long long)g.m * g.n * g.o;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npts;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        nat_coords(g, q, i, j, k);
        if (is_interior(g, i, j, k)) continue;
        double acc[3] = {gv[3 * q], gv[3 * q + 1], gv[3 * q + 2]};
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy && !dz) continue;
                    // row p = q - d reaches q through its block at offset d
                    const long long p = nbr_nat(g, i, j, k, -dx, -dy, -dz);
                    if (p < 0) continue;
                    int pi, pj, pk;
                    nat_coords(g, p, pi, pj, pk);
                    if (!is_interior(g, pi, pj, pk)) continue;
                    double blk[9];
                    if (KIND == OP_CONST) {
                        const int b = 13 + dx + 3 * dy + 9 * dz;
                        for (int e = 0; e < 9; e++) blk[e] = cop.a[b][e];
                    } else {
                        const int d[3] = {dx, dy, dz};
                        lame_block(lop, g, pi, pj, pk, d, blk);
                    }
                    const double w0 = w[3 * p], w1 = w[3 * p + 1], w2 = w[3 * p + 2];
                    acc[0] -= blk[0] * w0 + blk[3] * w1 + blk[6] * w2;
                    acc[1] -= blk[1] * w0 + blk[4] * w1 + blk[7] * w2;
                    acc[2] -= blk[2] * w0 + blk[5] * w1 + blk[8] * w2;
                }
        if (KIND == OP_CONST) {
            const double *f = cop.inv_fix;   // w_D = F^{-T} acc
            w[3 * q] = dot3(f[0], acc[0], f[3], acc[1], f[6], acc[2]);
            w[3 * q + 1] = dot3(f[1], acc[0], f[4], acc[1], f[7], acc[2]);
            w[3 * q + 2] = dot3(f[2], acc[0], f[5], acc[1], f[8], acc[2]);
        } else {
            const int s = slot(g, i, j, k);
            const double f = lame_fix(lop, s);
            w[3 * q] = acc[0] / f;
            w[3 * q + 1] = acc[1] / f;
            w[3 * q + 2] = acc[2] / f;
        }
    }
}

// Per row p, the row's contributions -w_p . d(Au)_p / d(mu, lam) at the 7
// nodes whose coefficients it uses: C[14p + 2s + {0: mu, 1: lam}], s = 0 for
// p itself and s = 1 + f for face neighbour f (order x-, x+, y-, y+, z-, z+).
__global__ void lame_grad_rows_kernel(Geom g, LameOp<double> op, const double *__restrict__ w,
                                      const double *__restrict__ u, double *__restrict__ C) {
    const long long npts = (long long)g.m * g.n * g.o;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        nat_coords(g, p, i, j, k);
        double gm[7], gl[7];
        for (int s = 0; s < 7; s++) gm[s] = gl[s] = 0.0;
        const double wp[3] = {w[3 * p], w[3 * p + 1], w[3 * p + 2]};
        const double up[3] = {u[3 * p], u[3 * p + 1], u[3 * p + 2]};
        const double hh[3] = {op.dx, op.dy, op.dz};
        if (is_interior(g, i, j, k)) {
            long long nf[6];
            for (int f = 0; f < 6; f++) {
                int d[3] = {0, 0, 0};
                d[f / 2] = (f & 1) ? 1 : -1;
                nf[f] = nbr_nat(g, i, j, k, d[0], d[1], d[2]);
            }
            // faces: -dt * v_fc * (u_q[c] - u_p[c]), v_fc = (c == ax ? lam_f + 2 mu_f : mu_f) / h^2,
            // mu_f = (mu_p + mu_q) / 2
            for (int f = 0; f < 6; f++) {
                const int ax = f / 2;
                const long long q = nf[f];
                const double s2 = op.dt / (hh[ax] * hh[ax]);
                double Gm = 0.0;
                for (int c = 0; c < 3; c++) Gm += (c == ax ? 2.0 : 1.0) * wp[c] * (u[3 * q + c] - up[c]);
                Gm *= s2;
                const double Gl = s2 * wp[ax] * (u[3 * q + ax] - up[ax]);
                gm[0] += 0.5 * Gm;
                gm[1 + f] += 0.5 * Gm;
                gl[0] += 0.5 * Gl;
                gl[1 + f] += 0.5 * Gl;
            }
            // edges: (Au)_p[r] += a_rc u_q[c], a_rc = -dt sgn (lam(p + sr e_r) + mu(p + sc e_c)) / den
            //        (Au)_p[c] += a_cr u_q[r], a_cr = -dt sgn (lam(p + sc e_c) + mu(p + sr e_r)) / den
            for (int pr = 0; pr < 3; pr++) {
                const int r = pr == 2 ? 1 : 0, c = pr == 0 ? 1 : 2;
                const double den = 4.0 * hh[r] * hh[c];
                for (int sr = -1; sr <= 1; sr += 2)
                    for (int sc = -1; sc <= 1; sc += 2) {
                        int d[3] = {0, 0, 0};
                        d[r] = sr;
                        d[c] = sc;
                        const long long q = nbr_nat(g, i, j, k, d[0], d[1], d[2]);
                        const double t = op.dt * (double)(sr * sc) / den;
                        const double E1 = t * wp[r] * u[3 * q + c];
                        const double E2 = t * wp[c] * u[3 * q + r];
                        const int fr = 1 + 2 * r + (sr > 0), fc = 1 + 2 * c + (sc > 0);
                        gl[fr] += E1;
                        gm[fc] += E1;
                        gl[fc] += E2;
                        gm[fr] += E2;
                    }
            }
        } else {
            // Dirichlet row: fix(mu, lam) u_p, fix = -2 dt ((lam + 2 mu)/dx^2 + mu/dy^2 + mu/dz^2)
            const double wu = dot3(wp[0], up[0], wp[1], up[1], wp[2], up[2]);
            const double ix2 = 1.0 / (op.dx * op.dx), iy2 = 1.0 / (op.dy * op.dy), iz2 = 1.0 / (op.dz * op.dz);
            gm[0] = 2.0 * op.dt * (2.0 * ix2 + iy2 + iz2) * wu;
            gl[0] = 2.0 * op.dt * ix2 * wu;
        }
        for (int s = 0; s < 7; s++) {
            C[14 * p + 2 * s] = gm[s];
            C[14 * p + 2 * s + 1] = gl[s];
        }
    }
}

// dmu[q] = C[q][self] + sum over the rows p = q - s e_ax whose face (ax, s)
// reaches q of C[p][face (ax, s)]; same for lam.
__global__ void lame_grad_gather_kernel(Geom g, const double *__restrict__ C, double *__restrict__ dmu,
                                        double *__restrict__ dlam) {
    const long long npts = (long long)g.m * g.n * g.o;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npts;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        nat_coords(g, q, i, j, k);
        double am = C[14 * q], al = C[14 * q + 1];
        for (int f = 0; f < 6; f++) {
            const int ax = f / 2, s = (f & 1) ? 1 : -1;
            int d[3] = {0, 0, 0};
            d[ax] = -s;
            const long long p = nbr_nat(g, i, j, k, d[0], d[1], d[2]);
            if (p < 0) continue;
            am += C[14 * p + 2 * (1 + f)];
            al += C[14 * p + 2 * (1 + f) + 1];
        }
        dmu[q] = am;
        dlam[q] = al;
    }
}

int grid_for(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 152 * 64 ? (b > 0 ? b : 1) : 152 * 64);
}

}  // namespace

void launch_mask_dirichlet(const Geom &g, const double *src, double *dst, cudaStream_t st) {
    mask_dirichlet_kernel<<<grid_for((long long)g.m * g.n * g.o), 256, 0, st>>>(g, src, dst);
}

void launch_adjoint_dirichlet(const LevelOp<double> &top, const Geom &g, const double *gv, double *w,
                              cudaStream_t st) {
    const int nb = grid_for((long long)g.m * g.n * g.o);
    if (top.kind == OP_CONST) adjoint_dirichlet_kernel<OP_CONST><<<nb, 256, 0, st>>>(g, top.cop, top.lop, gv, w);
    else adjoint_dirichlet_kernel<OP_LAME><<<nb, 256, 0, st>>>(g, top.cop, top.lop, gv, w);
}

void launch_lame_grad(const LameOp<double> &op, const Geom &g, const double *w, const double *u, double *C,
                      double *dmu, double *dlam, cudaStream_t st) {
    const int nb = grid_for((long long)g.m * g.n * g.o);
    lame_grad_rows_kernel<<<nb, 256, 0, st>>>(g, op, w, u, C);
    lame_grad_gather_kernel<<<nb, 256, 0, st>>>(g, C, dmu, dlam);
}

}  // namespace stzmg
