// Right-hand side assembly on the device: node divergence of a cell-centred
// symmetric tensor field, the r_field of the reference simulation
// (src/shear_sim_3d.hh:283-385, default case with the plates at rest) built
// from the 8-cell averaged differences of calculate_first_order_stresses
// (src/shear_sim_3d.cpp:979-998).
//
// The cell field is natural order with 6 components per cell (s11, s12, s13,
// s22, s23, s33); cell (i,j,k) is centred at (i+1/2, j+1/2, k+1/2), so node
// (i,j,k) sits between cells i-1 and i along each axis.  A periodic dimension
// has as many cells as nodes, a non-periodic one one fewer.  Dirichlet nodes
// get 0.  The sums are evaluated in the reference's order with explicit
// round-to-nearest adds and multiplies (no FMA contraction), so the result is
// bit-identical to a sequential evaluation.
#include "launch.h"

namespace stzmg {

struct CellGrid {
    int mc, nc, oc;
};

__device__ inline int cell_wrap(int a, int len, int prd) {
    if (prd) {
        if (a < 0) return a + len;
        if (a >= len) return a - len;
    }
    return a;
}

__device__ inline double cval(const double *__restrict__ eps, const CellGrid &c, const Geom &g, int i, int j, int k,
                              int comp) {
    i = cell_wrap(i, c.mc, g.xp);
    j = cell_wrap(j, c.nc, g.yp);
    k = cell_wrap(k, c.oc, g.zp);
    return eps[6 * ((size_t)i + (size_t)c.mc * ((size_t)j + (size_t)c.nc * k)) + comp];
}

// sum of the four differences along one axis, reference order
__device__ inline double dsum(const double *eps, const CellGrid &c, const Geom &g, int i, int j, int k, int comp,
                              int axis) {
    // offsets of the 8 cells around node (i,j,k): pairs (a, a - e_axis)
    // x:  (0,0,0)-(-1,0,0) + (0,-1,0)-(-1,-1,0) + (0,0,-1)-(-1,0,-1) + (0,-1,-1)-(-1,-1,-1)
    // y:  (0,0,0)-(0,-1,0) + (-1,0,0)-(-1,-1,0) + (0,0,-1)-(0,-1,-1) + (-1,0,-1)-(-1,-1,-1)
    // z:  (0,0,0)-(0,0,-1) + (-1,0,0)-(-1,0,-1) + (0,-1,0)-(0,-1,-1) + (-1,-1,0)-(-1,-1,-1)
    int a[4][3];
    if (axis == 0) {
        int t[4][3] = {{0, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, -1, -1}};
        for (int u = 0; u < 4; u++) for (int v = 0; v < 3; v++) a[u][v] = t[u][v];
    } else if (axis == 1) {
        int t[4][3] = {{0, 0, 0}, {-1, 0, 0}, {0, 0, -1}, {-1, 0, -1}};
        for (int u = 0; u < 4; u++) for (int v = 0; v < 3; v++) a[u][v] = t[u][v];
    } else {
        int t[4][3] = {{0, 0, 0}, {-1, 0, 0}, {0, -1, 0}, {-1, -1, 0}};
        for (int u = 0; u < 4; u++) for (int v = 0; v < 3; v++) a[u][v] = t[u][v];
    }
    double s = 0.0;
    for (int u = 0; u < 4; u++) {
        int di = a[u][0], dj = a[u][1], dk = a[u][2];
        double hi = cval(eps, c, g, i + di, j + dj, k + dk, comp);
        double lo = cval(eps, c, g, i + di - (axis == 0), j + dj - (axis == 1), k + dk - (axis == 2), comp);
        s = (u == 0) ? __dadd_rn(hi, -lo) : __dadd_rn(__dadd_rn(s, hi), -lo);
    }
    return s;
}

__global__ void rhs_divergence_kernel(Geom g, CellGrid c, const double *__restrict__ eps, double qx, double qy,
                                      double qz, double *__restrict__ r) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    int s = slot(g, i, j, k);
    double v[3] = {0.0, 0.0, 0.0};
    if (is_interior(g, i, j, k)) {
        // component indices: s11 0, s12 1, s13 2, s22 3, s23 4, s33 5
        const int cx[3] = {0, 1, 2}, cy[3] = {1, 3, 4}, cz[3] = {2, 4, 5};
        for (int d = 0; d < 3; d++) {
            double ex = __dmul_rn(qx, dsum(eps, c, g, i, j, k, cx[d], 0));
            double ey = __dmul_rn(qy, dsum(eps, c, g, i, j, k, cy[d], 1));
            double ez = __dmul_rn(qz, dsum(eps, c, g, i, j, k, cz[d], 2));
            v[d] = __dadd_rn(__dadd_rn(ex, ey), ez);
        }
    }
    r[s] = v[0];
    r[s + g.npad] = v[1];
    r[s + 2 * g.npad] = v[2];
}

void launch_rhs_divergence(const Geom &g, const double *eps, double dx, double dy, double dz, double *r,
                           cudaStream_t st) {
    CellGrid c{g.xp ? g.m : g.m - 1, g.yp ? g.n : g.n - 1, g.zp ? g.o : g.o - 1};
    long npts = (long)g.m * g.n * g.o;
    // 0.25 * (1/dx), as the reference forms .25*dx_inv
    rhs_divergence_kernel<<<(unsigned)((npts + 255) / 256), 256, 0, st>>>(
        g, c, eps, 0.25 * (1.0 / dx), 0.25 * (1.0 / dy), 0.25 * (1.0 / dz), r);
}

// ------------------------------------------------------------ stress update
// The projection-step stress update of the reference
// (src/shear_sim_3d.cpp:681-710): for every cell, the velocity derivatives of
// calculate_first_order_velocities (src/shear_sim_3d.cpp:901-916) -- four
// edge differences of the cell's 8 corner nodes, in the reference's order,
// times 0.25/dx -- then ds = dt C : grad(u) with constant lambda, mu, added to
// the cell's stress, and sym_mat3::modsq(ds) (src/mat3.hh:338-340) summed per
// block for proj_mag.  u is the solver's FP64 solution (colour-blocked).
// Explicit round-to-nearest operations: bit-identical to a sequential
// evaluation of the same expressions.
struct StressCoef {
    double qx, qy, qz;        // 0.25 * (1/dx) ...
    double dt, lam, mu;
};

__device__ inline double u_at(const double *__restrict__ u, const Geom &g, int i, int j, int k, int comp) {
    if (i >= g.m) i -= g.m;   // periodic wrap of the cell's upper corner
    if (j >= g.n) j -= g.n;
    if (k >= g.o) k -= g.o;
    return u[slot(g, i, j, k) + (size_t)comp * g.npad];
}

// sum of the four edge differences of one component along `axis`, reference order
__device__ inline double edge_sum(const double *u, const Geom &g, int i, int j, int k, int comp, int axis) {
    // x: (1,0,0)-(0,0,0) + (1,1,0)-(0,1,0) + (1,0,1)-(0,0,1) + (1,1,1)-(0,1,1)
    // y: (0,1,0)-(0,0,0) + (1,1,0)-(1,0,0) + (0,1,1)-(0,0,1) + (1,1,1)-(1,0,1)
    // z: (0,0,1)-(0,0,0) + (1,0,1)-(1,0,0) + (0,1,1)-(0,1,0) + (1,1,1)-(1,1,0)
    const int lo[3][4][3] = {{{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}},
                             {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}},
                             {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}}};
    double s = 0.0;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int a = lo[axis][e][0], b = lo[axis][e][1], c = lo[axis][e][2];
        const double hi = u_at(u, g, i + a + (axis == 0), j + b + (axis == 1), k + c + (axis == 2), comp);
        const double lw = u_at(u, g, i + a, j + b, k + c, comp);
        s = e == 0 ? __dadd_rn(hi, -lw) : __dadd_rn(__dadd_rn(s, hi), -lw);
    }
    return s;
}

__global__ void stress_update_kernel(Geom g, CellGrid cg, StressCoef q, const double *__restrict__ u,
                                     double *__restrict__ sigma, double *__restrict__ partial) {
    const long ncells = (long)cg.mc * cg.nc * cg.oc;
    double proj = 0.0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ncells; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % cg.mc), j = (int)((t / cg.mc) % cg.nc), k = (int)(t / ((long)cg.mc * cg.nc));
        double d[3][3];   // d[comp][axis]: du/dx, du/dy, du/dz, dv/dx, ...
        const double qa[3] = {q.qx, q.qy, q.qz};
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int a = 0; a < 3; a++) d[c][a] = __dmul_rn(qa[a], edge_sum(u, g, i, j, k, c, a));
        const double du_dx = d[0][0], du_dy = d[0][1], du_dz = d[0][2];
        const double dv_dx = d[1][0], dv_dy = d[1][1], dv_dz = d[1][2];
        const double dw_dx = d[2][0], dw_dy = d[2][1], dw_dz = d[2][2];
        const double l2m = __dadd_rn(q.lam, __dmul_rn(2.0, q.mu)), dtmu = __dmul_rn(q.dt, q.mu);
        double ds[6];
        ds[0] = __dmul_rn(q.dt, __dadd_rn(__dmul_rn(q.lam, __dadd_rn(dw_dz, dv_dy)), __dmul_rn(l2m, du_dx)));
        ds[1] = __dmul_rn(dtmu, __dadd_rn(du_dy, dv_dx));
        ds[2] = __dmul_rn(dtmu, __dadd_rn(du_dz, dw_dx));
        ds[3] = __dmul_rn(q.dt, __dadd_rn(__dmul_rn(q.lam, __dadd_rn(dw_dz, du_dx)), __dmul_rn(l2m, dv_dy)));
        ds[4] = __dmul_rn(dtmu, __dadd_rn(dv_dz, dw_dy));
        ds[5] = __dmul_rn(q.dt, __dadd_rn(__dmul_rn(q.lam, __dadd_rn(dv_dy, du_dx)), __dmul_rn(l2m, dw_dz)));
        // sym_mat3::modsq: 0.5 (a11^2 + a12^2 + a13^2 + a12^2 + a22^2 + a23^2 + a13^2 + a23^2 + a33^2)
        const int ord[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
        double m2 = 0.0;
#pragma unroll
        for (int e = 0; e < 9; e++) m2 = __dadd_rn(m2, __dmul_rn(ds[ord[e]], ds[ord[e]]));
        proj += 0.5 * m2;
        double *sg = sigma + 6 * t;
#pragma unroll
        for (int e = 0; e < 6; e++) sg[e] = __dadd_rn(sg[e], ds[e]);
    }
    __shared__ double red[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) proj += __shfl_down_sync(0xffffffffu, proj, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = proj;
    __syncthreads();
    if (threadIdx.x < 32) {
        proj = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) proj += __shfl_down_sync(0xffffffffu, proj, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = proj;
    }
}

void launch_stress_update(const Geom &g, const double *u, double *sigma, double lam, double mu, double dt, double dx,
                          double dy, double dz, double *partial, int nblocks, cudaStream_t st) {
    CellGrid c{g.xp ? g.m : g.m - 1, g.yp ? g.n : g.n - 1, g.zp ? g.o : g.o - 1};
    StressCoef q{0.25 * (1.0 / dx), 0.25 * (1.0 / dy), 0.25 * (1.0 / dz), dt, lam, mu};
    stress_update_kernel<<<nblocks, 256, 0, st>>>(g, c, q, u, sigma, partial);
}

}  // namespace stzmg
