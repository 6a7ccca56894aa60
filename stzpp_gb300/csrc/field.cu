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

}  // namespace stzmg
