// Shared device-side definitions of the GB300 multigrid: level geometry,
// the colour-blocked field layout, and the operator descriptors.
//
// Layout.  A level with m x n x o nodes (x fastest) is stored as 8 sub-grids,
// one per parity class q = (i&1) + 2(j&1) + 4(k&1) -- the 8 colours of the
// Gauss-Seidel smoother.  Each sub-grid has M2 x N2 x O2 = ceil(m/2) x ceil(n/2)
// x ceil(o/2) slots (odd sizes leave a few unused slots), so node (i,j,k)
// lives at  q*S + ((k>>1)*N2 + (j>>1))*M2 + (i>>1),  S = M2*N2*O2.
// A colour pass therefore reads and writes one contiguous sub-grid, and the
// neighbours of consecutive threads are consecutive in every other sub-grid.
// Vector fields are SoA: component c of a field starts at c*npad, npad = 8*S.
// Dense coefficient fields are SoA too: entry e = 9*block + row*3 + col of
// node p is at coef[e*npad + p], block = (dx+1) + 3(dy+1) + 9(dz+1).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace stzmg {

struct Geom {
    int m, n, o;      // nodes per dimension
    int xp, yp, zp;   // periodicity flags
    int M2, N2, O2;   // sub-grid extents
    int S;            // slots per sub-grid
    int npad;         // 8*S
};

inline Geom make_geom(int m, int n, int o, int xp, int yp, int zp) {
    Geom g;
    g.m = m; g.n = n; g.o = o;
    g.xp = xp; g.yp = yp; g.zp = zp;
    g.M2 = (m + 1) / 2; g.N2 = (n + 1) / 2; g.O2 = (o + 1) / 2;
    g.S = g.M2 * g.N2 * g.O2;
    g.npad = 8 * g.S;
    return g;
}

__host__ __device__ inline int slot(const Geom &g, int i, int j, int k) {
    int q = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
    return q * g.S + ((k >> 1) * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
}

// Wrap an unwrapped index into [0, len) for a periodic dimension; for a
// non-periodic one return -1 when it leaves the grid.
__host__ __device__ inline int wrap_or_out(int a, int len, int prd) {
    if (a >= 0 && a < len) return a;
    if (!prd) return -1;
    a %= len;
    return a < 0 ? a + len : a;
}

// Per-dimension slot offsets of the three neighbours d = -1, 0, +1 of a node:
// the slot of neighbour (di,dj,dk) is ox[di+1] + oy[dj+1] + oz[dk+1], or
// invalid when any part is negative (outside a non-periodic grid).
struct NbrOffsets {
    int ox[3], oy[3], oz[3];
};

__device__ inline NbrOffsets nbr_offsets(const Geom &g, int i, int j, int k) {
    NbrOffsets t;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        int a = wrap_or_out(i + d, g.m, g.xp);
        t.ox[d + 1] = a < 0 ? INT32_MIN / 4 : (a & 1) * g.S + (a >> 1);
        int b = wrap_or_out(j + d, g.n, g.yp);
        t.oy[d + 1] = b < 0 ? INT32_MIN / 4 : (b & 1) * 2 * g.S + (b >> 1) * g.M2;
        int c = wrap_or_out(k + d, g.o, g.zp);
        t.oz[d + 1] = c < 0 ? INT32_MIN / 4 : (c & 1) * 4 * g.S + (c >> 1) * g.M2 * g.N2;
    }
    return t;
}

// Neighbour offsets from sub-grid coordinates without divisions: node
// (2I+a, 2J+b, 2K+c); same result as nbr_offsets(g, 2I+a, 2J+b, 2K+c).
__device__ inline void dim_offsets(int I, int a, int n, int N2, int prd, int pstride, int istride, int *o) {
    const int BAD = INT32_MIN / 4;
    o[1] = a * pstride + I * istride;
    if (n == 1) {   // a single periodic node is its own neighbour
        o[0] = o[2] = prd ? o[1] : BAD;
        return;
    }
    if (a) o[0] = I * istride;
    else o[0] = I > 0 ? pstride + (I - 1) * istride : (prd ? pstride + (N2 - 1) * istride : BAD);
    if (2 * I + a + 1 < n) o[2] = a ? (I + 1) * istride : pstride + I * istride;
    else o[2] = prd ? 0 : BAD;
}

__device__ inline NbrOffsets nbr_offsets_sub(const Geom &g, int I, int J, int K, int a, int b, int c) {
    NbrOffsets t;
    dim_offsets(I, a, g.m, g.M2, g.xp, g.S, 1, t.ox);
    dim_offsets(J, b, g.n, g.N2, g.yp, 2 * g.S, g.M2, t.oy);
    dim_offsets(K, c, g.o, g.O2, g.zp, 4 * g.S, g.M2 * g.N2, t.oz);
    return t;
}

// Node coordinates of thread t within colour q's sub-grid; false for an
// unused slot.
__device__ inline bool colour_node(const Geom &g, int q, int t, int &i, int &j, int &k) {
    int I = t % g.M2, r = t / g.M2;
    int J = r % g.N2, K = r / g.N2;
    i = 2 * I + (q & 1);
    j = 2 * J + ((q >> 1) & 1);
    k = 2 * K + ((q >> 2) & 1);
    return i < g.m && j < g.n && k < g.o;
}

// Thread mapping of kernels that visit every node: a block of 8 warps covers
// the same 32 consecutive sub-grid slots in all 8 colours (warp w = colour w),
// i.e. a compact 64x2x2 region of the level, so neighbour reads are shared in
// L1 across the colours; within a warp the slots stay consecutive (coalesced).
// Launch with blockDim 256 and ceil(S/32) blocks.  Returns the slot or -1.
__device__ inline int interleaved_slot(const Geom &g) {
    const int q = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + (threadIdx.x & 31);
    return t < g.S ? q * g.S + t : -1;
}

// Node coordinates of slot p (any colour).
__device__ inline bool slot_node(const Geom &g, int p, int &i, int &j, int &k) {
    int q = p / g.S;
    return colour_node(g, q, p - q * g.S, i, j, k);
}

// shear_sim_3d::interior: full stencil unless on a Dirichlet face.
__host__ __device__ inline bool is_interior(const Geom &g, int i, int j, int k) {
    return (g.xp || (i != 0 && i != g.m - 1)) && (g.yp || (j != 0 && j != g.n - 1)) &&
           (g.zp || (k != 0 && k != g.o - 1));
}

// Operator kinds.  OP_PLANE is a coarse operator that does not vary across
// an x-y plane (the Galerkin operators of a shared stencil on a grid periodic
// in x and y): one row of 27 blocks per z-plane.
enum OpKind { OP_CONST = 0, OP_LAME = 1, OP_DENSE = 2, OP_PLANE = 3 };

// Shared constant stencil (external_ptr path): interior nodes use a[27][9],
// Dirichlet nodes use fix; inverses of both centre blocks precomputed.
// `elastic` marks the sparsity of the elasticity stencil (diagonal faces,
// two-entry symmetric edges, zero corners), which the kernels exploit.
template <typename T>
struct ConstOp {
    T a[27][9];
    T fix[9];
    T inv_int[9];
    T inv_fix[9];
    int elastic;
    int centre_diag;   // the centre block a[13] is diagonal
};

// Per-node Lame coefficients (variable-mu operator, matrix-free).
template <typename T>
struct LameOp {
    const T *mu;    // colour-blocked, npad
    const T *lam;
    T dx, dy, dz, dt;
    // reciprocals, so that rows multiply instead of divide (divisions are
    // expensive, FP64 ones on this GPU especially): 1/h^2 per axis and
    // 1/(4 h_r h_c) per axis pair (x,y), (x,z), (y,z)
    T ih2[3], iedge[3];
};

template <typename T>
inline LameOp<T> make_lame_op(const T *mu, const T *lam, double dx, double dy, double dz, double dt) {
    LameOp<T> o;
    o.mu = mu;
    o.lam = lam;
    o.dx = (T)dx; o.dy = (T)dy; o.dz = (T)dz; o.dt = (T)dt;
    o.ih2[0] = (T)(1.0 / (dx * dx)); o.ih2[1] = (T)(1.0 / (dy * dy)); o.ih2[2] = (T)(1.0 / (dz * dz));
    o.iedge[0] = (T)(1.0 / (4.0 * dx * dy)); o.iedge[1] = (T)(1.0 / (4.0 * dx * dz)); o.iedge[2] = (T)(1.0 / (4.0 * dy * dz));
    return o;
}

// Dense per-node 27-block coefficients (RAT levels).
template <typename T>
struct DenseOp {
    const T *coef;  // 243 * npad
    const T *dinv;  // 9 * npad, inverse of the centre block
};

// Plane-invariant coefficients: entry e of block b on plane k at
// coef[(9*b + e) * O + k]; inverse centre blocks at dinv[e * O + k].
// `sparse` marks operators whose entry (r,c) of the block at offset d is zero
// unless r == c or both d_r and d_c are non-zero (the structure of the
// Galerkin operators of the constant elasticity stencil: 153 of 243 entries).
template <typename T>
struct PlaneOp {
    const T *coef;
    const T *dinv;
    int O;
    int sparse;
};

// Round-to-nearest product and fused multiply-add, overloaded on the type.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// a0 b0 + a1 b1 + a2 b2, always rounded as fma(a2, b2, fma(a1, b1, a0 b0)):
// written as a plain expression the compiler may fuse either product, and
// kernels that must agree bit for bit (the tiled and the colour sweeps and
// residuals) could then round differently.
template <typename T>
__device__ __forceinline__ T dot3(T a0, T b0, T a1, T b1, T a2, T b2) {
    return fma_rn(a2, b2, fma_rn(a1, b1, mul_rn(a0, b0)));
}

template <typename T>
__device__ inline void matvec_sub(const T *a, const T *v, T *acc) {
    acc[0] -= dot3(a[0], v[0], a[1], v[1], a[2], v[2]);
    acc[1] -= dot3(a[3], v[0], a[4], v[1], a[5], v[2]);
    acc[2] -= dot3(a[6], v[0], a[7], v[1], a[8], v[2]);
}

template <typename T>
__host__ __device__ inline bool inverse3(const T *a, T *inv) {
    T a11 = a[0], a12 = a[1], a13 = a[2], a21 = a[3], a22 = a[4], a23 = a[5], a31 = a[6],
      a32 = a[7], a33 = a[8];
    T det = a11 * (a22 * a33 - a23 * a32) + a21 * (a13 * a32 - a12 * a33) + a31 * (a12 * a23 - a13 * a22);
    T idet = T(1) / det;
    inv[0] = (a22 * a33 - a23 * a32) * idet; inv[1] = (a13 * a32 - a12 * a33) * idet;
    inv[2] = (a12 * a23 - a13 * a22) * idet; inv[3] = (a23 * a31 - a21 * a33) * idet;
    inv[4] = (a11 * a33 - a13 * a31) * idet; inv[5] = (a13 * a21 - a11 * a23) * idet;
    inv[6] = (a21 * a32 - a22 * a31) * idet; inv[7] = (a12 * a31 - a11 * a32) * idet;
    inv[8] = (a11 * a22 - a12 * a21) * idet;
    return det != T(0) && det == det && idet - idet == T(0);
}

}  // namespace stzmg
