// Grid transfers, layout permutes, mixed-precision helpers and the direct
// bottom solve.
//
// Interpolation P (region::interpolation + interpolate_full/partial,
// mg_3d_template/region.cc:1816-1843, 2061-2121) is a tensor product of 1-D
// maps: an even fine index coincides with coarse f/2 (weight 1); an odd one
// takes 1/2 from each of (f-1)/2 and (f+1)/2 (the latter wrapped in a
// periodic dimension), except the last node of an even non-periodic dimension,
// which coincides with the last coarse node.  Restriction
// (region::restriction + restrict_full/partial, region.cc:1766-1812,
// 2129-2271) is (1/8) P^T of the fine residual, gathered per coarse node,
// including one quirk of the reference kept for parity: for the fine node at
// sub-position (0,1,1) of a coarse cell, restrict_partial (mask 145) splits
// between the two y parents according to the cell's x-collapse flag.
#include "launch.h"
#include "transfer.cuh"

namespace stzmg {

constexpr int kTB = 256;

// Restriction, one thread per coarse node on a 3-D grid (blockDim 32 x 8,
// grid z = coarse planes).  Nodes away from non-periodic edges take the
// regular path: all 27 children with the fixed weights (1/8)(1/2,1,1/2)^3.
__device__ inline bool regular_dim(int I, int mc, int mf, int prd) {
    if (prd) return true;
    return I >= 1 && 2 * I + 1 < mf && ((mf & 1) || I < mc - 2);
}

template <typename T>
__global__ void restriction_kernel(Geom gf, Geom gc, const T *__restrict__ res, T *__restrict__ rc) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y, K = blockIdx.z;
    if (I >= gc.m || J >= gc.n) return;
    const int p = slot(gc, I, J, K);
    T acc[3] = {T(0), T(0), T(0)};
    if (regular_dim(I, gc.m, gf.m, gf.xp) && regular_dim(J, gc.n, gf.n, gf.yp) && regular_dim(K, gc.o, gf.o, gf.zp)) {
        int fx[3], fy[3], fz[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            fx[d] = wrapi(2 * I + d - 1, gf.m);
            fy[d] = wrapi(2 * J + d - 1, gf.n);
            fz[d] = wrapi(2 * K + d - 1, gf.o);
        }
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    // 0.125 * wx * wy * wz with w = 1 at the centre child, 1/2 off it
                    const T w = T(0.125) * (c == 1 ? T(1) : T(0.5)) * (b == 1 ? T(1) : T(0.5)) * (a == 1 ? T(1) : T(0.5));
                    T v[3];
                    load3(res, gf.npad, slot(gf, fx[c], fy[b], fz[a]), v);
                    acc[0] += w * v[0];
                    acc[1] += w * v[1];
                    acc[2] += w * v[2];
                }
    } else {
        restrict_node<T>(gf, gc, res, p, I, J, K, acc);
    }
    rc[p] = acc[0];
    rc[p + gc.npad] = acc[1];
    rc[p + 2 * gc.npad] = acc[2];
}

// Interpolation, one thread per coarse cell (ci,cj,ck): the cell's 8 corner
// values are loaded once and added, with the weights of P, to the fine nodes
// 2c + s, s in {0,1}^3, that exist.  Every fine node belongs to exactly one
// cell (c = f >> 1).
template <typename T>
__global__ void interpolation_kernel(Geom gf, Geom gc, const T *__restrict__ xc, T *__restrict__ xf) {
    const int ci = blockIdx.x * blockDim.x + threadIdx.x, cj = blockIdx.y * blockDim.y + threadIdx.y, ck = blockIdx.z;
    if (ci >= gc.m || cj >= gc.n) return;
    const int c[3] = {ci, cj, ck}, mc[3] = {gc.m, gc.n, gc.o}, mf[3] = {gf.m, gf.n, gf.o},
              prd[3] = {gf.xp, gf.yp, gf.zp};
    int up[3];      // wrapped c+1 (or -1)
    bool ex[3][2];  // child s exists
    bool col[3];    // child s=1 coincides with coarse c+1 (collapse)
#pragma unroll
    for (int d = 0; d < 3; d++) {
        up[d] = c[d] + 1 < mc[d] ? c[d] + 1 : (prd[d] ? 0 : -1);
        ex[d][0] = 2 * c[d] < mf[d];
        ex[d][1] = 2 * c[d] + 1 < mf[d];
        col[d] = !prd[d] && !(mf[d] & 1) && 2 * c[d] + 1 == mf[d] - 1;
    }
    T v[2][2][2][3];
#pragma unroll
    for (int az = 0; az < 2; az++)
#pragma unroll
        for (int ay = 0; ay < 2; ay++)
#pragma unroll
            for (int ax = 0; ax < 2; ax++) {
                const int X = ax ? up[0] : ci, Y = ay ? up[1] : cj, Z = az ? up[2] : ck;
                if (X < 0 || Y < 0 || Z < 0) {
                    v[az][ay][ax][0] = v[az][ay][ax][1] = v[az][ay][ax][2] = T(0);
                } else {
                    load3(xc, gc.npad, slot(gc, X, Y, Z), v[az][ay][ax]);
                }
            }
    // the 8 fine values first (all loads in flight together), then the sums
    // and the stores: the stores cannot be moved ahead of later loads
    T f[2][2][2][3];
    int fp[2][2][2];
#pragma unroll
    for (int sz = 0; sz < 2; sz++)
#pragma unroll
        for (int sy = 0; sy < 2; sy++)
#pragma unroll
            for (int sx = 0; sx < 2; sx++) {
                const bool here = ex[2][sz] && ex[1][sy] && ex[0][sx];
                fp[sz][sy][sx] = here ? slot(gf, 2 * ci + sx, 2 * cj + sy, 2 * ck + sz) : -1;
                if (here) load3(xf, gf.npad, fp[sz][sy][sx], f[sz][sy][sx]);
            }
#pragma unroll
    for (int sz = 0; sz < 2; sz++) {
#pragma unroll
        for (int sy = 0; sy < 2; sy++) {
#pragma unroll
            for (int sx = 0; sx < 2; sx++) {
                const int p = fp[sz][sy][sx];
                if (p < 0) continue;
                // parents per dimension: s = 0 -> {c}; s = 1 -> {c, c+1} or {c+1} (collapse)
                const int z0 = (sz && col[2]) ? 1 : 0, z1 = sz && !col[2] ? 1 : z0;
                const int y0 = (sy && col[1]) ? 1 : 0, y1 = sy && !col[1] ? 1 : y0;
                const int x0 = (sx && col[0]) ? 1 : 0, x1 = sx && !col[0] ? 1 : x0;
                T s3[3] = {T(0), T(0), T(0)};
                int cnt = 0;
#pragma unroll
                for (int az = 0; az < 2; az++)
#pragma unroll
                    for (int ay = 0; ay < 2; ay++)
#pragma unroll
                        for (int ax = 0; ax < 2; ax++) {
                            if (az < z0 || az > z1 || ay < y0 || ay > y1 || ax < x0 || ax > x1) continue;
                            s3[0] += v[az][ay][ax][0];
                            s3[1] += v[az][ay][ax][1];
                            s3[2] += v[az][ay][ax][2];
                            cnt++;
                        }
                const T w = T(1) / T(cnt);
                xf[p] = f[sz][sy][sx][0] + w * s3[0];
                xf[p + gf.npad] = f[sz][sy][sx][1] + w * s3[1];
                xf[p + 2 * gf.npad] = f[sz][sy][sx][2] + w * s3[2];
            }
        }
    }
}

template <typename T>
__global__ void nat_to_cb_kernel(Geom g, const double *__restrict__ nat, T *__restrict__ cb) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    int s = slot(g, i, j, k);
    cb[s] = (T)nat[3 * t];
    cb[s + g.npad] = (T)nat[3 * t + 1];
    cb[s + 2 * g.npad] = (T)nat[3 * t + 2];
}

template <typename T>
__global__ void cb_to_nat_kernel(Geom g, const T *__restrict__ cb, double *__restrict__ nat) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    int s = slot(g, i, j, k);
    nat[3 * t] = (double)cb[s];
    nat[3 * t + 1] = (double)cb[s + g.npad];
    nat[3 * t + 2] = (double)cb[s + 2 * g.npad];
}

template <typename T>
__global__ void scalar_nat_to_cb_kernel(Geom g, const double *__restrict__ nat, T *__restrict__ cb) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    cb[slot(g, i, j, k)] = (T)nat[t];
}

__global__ void coef_nat_to_cb_kernel(Geom g, const double *__restrict__ nat, double *__restrict__ cb) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    size_t s = slot(g, i, j, k);
    // a Dirichlet node keeps only its centre block (fill_entries stores one entry for it)
    const bool in = is_interior(g, i, j, k);
    for (int e = 0; e < 243; e++) cb[(size_t)e * g.npad + s] = (in || e / 9 == 13) ? nat[243 * t + e] : 0.0;
}

__global__ void coef_cb_to_nat_kernel(Geom g, const double *__restrict__ cb, double *__restrict__ nat) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    size_t s = slot(g, i, j, k);
    for (int e = 0; e < 243; e++) nat[243 * t + e] = cb[(size_t)e * g.npad + s];
}

__global__ void convert_kernel(const double *__restrict__ src, float *__restrict__ dst, size_t n) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; t < n; t += (size_t)gridDim.x * blockDim.x) dst[t] = (float)src[t];
}

__global__ void add_correction_kernel(double *__restrict__ x, const float *__restrict__ e, size_t n) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; t < n; t += (size_t)gridDim.x * blockDim.x) x[t] += (double)e[t];
}

__global__ void scale_kernel(double *__restrict__ v, double s, size_t n) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; t < n; t += (size_t)gridDim.x * blockDim.x) v[t] *= s;
}

// x = Ainv r with one warp per row (Ainv row-major, lanes stride the columns).
template <typename T>
__global__ void bottom_direct_kernel(int nrow, const double *__restrict__ ainv, const int *__restrict__ nat_slot,
                                     int npad, const T *__restrict__ r, T *__restrict__ x) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= nrow) return;
    double acc = 0.0;
    const double *a = ainv + (size_t)row * nrow;
    for (int col = lane; col < nrow; col += 32) {
        int s = nat_slot[col / 3] + (col % 3) * npad;
        acc += a[col] * (double)r[s];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) x[nat_slot[row / 3] + (row % 3) * npad] = (T)acc;
}

// ---------------------------------------------------------------- bottom inverse
// Gauss-Jordan elimination with partial pivoting on the augmented matrix
// [M | I] (n x 2n, row-major, FP64); afterwards the right half is M^-1.
// Column c: pivot search (one block), row swap + scaling + copy of column c,
// then elimination of column c from every other row.
__global__ void gj_pivot_kernel(const double *__restrict__ a, int n, int c, int *piv, int *bad) {
    __shared__ double bv[1024];
    __shared__ int bi[1024];
    double best = -1.0;
    int arg = c;
    for (int r = c + threadIdx.x; r < n; r += blockDim.x) {
        double v = fabs(a[(size_t)r * 2 * n + c]);
        if (v > best) { best = v; arg = r; }
    }
    bv[threadIdx.x] = best;
    bi[threadIdx.x] = arg;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            double v2 = bv[threadIdx.x + o];
            int i2 = bi[threadIdx.x + o];
            if (v2 > bv[threadIdx.x] || (v2 == bv[threadIdx.x] && i2 < bi[threadIdx.x])) {
                bv[threadIdx.x] = v2;
                bi[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *piv = bi[0];
        if (!(bv[0] > 0.0) || !(bv[0] - bv[0] == 0.0)) atomicExch(bad, 1);
    }
}

__global__ void gj_swap_scale_kernel(double *__restrict__ a, int n, int c, const int *piv, double *__restrict__ col) {
    const int p = *piv;
    const size_t w = 2 * (size_t)n;
    // swap rows c and p
    for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) {
        double t = a[(size_t)c * w + q];
        a[(size_t)c * w + q] = a[(size_t)p * w + q];
        a[(size_t)p * w + q] = t;
    }
    __syncthreads();
    const double inv = 1.0 / a[(size_t)c * w + c];
    __syncthreads();
    for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) a[(size_t)c * w + q] *= inv;
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) col[r] = r == c ? 0.0 : a[(size_t)r * w + c];
}

__global__ void gj_eliminate_kernel(double *__restrict__ a, int n, int c, const double *__restrict__ col) {
    const size_t w = 2 * (size_t)n;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (q >= 2 * n) return;
    const double f = col[r];
    if (f != 0.0) a[(size_t)r * w + q] -= f * a[(size_t)c * w + q];
}

__global__ void gj_extract_kernel(const double *__restrict__ a, int n, double *__restrict__ inv) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)n * n) return;
    size_t r = t / n, q = t % n;
    inv[t] = a[r * 2 * n + n + q];
}

void launch_gauss_jordan(double *aug, int n, double *inv, int *piv, double *col, int *bad, cudaStream_t st) {
    dim3 eg((2 * n + 255) / 256, n);
    for (int c = 0; c < n; c++) {
        gj_pivot_kernel<<<1, 1024, 0, st>>>(aug, n, c, piv, bad);
        gj_swap_scale_kernel<<<1, 1024, 0, st>>>(aug, n, c, piv, col);
        gj_eliminate_kernel<<<eg, 256, 0, st>>>(aug, n, c, col);
    }
    gj_extract_kernel<<<(unsigned)(((size_t)n * n + 255) / 256), 256, 0, st>>>(aug, n, inv);
}

static inline unsigned blocks_for(long n) { return (unsigned)((n + kTB - 1) / kTB); }
static inline unsigned grid_stride_blocks(size_t n) {
    size_t b = (n + kTB - 1) / kTB;
    return (unsigned)(b > 152 * 16 ? 152 * 16 : (b ? b : 1));
}

template <typename T>
void launch_restriction(const Geom &gf, const Geom &gc, const T *res_f, T *r_c, cudaStream_t st) {
    dim3 blk(32, 8), grd((gc.m + 31) / 32, (gc.n + 7) / 8, gc.o);
    restriction_kernel<T><<<grd, blk, 0, st>>>(gf, gc, res_f, r_c);
}
template <typename T>
void launch_interpolation(const Geom &gf, const Geom &gc, const T *x_c, T *x_f, cudaStream_t st) {
    dim3 blk(32, 8), grd((gc.m + 31) / 32, (gc.n + 7) / 8, gc.o);
    interpolation_kernel<T><<<grd, blk, 0, st>>>(gf, gc, x_c, x_f);
}
template <typename T>
void launch_nat_to_cb(const Geom &g, const double *nat, T *cb, cudaStream_t st) {
    nat_to_cb_kernel<T><<<blocks_for((long)g.m * g.n * g.o), kTB, 0, st>>>(g, nat, cb);
}
template <typename T>
void launch_cb_to_nat(const Geom &g, const T *cb, double *nat, cudaStream_t st) {
    cb_to_nat_kernel<T><<<blocks_for((long)g.m * g.n * g.o), kTB, 0, st>>>(g, cb, nat);
}
template <typename T>
void launch_scalar_nat_to_cb(const Geom &g, const double *nat, T *cb, cudaStream_t st) {
    scalar_nat_to_cb_kernel<T><<<blocks_for((long)g.m * g.n * g.o), kTB, 0, st>>>(g, nat, cb);
}
void launch_coef_nat_to_cb(const Geom &g, const double *nat, double *cb, cudaStream_t st) {
    coef_nat_to_cb_kernel<<<blocks_for((long)g.m * g.n * g.o), kTB, 0, st>>>(g, nat, cb);
}
void launch_coef_cb_to_nat(const Geom &g, const double *cb, double *nat, cudaStream_t st) {
    coef_cb_to_nat_kernel<<<blocks_for((long)g.m * g.n * g.o), kTB, 0, st>>>(g, cb, nat);
}
void launch_convert(const double *src, float *dst, size_t n, cudaStream_t st) {
    convert_kernel<<<grid_stride_blocks(n), kTB, 0, st>>>(src, dst, n);
}
void launch_add_correction(double *x, const float *e, size_t n, cudaStream_t st) {
    add_correction_kernel<<<grid_stride_blocks(n), kTB, 0, st>>>(x, e, n);
}
void launch_scale(double *v, double s, size_t n, cudaStream_t st) {
    scale_kernel<<<grid_stride_blocks(n), kTB, 0, st>>>(v, s, n);
}
template <typename T>
void launch_bottom_direct(int nrow, const double *ainv_t, const int *nat_slot, int npad, const T *r, T *x,
                          cudaStream_t st) {
    bottom_direct_kernel<T><<<blocks_for(32L * nrow), kTB, 0, st>>>(nrow, ainv_t, nat_slot, npad, r, x);
}

template void launch_restriction<float>(const Geom &, const Geom &, const float *, float *, cudaStream_t);
template void launch_restriction<double>(const Geom &, const Geom &, const double *, double *, cudaStream_t);
template void launch_interpolation<float>(const Geom &, const Geom &, const float *, float *, cudaStream_t);
template void launch_interpolation<double>(const Geom &, const Geom &, const double *, double *, cudaStream_t);
template void launch_nat_to_cb<float>(const Geom &, const double *, float *, cudaStream_t);
template void launch_nat_to_cb<double>(const Geom &, const double *, double *, cudaStream_t);
template void launch_cb_to_nat<float>(const Geom &, const float *, double *, cudaStream_t);
template void launch_cb_to_nat<double>(const Geom &, const double *, double *, cudaStream_t);
template void launch_scalar_nat_to_cb<float>(const Geom &, const double *, float *, cudaStream_t);
template void launch_scalar_nat_to_cb<double>(const Geom &, const double *, double *, cudaStream_t);
template void launch_bottom_direct<float>(int, const double *, const int *, int, const float *, float *, cudaStream_t);
template void launch_bottom_direct<double>(int, const double *, const int *, int, const double *, double *, cudaStream_t);

}  // namespace stzmg
