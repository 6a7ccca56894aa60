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

namespace stzmg {

constexpr int kTB = 256;

// Weight of fine index f (unwrapped, f in {2I-1, 2I, 2I+1}) as a child of
// coarse index I along one dimension: 1, 0.5, or 0 when f is not a child.
__host__ __device__ inline double child_w(int I, int f, int mf, int prd) {
    if (!prd && (f < 0 || f >= mf)) return 0.0;
    const bool collapse_dim = !prd && !(mf & 1);   // last fine node coincides with last coarse node
    if (f == 2 * I) return 1.0;                     // (2I < mf guaranteed by the range test above)
    if (f == 2 * I - 1) return (collapse_dim && f == mf - 1) ? 1.0 : 0.5;
    /* f == 2I + 1 */
    return (collapse_dim && f == mf - 1) ? 0.0 : 0.5;
}

__device__ inline int wrapi(int a, int len) {
    if (a < 0) return a + len;
    if (a >= len) return a - len;
    return a;
}

template <typename T>
__global__ void restriction_kernel(Geom gf, Geom gc, const T *__restrict__ res, T *__restrict__ rc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, I, J, K;
    if (p >= gc.npad) return;
    double acc[3] = {0.0, 0.0, 0.0};
    if (slot_node(gc, p, I, J, K)) {
        const bool xs = !gf.xp && !(gf.m & 1) && I == gc.m - 2;
        for (int dz = -1; dz <= 1; dz++) {
            int fz = 2 * K + dz;
            double wz = child_w(K, fz, gf.o, gf.zp);
            if (wz == 0.0) continue;
            int fzw = wrapi(fz, gf.o);
            for (int dy = -1; dy <= 1; dy++) {
                int fy = 2 * J + dy;
                double wy = child_w(J, fy, gf.n, gf.yp);
                if (!gf.yp && (fy < 0 || fy >= gf.n)) continue;
                int fyw = wrapi(fy, gf.n);
                for (int dx = -1; dx <= 1; dx++) {
                    int fx = 2 * I + dx;
                    double wx = child_w(I, fx, gf.m, gf.xp);
                    if (wx == 0.0) continue;
                    double wyy = wy;
                    if (dx == 0 && (fy & 1) && (fz & 1)) wyy = xs ? (dy < 0 ? 1.0 : 0.0) : 0.5;
                    if (wyy == 0.0) continue;
                    int s = slot(gf, wrapi(fx, gf.m), fyw, fzw);
                    double w = 0.125 * wx * wyy * wz;
                    acc[0] += w * (double)res[s];
                    acc[1] += w * (double)res[s + gf.npad];
                    acc[2] += w * (double)res[s + 2 * gf.npad];
                }
            }
        }
    }
    rc[p] = (T)acc[0];
    rc[p + gc.npad] = (T)acc[1];
    rc[p + 2 * gc.npad] = (T)acc[2];
}

// Parents of fine index f (wrapped coarse indices) and their common weight.
__device__ inline int parents(int f, int mf, int mc, int prd, int *c, double *w) {
    if ((f & 1) == 0) { c[0] = f >> 1; *w = 1.0; return 1; }
    if (!prd && !(mf & 1) && f == mf - 1) { c[0] = (f >> 1) + 1; *w = 1.0; return 1; }
    c[0] = f >> 1;
    c[1] = wrapi((f >> 1) + 1, mc);
    *w = 0.5;
    return 2;
}

template <typename T>
__global__ void interpolation_kernel(Geom gf, Geom gc, const T *__restrict__ xc, T *__restrict__ xf) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (p >= gf.npad || !slot_node(gf, p, i, j, k)) return;
    int cx[2], cy[2], cz[2];
    double wx, wy, wz;
    int nx = parents(i, gf.m, gc.m, gf.xp, cx, &wx);
    int ny = parents(j, gf.n, gc.n, gf.yp, cy, &wy);
    int nz = parents(k, gf.o, gc.o, gf.zp, cz, &wz);
    T s[3] = {T(0), T(0), T(0)};
    for (int a = 0; a < nz; a++)
        for (int b = 0; b < ny; b++)
            for (int c = 0; c < nx; c++) {
                int q = slot(gc, cx[c], cy[b], cz[a]);
                s[0] += xc[q];
                s[1] += xc[q + gc.npad];
                s[2] += xc[q + 2 * gc.npad];
            }
    const T w = (T)(wx * wy * wz);
    xf[p] += w * s[0];
    xf[p + gf.npad] += w * s[1];
    xf[p + 2 * gf.npad] += w * s[2];
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

template <typename T>
__global__ void bottom_direct_kernel(int nrow, const double *__restrict__ ainv_t, const int *__restrict__ nat_slot,
                                     int npad, const T *__restrict__ r, T *__restrict__ x) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    double acc = 0.0;
    for (int col = 0; col < nrow; col++) {
        int s = nat_slot[col / 3] + (col % 3) * npad;
        acc += ainv_t[(size_t)col * nrow + row] * (double)r[s];
    }
    x[nat_slot[row / 3] + (row % 3) * npad] = (T)acc;
}

static inline unsigned blocks_for(long n) { return (unsigned)((n + kTB - 1) / kTB); }
static inline unsigned grid_stride_blocks(size_t n) {
    size_t b = (n + kTB - 1) / kTB;
    return (unsigned)(b > 152 * 16 ? 152 * 16 : (b ? b : 1));
}

template <typename T>
void launch_restriction(const Geom &gf, const Geom &gc, const T *res_f, T *r_c, cudaStream_t st) {
    restriction_kernel<T><<<blocks_for(gc.npad), kTB, 0, st>>>(gf, gc, res_f, r_c);
}
template <typename T>
void launch_interpolation(const Geom &gf, const Geom &gc, const T *x_c, T *x_f, cudaStream_t st) {
    interpolation_kernel<T><<<blocks_for(gf.npad), kTB, 0, st>>>(gf, gc, x_c, x_f);
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
    bottom_direct_kernel<T><<<blocks_for(nrow), kTB, 0, st>>>(nrow, ainv_t, nat_slot, npad, r, x);
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
