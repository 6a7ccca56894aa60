// Multicolour block Gauss-Seidel and residual kernels.
//
// Replaces the lexicographic sweep of region::gauss_seidel
// (mg_3d_template/region.cc:1557-1762) by an 8-colour sweep: colour
// q = (i&1) + 2(j&1) + 4(k&1) is updated by one launch, all its nodes in
// parallel, each reading the current values of the other colours
// (x_c = inv(A_c)(r - sum_{q != c} A_q x_q)).  For even periodic sizes no two
// nodes of a colour are coupled, so a colour pass is order independent.
// The residual kernel is region::residual (region.cc:1008-1055) over all
// nodes, with an optional sum of |r|^2 reduced per block in FP64 (warp
// shuffles) into a partial-sum array, then summed by one block, so the norm
// is deterministic.
#include "launch.h"
#include "ops.cuh"

namespace stzmg {

constexpr int kBlock = 256;

// ------------------------------------------------------------------ GS
template <typename T, bool ELASTIC>
__global__ void __launch_bounds__(kBlock) gs_const_kernel(Geom g, int q, const __grid_constant__ ConstOp<T> op,
                                                          const T *__restrict__ r, T *__restrict__ x) {
    int t = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (t >= g.S || !colour_node(g, q, t, i, j, k)) return;
    const int p = q * g.S + t;
    T acc[3];
    load3(r, g.npad, p, acc);
    const T *inv;
    if (is_interior(g, i, j, k)) {
        NbrOffsets nb = nbr_offsets(g, i, j, k);
        const_row<T, ELASTIC, false>(op, g, nb, x, acc);
        inv = op.inv_int;
    } else {
        inv = op.inv_fix;
    }
    x[p] = inv[0] * acc[0] + inv[1] * acc[1] + inv[2] * acc[2];
    x[p + g.npad] = inv[3] * acc[0] + inv[4] * acc[1] + inv[5] * acc[2];
    x[p + 2 * g.npad] = inv[6] * acc[0] + inv[7] * acc[1] + inv[8] * acc[2];
}

template <typename T>
__global__ void __launch_bounds__(kBlock) gs_lame_kernel(Geom g, int q, LameOp<T> op, const T *__restrict__ r,
                                                         T *__restrict__ x) {
    int t = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (t >= g.S || !colour_node(g, q, t, i, j, k)) return;
    const int p = q * g.S + t;
    T acc[3];
    load3(r, g.npad, p, acc);
    if (is_interior(g, i, j, k)) {
        NbrOffsets nb = nbr_offsets(g, i, j, k);
        T cen[3];
        lame_row<T, false>(op, g, nb, p, x, acc, cen);
        x[p] = acc[0] / cen[0];
        x[p + g.npad] = acc[1] / cen[1];
        x[p + 2 * g.npad] = acc[2] / cen[2];
    } else {
        T f = lame_fix(op, p);
        x[p] = acc[0] / f;
        x[p + g.npad] = acc[1] / f;
        x[p + 2 * g.npad] = acc[2] / f;
    }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) gs_dense_kernel(Geom g, int q, DenseOp<T> op, const T *__restrict__ r,
                                                          T *__restrict__ x) {
    int t = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (t >= g.S || !colour_node(g, q, t, i, j, k)) return;
    const int p = q * g.S + t;
    T acc[3];
    load3(r, g.npad, p, acc);
    NbrOffsets nb = nbr_offsets(g, i, j, k);
    dense_row<T, false>(op, g, nb, p, x, acc);
    const size_t np = (size_t)g.npad;
    T inv[9];
#pragma unroll
    for (int e = 0; e < 9; e++) inv[e] = __ldg(op.dinv + (size_t)e * np + p);
    x[p] = inv[0] * acc[0] + inv[1] * acc[1] + inv[2] * acc[2];
    x[p + g.npad] = inv[3] * acc[0] + inv[4] * acc[1] + inv[5] * acc[2];
    x[p + 2 * g.npad] = inv[6] * acc[0] + inv[7] * acc[1] + inv[8] * acc[2];
}

// ------------------------------------------------------------- residual
template <typename T>
__device__ inline void block_sum_sq(double v, double *partial) {
    __shared__ double red[kBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < kBlock / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

// res (type R) = r - A x over every slot (unused slots get 0).  When partial
// is non-null each block writes sum |res|^2 (computed in FP64 from the
// residual before rounding to R) to partial[blockIdx.x].
template <typename T, typename R, int KIND, bool ELASTIC>
__global__ void __launch_bounds__(kBlock) residual_kernel(Geom g, const __grid_constant__ ConstOp<T> cop, LameOp<T> lop,
                                                          DenseOp<T> dop, const T *__restrict__ r,
                                                          const T *__restrict__ x, R *__restrict__ res,
                                                          double *__restrict__ partial) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    double sq = 0.0;
    if (p < g.npad) {
        T acc[3] = {T(0), T(0), T(0)};
        if (slot_node(g, p, i, j, k)) {
            load3(r, g.npad, p, acc);
            if (KIND == OP_DENSE) {
                NbrOffsets nb = nbr_offsets(g, i, j, k);
                dense_row<T, true>(dop, g, nb, p, x, acc);
            } else if (is_interior(g, i, j, k)) {
                NbrOffsets nb = nbr_offsets(g, i, j, k);
                if (KIND == OP_CONST) const_row<T, ELASTIC, true>(cop, g, nb, x, acc);
                else lame_row<T, true>(lop, g, nb, p, x, acc, nullptr);
            } else {
                T v[3];
                load3(x, g.npad, p, v);
                if (KIND == OP_CONST) {
                    matvec_sub(cop.fix, v, acc);
                } else {
                    T f = lame_fix(lop, p);
                    acc[0] -= f * v[0]; acc[1] -= f * v[1]; acc[2] -= f * v[2];
                }
            }
            sq = (double)acc[0] * (double)acc[0] + (double)acc[1] * (double)acc[1] + (double)acc[2] * (double)acc[2];
        }
        if (res) {
            res[p] = (R)acc[0];
            res[p + g.npad] = (R)acc[1];
            res[p + 2 * g.npad] = (R)acc[2];
        }
    }
    if (partial) block_sum_sq<T>(sq, partial);
}

__global__ void sum_partials_kernel(const double *__restrict__ partial, int n, double *__restrict__ out) {
    __shared__ double red[1024 / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (int)(blockDim.x / 32) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) out[0] = v;
    }
}

// ------------------------------------------------------------- launchers
template <typename T>
void launch_gs_colour(const LevelOp<T> &op, const Geom &g, int q, const T *r, T *x, cudaStream_t st) {
    int blocks = (g.S + kBlock - 1) / kBlock;
    switch (op.kind) {
        case OP_CONST:
            if (op.cop.elastic) gs_const_kernel<T, true><<<blocks, kBlock, 0, st>>>(g, q, op.cop, r, x);
            else gs_const_kernel<T, false><<<blocks, kBlock, 0, st>>>(g, q, op.cop, r, x);
            break;
        case OP_LAME: gs_lame_kernel<T><<<blocks, kBlock, 0, st>>>(g, q, op.lop, r, x); break;
        default: gs_dense_kernel<T><<<blocks, kBlock, 0, st>>>(g, q, op.dop, r, x); break;
    }
}

template <typename T>
void launch_gs_sweep(const LevelOp<T> &op, const Geom &g, const T *r, T *x, cudaStream_t st) {
    for (int q = 0; q < 8; q++) launch_gs_colour(op, g, q, r, x, st);
}

int residual_blocks(const Geom &g) { return (g.npad + kBlock - 1) / kBlock; }

template <typename T, typename R>
void launch_residual(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, R *res, double *partial,
                     double *out, cudaStream_t st) {
    int blocks = residual_blocks(g);
    switch (op.kind) {
        case OP_CONST:
            if (op.cop.elastic)
                residual_kernel<T, R, OP_CONST, true><<<blocks, kBlock, 0, st>>>(g, op.cop, op.lop, op.dop, r, x, res, partial);
            else
                residual_kernel<T, R, OP_CONST, false><<<blocks, kBlock, 0, st>>>(g, op.cop, op.lop, op.dop, r, x, res, partial);
            break;
        case OP_LAME:
            residual_kernel<T, R, OP_LAME, false><<<blocks, kBlock, 0, st>>>(g, op.cop, op.lop, op.dop, r, x, res, partial);
            break;
        default:
            residual_kernel<T, R, OP_DENSE, false><<<blocks, kBlock, 0, st>>>(g, op.cop, op.lop, op.dop, r, x, res, partial);
            break;
    }
    if (partial && out) sum_partials_kernel<<<1, 1024, 0, st>>>(partial, blocks, out);
}

template void launch_gs_colour<float>(const LevelOp<float> &, const Geom &, int, const float *, float *, cudaStream_t);
template void launch_gs_colour<double>(const LevelOp<double> &, const Geom &, int, const double *, double *, cudaStream_t);
template void launch_gs_sweep<float>(const LevelOp<float> &, const Geom &, const float *, float *, cudaStream_t);
template void launch_gs_sweep<double>(const LevelOp<double> &, const Geom &, const double *, double *, cudaStream_t);
template void launch_residual<float, float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *, double *, double *, cudaStream_t);
template void launch_residual<double, double>(const LevelOp<double> &, const Geom &, const double *, const double *, double *, double *, double *, cudaStream_t);
template void launch_residual<double, float>(const LevelOp<double> &, const Geom &, const double *, const double *, float *, double *, double *, cudaStream_t);

}  // namespace stzmg
