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
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "launch.h"
#include "ops.cuh"

namespace stzmg {

constexpr int kBlock = 256;

// Colour kernels run on a 3-D grid: block (32, 8), grid (ceil(M2/32),
// ceil(N2/8), number of sub-grid planes); thread -> sub-grid coordinates
// (I, J, K) of colour q; the sub-grid planes K in reverse order when rev.
#define COLOUR_NODE_PROLOGUE                                                                    \
    const int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y; \
    const int K = rev ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;                     \
    if (I >= g.M2 || J >= g.N2) return;                                                         \
    const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);             \
    if (i >= g.m || j >= g.n || k >= g.o) return;                                               \
    const int p = q * g.S + (K * g.N2 + J) * g.M2 + I;

// ------------------------------------------------------------------ GS
template <typename T, bool ELASTIC>
__global__ void __launch_bounds__(kBlock) gs_const_kernel(Geom g, int q, int rev, const __grid_constant__ ConstOp<T> op,
                                                          const T *__restrict__ r, T *__restrict__ x) {
    COLOUR_NODE_PROLOGUE
    T acc[3];
    load3(r, g.npad, p, acc);
    const T *inv;
    if (is_interior(g, i, j, k)) {
        NbrOffsets nb = nbr_offsets_sub(g, I, J, K, q & 1, (q >> 1) & 1, q >> 2);
        const_row<T, ELASTIC, false>(op, g, nb, x, acc);
        inv = op.inv_int;
    } else {
        inv = op.inv_fix;
    }
    x[p] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
    x[p + g.npad] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
    x[p + 2 * g.npad] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) gs_lame_kernel(Geom g, int q, int rev, LameOp<T> op, const T *__restrict__ r,
                                                         T *__restrict__ x) {
    COLOUR_NODE_PROLOGUE
    T acc[3];
    load3(r, g.npad, p, acc);
    if (is_interior(g, i, j, k)) {
        NbrOffsets nb = nbr_offsets_sub(g, I, J, K, q & 1, (q >> 1) & 1, q >> 2);
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
__global__ void __launch_bounds__(kBlock) gs_dense_kernel(Geom g, int q, int rev, DenseOp<T> op, const T *__restrict__ r,
                                                          T *__restrict__ x) {
    COLOUR_NODE_PROLOGUE
    T acc[3];
    load3(r, g.npad, p, acc);
    NbrOffsets nb = nbr_offsets_sub(g, I, J, K, q & 1, (q >> 1) & 1, q >> 2);
    dense_row<T, false>(op, g, nb, p, x, acc);
    const size_t np = (size_t)g.npad;
    T inv[9];
#pragma unroll
    for (int e = 0; e < 9; e++) inv[e] = __ldg(op.dinv + (size_t)e * np + p);
    x[p] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
    x[p + g.npad] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
    x[p + 2 * g.npad] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
}

// Plane-invariant levels: every block of the 3-D grid lies on one sub-grid
// plane, so the row of that plane (243 block entries and the 9 entries of the
// inverse centre block) is staged in shared memory once per block.
template <typename T, bool SPARSE>
__global__ void __launch_bounds__(kBlock) gs_plane_kernel(Geom g, int q, int rev, PlaneOp<T> op, const T *__restrict__ r,
                                                          T *__restrict__ x) {
    __shared__ T cf[252];
    {
        const int k = 2 * (rev ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z) + (q >> 2);
        for (int e = threadIdx.y * blockDim.x + threadIdx.x; e < 252; e += blockDim.x * blockDim.y)
            cf[e] = k < g.o ? (e < 243 ? op.coef[e * op.O + k] : op.dinv[(e - 243) * op.O + k]) : T(0);
        __syncthreads();
    }
    COLOUR_NODE_PROLOGUE
    T acc[3];
    load3(r, g.npad, p, acc);
    NbrOffsets nb = nbr_offsets_sub(g, I, J, K, q & 1, (q >> 1) & 1, q >> 2);
    plane_row_coef<T, SPARSE, false>(cf, 1, g, nb, x, acc);
    const T *inv = cf + 243;
    x[p] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
    x[p + g.npad] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
    x[p + 2 * g.npad] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
}

// ------------------------------------------------------ plane-phase sweep
// Colours 0-3 live on even z-planes and colours 4-7 on odd ones, and a
// colour only couples to the other colours of its plane and to the planes
// above and below.  So one block can run colours 4c .. 4c+3 of one plane in
// order, separated by __syncthreads, without any dependency on other blocks:
// a full 8-colour sweep is two launches (even planes, then odd planes), with
// the same arithmetic and the same result as eight colour launches.
template <typename T, int KIND, bool ELASTIC, bool SPARSE>
__device__ inline void gs_node(const LevelOp<T> &op, const Geom &g, int q, int I, int J, int K, const T *cf,
                               const T *__restrict__ r, T *__restrict__ x) {
    const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + ((q >> 2) & 1);
    if (i >= g.m || j >= g.n || k >= g.o) return;
    const int p = q * g.S + (K * g.N2 + J) * g.M2 + I;
    T acc[3];
    load3(r, g.npad, p, acc);
    NbrOffsets nb = nbr_offsets(g, i, j, k);
    T inv[9];
    if (KIND == OP_CONST) {
        const T *src;
        if (is_interior(g, i, j, k)) {
            const_row<T, ELASTIC, false>(op.cop, g, nb, x, acc);
            src = op.cop.inv_int;
        } else {
            src = op.cop.inv_fix;
        }
#pragma unroll
        for (int e = 0; e < 9; e++) inv[e] = src[e];
    } else if (KIND == OP_LAME) {
        T c3[3];
        if (is_interior(g, i, j, k)) {
            lame_row<T, false>(op.lop, g, nb, p, x, acc, c3);
        } else {
            c3[0] = c3[1] = c3[2] = lame_fix(op.lop, p);
        }
        x[p] = acc[0] / c3[0];
        x[p + g.npad] = acc[1] / c3[1];
        x[p + 2 * g.npad] = acc[2] / c3[2];
        return;
    } else if (KIND == OP_PLANE) {
        plane_row_coef<T, SPARSE, false>(cf, 1, g, nb, x, acc);
#pragma unroll
        for (int e = 0; e < 9; e++) inv[e] = cf[243 + e];
    } else {
        dense_row<T, false>(op.dop, g, nb, p, x, acc);
        const size_t np = (size_t)g.npad;
#pragma unroll
        for (int e = 0; e < 9; e++) inv[e] = __ldg(op.dop.dinv + (size_t)e * np + p);
    }
    x[p] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
    x[p + g.npad] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
    x[p + 2 * g.npad] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
}

constexpr int kPhaseThreads = 512;

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
__global__ void __launch_bounds__(kPhaseThreads) gs_phase_kernel(Geom g, int c, const __grid_constant__ LevelOp<T> op,
                                                                 const T *__restrict__ r, T *__restrict__ x) {
    __shared__ T cf[252];
    const int K = blockIdx.x;   // sub-grid plane: node plane k = 2K + c
    if (KIND == OP_PLANE) {
        const int k = 2 * K + c;
        for (int e = threadIdx.x; e < 252; e += blockDim.x)
            cf[e] = k < g.o ? (e < 243 ? op.pop.coef[e * op.pop.O + k] : op.pop.dinv[(e - 243) * op.pop.O + k]) : T(0);
        __syncthreads();
    }
    const int plane = g.M2 * g.N2;
    for (int qxy = 0; qxy < 4; qxy++) {
        const int q = qxy + 4 * c;
        for (int t = threadIdx.x; t < plane; t += blockDim.x) {
            // keep the shared-memory coefficient reads inside the loop (hoisting
            // all 243 of them into registers would spill)
            asm volatile("" ::: "memory");
            const int J = t / g.M2, I = t - J * g.M2;
            gs_node<T, KIND, ELASTIC, SPARSE>(op, g, q, I, J, K, cf, r, x);
        }
        __syncthreads();
    }
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
static void launch_phases(const LevelOp<T> &op, const Geom &g, const T *r, T *x, cudaStream_t st) {
    const int plane = g.M2 * g.N2;
    const int threads = plane >= kPhaseThreads ? kPhaseThreads : ((plane + 31) / 32) * 32;
    const int even = (g.o + 1) / 2, odd = g.o / 2;
    gs_phase_kernel<T, KIND, ELASTIC, SPARSE><<<even, threads, 0, st>>>(g, 0, op, r, x);
    if (odd > 0) gs_phase_kernel<T, KIND, ELASTIC, SPARSE><<<odd, threads, 0, st>>>(g, 1, op, r, x);
}

// ------------------------------------------------------------- residual
template <typename T>
__device__ inline void block_sum_sq(double v, double *partial) {
    __shared__ double red[kBlock / 32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        v = tid < kBlock / 32 ? red[tid] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (tid == 0) partial[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = v;
    }
}

// res (type R) = r - A x over every slot (unused slots get 0).  When partial
// is non-null each block writes sum |res|^2 (computed in FP64 from the
// residual before rounding to R) to partial[blockIdx.x].
template <typename T, typename R, int KIND, bool ELASTIC, bool NORM>
__global__ void __launch_bounds__(kBlock) residual_kernel(Geom g, const __grid_constant__ ConstOp<T> cop, LameOp<T> lop,
                                                          DenseOp<T> dop, PlaneOp<T> pop, const T *__restrict__ r,
                                                          const T *__restrict__ x, R *__restrict__ res,
                                                          double *__restrict__ partial) {
    // block (32, 8): lanes run along x, threadIdx.y is the colour, so a block
    // covers a 64x2x2 box of nodes in all 8 colours (neighbour reads shared in L1)
    const int q = threadIdx.y;
    const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y, K = blockIdx.z;
    const int a = q & 1, b = (q >> 1) & 1, c = q >> 2;
    const int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
    double sq = 0.0;
    if (I < g.M2) {
        const int p = q * g.S + (K * g.N2 + J) * g.M2 + I;
        T acc[3] = {T(0), T(0), T(0)};
        if (i < g.m && j < g.n && k < g.o) {
            load3(r, g.npad, p, acc);
            if (KIND == OP_DENSE) {
                NbrOffsets nb = nbr_offsets_sub(g, I, J, K, a, b, c);
                dense_row<T, true>(dop, g, nb, p, x, acc);
            } else if (KIND == OP_PLANE) {
                NbrOffsets nb = nbr_offsets_sub(g, I, J, K, a, b, c);
                if (pop.sparse) plane_row_coef<T, true, true>(pop.coef + k, pop.O, g, nb, x, acc);
                else plane_row_coef<T, false, true>(pop.coef + k, pop.O, g, nb, x, acc);
            } else if (is_interior(g, i, j, k)) {
                NbrOffsets nb = nbr_offsets_sub(g, I, J, K, a, b, c);
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
            if (NORM)
                sq = (double)acc[0] * (double)acc[0] + (double)acc[1] * (double)acc[1] + (double)acc[2] * (double)acc[2];
        }
        if (res) {
            res[p] = (R)acc[0];
            res[p + g.npad] = (R)acc[1];
            res[p + 2 * g.npad] = (R)acc[2];
        }
    }
    if (NORM) block_sum_sq<T>(sq, partial);
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

void launch_sum_partials(const double *partial, int n, double *out, cudaStream_t st) {
    sum_partials_kernel<<<1, 1024, 0, st>>>(partial, n, out);
}

// ------------------------------------------------------------- launchers
// Colour q on every sub-grid plane, taken in reverse order when rev.
template <typename T>
static void launch_gs_colour_planes(const LevelOp<T> &op, const Geom &g, int q, int rev, const T *r, T *x,
                                    cudaStream_t st) {
    const dim3 blocks((g.M2 + 31) / 32, (g.N2 + 7) / 8, g.O2), blk(32, 8);
    switch (op.kind) {
        case OP_CONST:
            if (op.cop.elastic) gs_const_kernel<T, true><<<blocks, blk, 0, st>>>(g, q, rev, op.cop, r, x);
            else gs_const_kernel<T, false><<<blocks, blk, 0, st>>>(g, q, rev, op.cop, r, x);
            break;
        case OP_LAME: gs_lame_kernel<T><<<blocks, blk, 0, st>>>(g, q, rev, op.lop, r, x); break;
        case OP_PLANE:
            if (op.pop.sparse) gs_plane_kernel<T, true><<<blocks, blk, 0, st>>>(g, q, rev, op.pop, r, x);
            else gs_plane_kernel<T, false><<<blocks, blk, 0, st>>>(g, q, rev, op.pop, r, x);
            break;
        default: gs_dense_kernel<T><<<blocks, blk, 0, st>>>(g, q, rev, op.dop, r, x); break;
    }
}

template <typename T>
void launch_gs_colour(const LevelOp<T> &op, const Geom &g, int q, const T *r, T *x, cudaStream_t st) {
    // Odd colours walk the planes downwards ("snake" order): a colour pass
    // starts where the previous one ended, on neighbour sub-grids still in L2.
    // Updates within one colour are independent, so the order changes no bit.
    // Fine FP32 level, 256x256x257, two sweeps: 658 -> 614 us.
    launch_gs_colour_planes(op, g, q, q & 1, r, x, st);
}

// Large planes: one launch per colour keeps millions of threads in flight;
// the plane-phase kernels (one block per plane) pay off where a colour of a
// plane is at most two nodes per thread, i.e. where launch latency dominates.
// (An odd periodic z would put both parities of a colour on one plane.)
template <typename T>
static bool large_planes(const Geom &g) {
    const int phase_max = sizeof(T) == 8 ? 256 : 2 * kPhaseThreads;   // FP64 needs every SM's FP64 units
    return (g.zp && (g.o & 1) && g.o > 1) || g.M2 * g.N2 > phase_max;
}

template <typename T>
void launch_gs_sweeps(const LevelOp<T> &op, const Geom &g, const T *r, T *x, T *tmp, int sweeps, cudaStream_t st) {
    int s = 0;
    // pairs of sweeps x -> tmp -> x by the tiled kernel (tile.cu), which needs
    // a second buffer; a last odd sweep in place (same result either way)
    // plane-invariant levels of 64x64 and more: 4+ tiles per plane beat one
    // block per plane (64x64x65, two FP32 sweeps: 58 vs 107 us); 32x32 does not
    const bool plane_tiles = op.kind == OP_PLANE && g.m * g.n >= 64 * 64;
    // the fine level of a shared elasticity stencil: full-width bands whose
    // planes arrive by TMA (band.cu)
    if (tmp && gs_band_applies(op, g)) {
        for (; s + 2 <= sweeps; s += 2) {
            if (!launch_gs_sweep_band(op, g, r, x, tmp, st)) break;
            launch_gs_sweep_band(op, g, r, tmp, x, st);
        }
    }
    if (tmp && (large_planes<T>(g) || plane_tiles) && gs_tile_applies(op, g))
        for (; s + 2 <= sweeps; s += 2) {
            launch_gs_sweep_tile(op, g, r, x, tmp, st);
            launch_gs_sweep_tile(op, g, r, tmp, x, st);
        }
    for (; s < sweeps; s++) launch_gs_sweep(op, g, r, x, st);
}

template <typename T>
int gs_sweep_kind(const LevelOp<T> &op, const Geom &g, const T *x, bool has_tmp) {
    const bool plane_tiles = op.kind == OP_PLANE && g.m * g.n >= 64 * 64;
    if (has_tmp && gs_band_applies(op, g) && gs_band_ready(g, x)) return 2;
    if (has_tmp && (large_planes<T>(g) || plane_tiles) && gs_tile_applies(op, g)) return 1;
    return large_planes<T>(g) ? 0 : 3;
}

template <typename T>
void launch_gs_sweep(const LevelOp<T> &op, const Geom &g, const T *r, T *x, cudaStream_t st) {
    if (large_planes<T>(g)) {
        for (int q = 0; q < 8; q++) launch_gs_colour(op, g, q, r, x, st);
        return;
    }
    switch (op.kind) {
        case OP_CONST:
            if (op.cop.elastic) launch_phases<T, OP_CONST, true, false>(op, g, r, x, st);
            else launch_phases<T, OP_CONST, false, false>(op, g, r, x, st);
            break;
        case OP_LAME: launch_phases<T, OP_LAME, false, false>(op, g, r, x, st); break;
        case OP_PLANE:
            if (op.pop.sparse) launch_phases<T, OP_PLANE, false, true>(op, g, r, x, st);
            else launch_phases<T, OP_PLANE, false, false>(op, g, r, x, st);
            break;
        default: launch_phases<T, OP_DENSE, false, false>(op, g, r, x, st); break;
    }
}

int residual_blocks(const Geom &g) { return ((g.M2 + 31) / 32) * g.N2 * g.O2; }

template <typename T, typename R, bool NORM>
static void launch_residual_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, R *res, double *partial,
                              cudaStream_t st) {
    const dim3 blocks((g.M2 + 31) / 32, g.N2, g.O2), blk(32, 8);
    switch (op.kind) {
        case OP_CONST:
            if (op.cop.elastic)
                residual_kernel<T, R, OP_CONST, true, NORM><<<blocks, blk, 0, st>>>(g, op.cop, op.lop, op.dop, op.pop, r, x, res, partial);
            else
                residual_kernel<T, R, OP_CONST, false, NORM><<<blocks, blk, 0, st>>>(g, op.cop, op.lop, op.dop, op.pop, r, x, res, partial);
            break;
        case OP_LAME:
            residual_kernel<T, R, OP_LAME, false, NORM><<<blocks, blk, 0, st>>>(g, op.cop, op.lop, op.dop, op.pop, r, x, res, partial);
            break;
        case OP_PLANE:
            residual_kernel<T, R, OP_PLANE, false, NORM><<<blocks, blk, 0, st>>>(g, op.cop, op.lop, op.dop, op.pop, r, x, res, partial);
            break;
        default:
            residual_kernel<T, R, OP_DENSE, false, NORM><<<blocks, blk, 0, st>>>(g, op.cop, op.lop, op.dop, op.pop, r, x, res, partial);
            break;
    }
}

template <typename T, typename R>
void launch_residual(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, R *res, double *partial,
                     double *out, cudaStream_t st) {
    if constexpr (std::is_same<T, R>::value) {
        // the band kernel on the levels the band sweep serves (no norm there)
        if (res && !partial && launch_residual_band<T>(op, g, r, x, reinterpret_cast<T *>(res), st))
            return;
    }
    if (std::is_same<T, R>::value && res && residual_tile_applies(op, g)) {
        launch_residual_tile<T>(op, g, r, x, reinterpret_cast<T *>(res), partial, st);
        if (partial && out) sum_partials_kernel<<<1, 1024, 0, st>>>(partial, residual_tile_blocks(g, sizeof(T) == 8), out);
        return;
    }
    if (partial) launch_residual_k<T, R, true>(op, g, r, x, res, partial, st);
    else launch_residual_k<T, R, false>(op, g, r, x, res, partial, st);
    if (partial && out) sum_partials_kernel<<<1, 1024, 0, st>>>(partial, residual_blocks(g), out);
}

template void launch_gs_colour<float>(const LevelOp<float> &, const Geom &, int, const float *, float *, cudaStream_t);
template void launch_gs_colour<double>(const LevelOp<double> &, const Geom &, int, const double *, double *, cudaStream_t);
template int gs_sweep_kind<float>(const LevelOp<float> &, const Geom &, const float *, bool);
template int gs_sweep_kind<double>(const LevelOp<double> &, const Geom &, const double *, bool);
template void launch_gs_sweep<float>(const LevelOp<float> &, const Geom &, const float *, float *, cudaStream_t);
template void launch_gs_sweep<double>(const LevelOp<double> &, const Geom &, const double *, double *, cudaStream_t);
template void launch_gs_sweeps<float>(const LevelOp<float> &, const Geom &, const float *, float *, float *, int,
                                      cudaStream_t);
template void launch_gs_sweeps<double>(const LevelOp<double> &, const Geom &, const double *, double *, double *, int,
                                       cudaStream_t);
template void launch_residual<float, float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *, double *, double *, cudaStream_t);
template void launch_residual<double, double>(const LevelOp<double> &, const Geom &, const double *, const double *, double *, double *, double *, cudaStream_t);
template void launch_residual<double, float>(const LevelOp<double> &, const Geom &, const double *, const double *, float *, double *, double *, cudaStream_t);

}  // namespace stzmg
