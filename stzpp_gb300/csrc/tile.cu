// Tiled Gauss-Seidel sweep for large levels periodic in x and y.
//
// The 8-colour sweep (smooth.cu) updates colour q = (i&1) + 2(j&1) + 4(k&1)
// one launch at a time, and every launch streams the neighbour sub-grids of
// the whole level again.  Colours 0-3 live on even z-planes and 4-7 on odd
// ones, and a colour couples only to the other colours of its own plane and
// to the planes above and below.  This sweep therefore takes two launches,
// even planes then odd planes, and gives every CTA one TX x TY tile of one
// plane, on which it runs the plane's four colours in order from shared
// memory -- with no synchronisation between CTAs:
//
//  * the sweep reads x_in and writes x_out (a second buffer), so the old
//    values stay readable to every CTA for the whole sweep;
//  * the in-plane chain colour 0 -> 1 -> 2 -> 3 needs each colour's new
//    values one node beyond where the next colour is computed, so colour n is
//    computed on the tile widened by 3 - n nodes, from old values staged on
//    the tile widened by 4 (the halo values are recomputed by the CTAs that
//    do not own them, from the same inputs with the same arithmetic, so they
//    are bit-identical to the owner's);
//  * the planes above and below come from x_in (even launch: odd planes,
//    still old) or from x_out (odd launch: even planes, already new), and are
//    staged in shared memory next to the plane itself.
//
// Every node sees exactly the neighbour values of the colour-by-colour order
// and the arithmetic of const_row / plane_row_coef (ops.cuh), so the result
// is bit-identical to the eight colour launches.
#include <algorithm>
#include <cstdlib>

#include "launch.h"
#include "ops.cuh"

namespace stzmg {

namespace {

constexpr int kTX = 32, kTY = 32, kHalo = 4;
constexpr int kSX = kTX + 2 * kHalo, kSY = kTY + 2 * kHalo;
// Each half-row (one x-parity) is staged as the 16-byte-aligned window of
// kHW sub-grid slots starting 4 slots before the tile (the halo needs 2).
constexpr int kHW = kTX / 2 + 8, kHOff = 2;
constexpr int kTileThreads = 256;

__device__ __forceinline__ int wrapn(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Three planes (k-1, k, k+1) of the widened tile, 3 components each, every
// row split by the parity of x so that a warp working on one colour reads
// consecutive words: node ii of row jj is at [..][jj][ii & 1][(ii >> 1) + kHOff].
template <typename T>
struct TileBuf {
    T v[3][3][kSY][2][kHW];
};

// Asynchronous 16-byte global -> shared copy (cp.async, no register round
// trip): every copy of a tile is in flight at once.  Both addresses are
// 16-byte aligned (sub-grid rows and slot windows are multiples of 4 floats).
__device__ __forceinline__ void copy16_async(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void copy_wait() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Issue the copies of plane k of the widened tile (rows j0 + JLO .. j0 + JLO
// + NR - 1, slot window starting at sub-grid column w0, periodic) from x into
// buffer plane pl, in 16-byte chunks; completed by copy_wait().
template <typename T, int JLO = 0, int NR = kSY>
__device__ void stage_plane(const Geom &g, const T *__restrict__ x, int k, int w0, int j0, TileBuf<T> &B, int pl) {
    constexpr int E = 16 / sizeof(T), NC = kHW / E;   // elements per chunk, chunks per half-row
    const size_t np = (size_t)g.npad;
    const int kq = (k & 1) << 2, kofs = (k >> 1) * g.N2;
    for (int idx = threadIdx.x; idx < 3 * NR * 2 * NC; idx += kTileThreads) {
        const int cn = idx % NC, r1 = idx / NC;        // chunk fastest: consecutive sub-grid slots
        const int p = r1 & 1, r2 = r1 >> 1;
        const int jj = JLO + r2 % NR, cc = r2 / NR;
        const int j = wrapn(j0 + jj, g.n);
        const int I = wrapn(w0 + cn * E, g.M2);        // a chunk never straddles the wrap (M2 % E == 0)
        const size_t s = (size_t)(kq + ((j & 1) << 1) + p) * g.S + (size_t)(kofs + (j >> 1)) * g.M2 + I + cc * np;
        copy16_async(&B.v[pl][cc][jj][p][cn * E], x + s);
    }
}

// Phase N (colour (a, b) = (N & 1, N >> 1) of the plane): every node of that
// colour in the tile widened by 3 - N.  All parities and widths are
// compile-time, so a neighbour read is one shared load at a fixed offset from
// the node's own address.
template <typename T, int KIND, bool ELASTIC, bool SPARSE, int N>
__device__ __forceinline__ void tile_phase(const Geom &g, int c, int k, int i0, int j0, bool zin, bool has_lo,
                                           bool has_hi, const LevelOp<T> &op, const T *cf, TileBuf<T> &B,
                                           const T *__restrict__ r, T *__restrict__ xout) {
    constexpr int a = N & 1, b = N >> 1, ext = 3 - N;
    constexpr int lox = kHalo - ext + ((kHalo - ext + a) & 1), loy = kHalo - ext + ((kHalo - ext + b) & 1);
    constexpr int nx = (kHalo + kTX + ext - lox + 1) / 2, ny = (kHalo + kTY + ext - loy + 1) / 2;
    constexpr int RS = 2 * kHW;                  // words per row of one component plane
    constexpr int CS = kSY * RS;                 // words per component plane
    const size_t np = (size_t)g.npad;
    const int q = N + 4 * c, K = k >> 1;
    T *const flat = &B.v[0][0][0][0][0];
    for (int t = threadIdx.x; t < nx * ny; t += kTileThreads) {
        const int yy = t / nx, xx = t - yy * nx;
        const int ii = lox + 2 * xx, jj = loy + 2 * yy;
        const int i = wrapn(i0 + ii, g.m), j = wrapn(j0 + jj, g.n);
        const int s = q * g.S + (K * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
        T acc[3] = {r[s], r[s + np], r[s + 2 * np]};
        // plane k is the middle buffer plane: component cc of it starts at (3 + cc) * CS
        T *const self = flat + 3 * CS + jj * RS + a * kHW + (ii >> 1) + kHOff;
        // neighbour (bdx, bdy, bdz)(bb), component cc
        auto fetch = [&](int bb, int cc) -> T {
            const int dx = bdx(bb), dy = bdy(bb), dz = bdz(bb);
            return self[(dz * 3 + cc) * CS + dy * RS + (((a + dx) & 1) - a) * kHW + ((a + dx) >> 1)];
        };
        T inv[9];
        if (KIND == OP_PLANE || zin) {
            if (KIND == OP_CONST) {
                // the order and arithmetic of const_row (ops.cuh)
                T v[27][3];
#pragma unroll
                for (int bb = 0; bb < 27; bb++) {
                    if (bb == 13) continue;
                    if (ELASTIC && nnz_axes(bb) == 3) continue;
#pragma unroll
                    for (int cc = 0; cc < 3; cc++) {
                        bool used = !ELASTIC;
#pragma unroll
                        for (int rr = 0; rr < 3; rr++) used = used || elastic_entry(bb, 3 * rr + cc);
                        v[bb][cc] = used ? fetch(bb, cc) : T(0);
                    }
                }
#pragma unroll
                for (int bb = 0; bb < 27; bb++) {
                    if (bb == 13) continue;
                    if (ELASTIC && nnz_axes(bb) == 3) continue;
                    if (ELASTIC) {
#pragma unroll
                        for (int e = 0; e < 9; e++)
                            if (elastic_entry(bb, e)) acc[e / 3] -= op.cop.a[bb][e] * v[bb][e % 3];
                    } else {
                        matvec_sub(op.cop.a[bb], v[bb], acc);
                    }
                }
#pragma unroll
                for (int e = 0; e < 9; e++) inv[e] = op.cop.inv_int[e];
            } else {
                // the order and arithmetic of plane_row_coef (ops.cuh); a
                // neighbour beyond a Dirichlet z-boundary contributes nothing
#pragma unroll
                for (int bb = 0; bb < 27; bb++) {
                    if (bb == 13) continue;
                    // one block at a time: hoisting all 243 coefficient and
                    // 78 neighbour reads into registers would cost occupancy
                    asm volatile("" ::: "memory");
                    const bool out = (bdz(bb) < 0 && !has_lo) || (bdz(bb) > 0 && !has_hi);
                    T vv[3];
#pragma unroll
                    for (int cc = 0; cc < 3; cc++) vv[cc] = out ? T(0) : fetch(bb, cc);
#pragma unroll
                    for (int e = 0; e < 9; e++)
                        if (!SPARSE || coarse_entry(bb, e)) acc[e / 3] -= cf[9 * bb + e] * vv[e % 3];
                }
#pragma unroll
                for (int e = 0; e < 9; e++) inv[e] = cf[243 + e];
            }
        } else {
#pragma unroll
            for (int e = 0; e < 9; e++) inv[e] = op.cop.inv_fix[e];
        }
        const T n0 = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
        const T n1 = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
        const T n2 = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
        self[0] = n0;
        self[CS] = n1;
        self[2 * CS] = n2;
        if (ii >= kHalo && ii < kHalo + kTX && jj >= kHalo && jj < kHalo + kTY) {
            xout[s] = n0;
            xout[s + np] = n1;
            xout[s + 2 * np] = n2;
        }
    }
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
__global__ void __launch_bounds__(kTileThreads)
    gs_tile_kernel(Geom g, int c, const __grid_constant__ LevelOp<T> op, const T *__restrict__ r,
                   const T *__restrict__ xin, T *__restrict__ xout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileBuf<T> &B = *reinterpret_cast<TileBuf<T> *>(smem_raw);
    __shared__ T cf[KIND == OP_PLANE ? 252 : 1];
    const int ntx = g.m / kTX;
    const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    const int k = 2 * (int)blockIdx.y + c;
    const int i0 = tx * kTX - kHalo, j0 = ty * kTY - kHalo;   // node of [.][0][0] (unwrapped, even)
    // z-neighbour planes: old (x_in) under the even launch, new (x_out) under the odd one
    const T *__restrict__ xz = c == 0 ? xin : xout;
    const bool has_lo = g.zp || k > 0, has_hi = g.zp || k < g.o - 1;
    const bool zin = g.zp || (k != 0 && k != g.o - 1);

    if (KIND == OP_PLANE)
        for (int e = threadIdx.x; e < 252; e += kTileThreads)
            cf[e] = e < 243 ? op.pop.coef[e * op.pop.O + k] : op.pop.dinv[(e - 243) * op.pop.O + k];
    const int w0 = (i0 >> 1) - kHOff;   // first staged sub-grid column, a multiple of 4
    stage_plane(g, xin, k, w0, j0, B, 1);
    if (has_lo) stage_plane(g, xz, k == 0 ? g.o - 1 : k - 1, w0, j0, B, 0);
    if (has_hi) stage_plane(g, xz, k == g.o - 1 ? 0 : k + 1, w0, j0, B, 2);
    copy_wait();
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 0>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, B, r, xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 1>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, B, r, xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 2>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, B, r, xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 3>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, B, r, xout);
}

// res = r - A x on one 32x32 tile of plane k (all 4 colours of the plane),
// from the same staged planes; every node's arithmetic is that of the
// residual kernel (const_row / plane_row_coef with the centre block, ops.cuh).
// With NORM each CTA writes the FP64 sum of |res|^2 over its tile to
// partial[CTA index].
template <typename T, int KIND, bool ELASTIC, bool SPARSE, bool NORM>
__global__ void __launch_bounds__(kTileThreads)
    residual_tile_kernel(Geom g, const __grid_constant__ LevelOp<T> op, const T *__restrict__ r,
                         const T *__restrict__ x, T *__restrict__ res, double *__restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileBuf<T> &B = *reinterpret_cast<TileBuf<T> *>(smem_raw);
    __shared__ T cf[KIND == OP_PLANE ? 252 : 1];
    const int ntx = g.m / kTX;
    const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    const int k = (int)blockIdx.y;
    const int i0 = tx * kTX - kHalo, j0 = ty * kTY - kHalo;
    const bool has_lo = g.zp || k > 0, has_hi = g.zp || k < g.o - 1;
    const bool zin = g.zp || (k != 0 && k != g.o - 1);
    if (KIND == OP_PLANE)
        for (int e = threadIdx.x; e < 252; e += kTileThreads)
            cf[e] = e < 243 ? op.pop.coef[e * op.pop.O + k] : op.pop.dinv[(e - 243) * op.pop.O + k];
    // only the rows one beyond the tile are read
    const int w0 = (i0 >> 1) - kHOff;
    constexpr int JLO = kHalo - 1, NR = kTY + 2;
    stage_plane<T, JLO, NR>(g, x, k, w0, j0, B, 1);
    if (has_lo && (KIND == OP_PLANE || zin))
        stage_plane<T, JLO, NR>(g, x, k == 0 ? g.o - 1 : k - 1, w0, j0, B, 0);
    if (has_hi && (KIND == OP_PLANE || zin))
        stage_plane<T, JLO, NR>(g, x, k == g.o - 1 ? 0 : k + 1, w0, j0, B, 2);
    copy_wait();
    __syncthreads();
    constexpr int RS = 2 * kHW, CS = kSY * RS;
    const size_t np = (size_t)g.npad;
    const int c = k & 1, K = k >> 1;
    T *const flat = &B.v[0][0][0][0][0];
    double sq = 0.0;
    // A warp takes the 16 nodes of one x-parity a in two adjacent rows (row
    // stride 2 kHW words: the two half-warps fall on disjoint shared-memory
    // banks in FP32); colour (a, b) with b the row parity.
    for (int t = threadIdx.x; t < kTX * kTY; t += kTileThreads) {
        const int xs = t & 15, b = (t >> 4) & 1, a = (t >> 5) & 1, pr = t >> 6;
        const int ii = kHalo + a + 2 * xs, jj = kHalo + b + 2 * pr;
        const int i = wrapn(i0 + ii, g.m), j = wrapn(j0 + jj, g.n);
        const int q = a + 2 * b + 4 * c;
        const int s = q * g.S + (K * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
        T acc[3] = {r[s], r[s + np], r[s + 2 * np]};
        const T *self = flat + 3 * CS + jj * RS + a * kHW + (ii >> 1) + kHOff;
        auto fetch = [&](int bb, int cc) -> T {
            const int dx = bdx(bb), dy = bdy(bb), dz = bdz(bb);
            return self[(dz * 3 + cc) * CS + dy * RS + (((a + dx) & 1) - a) * kHW + ((a + dx) >> 1)];
        };
        if (KIND == OP_CONST) {
            if (zin) {
                // const_row<T, ELASTIC, true>
                T v[27][3];
#pragma unroll
                for (int bb = 0; bb < 27; bb++) {
                    if (ELASTIC && nnz_axes(bb) == 3) continue;
#pragma unroll
                    for (int cc = 0; cc < 3; cc++) {
                        bool used = !ELASTIC || bb == 13;
#pragma unroll
                        for (int rr = 0; rr < 3; rr++) used = used || elastic_entry(bb, 3 * rr + cc);
                        v[bb][cc] = used ? fetch(bb, cc) : T(0);
                    }
                }
#pragma unroll
                for (int bb = 0; bb < 27; bb++) {
                    if (ELASTIC && nnz_axes(bb) == 3) continue;
                    if (ELASTIC && bb != 13) {
#pragma unroll
                        for (int e = 0; e < 9; e++)
                            if (elastic_entry(bb, e)) acc[e / 3] -= op.cop.a[bb][e] * v[bb][e % 3];
                    } else if (bb == 13 && op.cop.centre_diag) {
                        acc[0] -= op.cop.a[13][0] * v[13][0];
                        acc[1] -= op.cop.a[13][4] * v[13][1];
                        acc[2] -= op.cop.a[13][8] * v[13][2];
                    } else {
                        matvec_sub(op.cop.a[bb], v[bb], acc);
                    }
                }
            } else {
                T v[3] = {self[0], self[CS], self[2 * CS]};
                matvec_sub(op.cop.fix, v, acc);
            }
        } else {
            // plane_row_coef<T, SPARSE, true>: all 27 blocks, none beyond a Dirichlet z-boundary
#pragma unroll
            for (int bb = 0; bb < 27; bb++) {
                asm volatile("" ::: "memory");
                const bool out = (bdz(bb) < 0 && !has_lo) || (bdz(bb) > 0 && !has_hi);
                T vv[3];
#pragma unroll
                for (int cc = 0; cc < 3; cc++) vv[cc] = out ? T(0) : fetch(bb, cc);
#pragma unroll
                for (int e = 0; e < 9; e++)
                    if (!SPARSE || coarse_entry(bb, e)) acc[e / 3] -= cf[9 * bb + e] * vv[e % 3];
            }
        }
        res[s] = acc[0];
        res[s + np] = acc[1];
        res[s + 2 * np] = acc[2];
        if (NORM) sq += (double)acc[0] * (double)acc[0] + (double)acc[1] * (double)acc[1] + (double)acc[2] * (double)acc[2];
    }
    if (NORM) {
        __shared__ double red[kTileThreads / 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
        __syncthreads();
        if (threadIdx.x < 32) {
            sq = threadIdx.x < kTileThreads / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
            if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = sq;
        }
    }
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
void launch_tile_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    const int tiles = (g.m / kTX) * (g.n / kTY);
    auto kern = gs_tile_kernel<T, KIND, ELASTIC, SPARSE>;
    const int smem = (int)sizeof(TileBuf<T>);
    static bool attr_set = false;   // per instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set = true;
    }
    for (int c = 0; c < 2; c++) {
        const int planes = c == 0 ? (g.o + 1) / 2 : g.o / 2;
        if (planes > 0) kern<<<dim3(tiles, planes), kTileThreads, smem, st>>>(g, c, op, r, xin, xout);
    }
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
void launch_res_tile_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, double *partial,
                       cudaStream_t st) {
    const int smem = (int)sizeof(TileBuf<T>);
    const dim3 grid((g.m / kTX) * (g.n / kTY), g.o);
    static bool attr_set = false;   // per instantiation
    if (!attr_set) {
        cudaFuncSetAttribute(residual_tile_kernel<T, KIND, ELASTIC, SPARSE, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(residual_tile_kernel<T, KIND, ELASTIC, SPARSE, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set = true;
    }
    if (partial)
        residual_tile_kernel<T, KIND, ELASTIC, SPARSE, true><<<grid, kTileThreads, smem, st>>>(g, op, r, x, res, partial);
    else
        residual_tile_kernel<T, KIND, ELASTIC, SPARSE, false><<<grid, kTileThreads, smem, st>>>(g, op, r, x, res, partial);
}

}  // namespace

// Where the tiled sweep runs.  Measured on a GB300 (two sweeps, 256x256x257
// problem): on the FP32 plane-invariant coarse levels it beats the colour
// launches (level 1: 221 vs 245 us); on the fine shared-stencil level (800 vs
// 653 us) and in FP64 (one CTA per SM for lack of shared memory) it loses, so
// by default it runs on FP32 plane-invariant levels only.  STZ_MG_TILE=0
// disables it, STZ_MG_TILE=1 uses it wherever it applies.
template <typename T>
bool gs_tile_applies(const LevelOp<T> &op, const Geom &g) {
    int mode = -1;
    if (const char *e = std::getenv("STZ_MG_TILE")) mode = std::atoi(e) != 0;
    if (mode == 0) return false;
    if (op.kind != OP_CONST && op.kind != OP_PLANE) return false;
    if (mode < 0 && (sizeof(T) != 4 || op.kind != OP_PLANE)) return false;
    // whole tiles of a level periodic in x and y; an odd periodic z would put
    // both parities of a colour on one plane
    return g.xp && g.yp && g.m % kTX == 0 && g.n % kTY == 0 && !(g.zp && (g.o & 1));
}

template <typename T>
void launch_gs_sweep_tile(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    if (op.kind == OP_CONST) {
        if (op.cop.elastic) launch_tile_k<T, OP_CONST, true, false>(op, g, r, xin, xout, st);
        else launch_tile_k<T, OP_CONST, false, false>(op, g, r, xin, xout, st);
    } else {
        if (op.pop.sparse) launch_tile_k<T, OP_PLANE, false, true>(op, g, r, xin, xout, st);
        else launch_tile_k<T, OP_PLANE, false, false>(op, g, r, xin, xout, st);
    }
}

// Where the tiled residual runs.  Measured on a GB300 (256x256x257 problem,
// FP32): on the plane-invariant level 1 it beats the colour-interleaved
// residual kernel 63.6 vs 165.5 us (that kernel re-reads the plane's 252
// coefficients per node from global memory); on the fine shared-stencil level
// it loses (251.5 vs 223.2 us), so by default it runs on FP32 plane-invariant
// levels of at least 64x64 nodes per plane.  STZ_MG_TILE=0 disables it,
// STZ_MG_TILE=1 uses it wherever it applies, FP64 included.
template <typename T>
bool residual_tile_applies(const LevelOp<T> &op, const Geom &g) {
    int mode = -1;
    if (const char *e = std::getenv("STZ_MG_TILE")) mode = std::atoi(e) != 0;
    if (mode == 0) return false;
    if (op.kind != OP_CONST && op.kind != OP_PLANE) return false;
    if (mode < 0 && (sizeof(T) != 4 || op.kind != OP_PLANE)) return false;
    return g.xp && g.yp && g.m % kTX == 0 && g.n % kTY == 0 && g.m * g.n >= 64 * 64;
}

int residual_tile_blocks(const Geom &g) { return (g.m / kTX) * (g.n / kTY) * g.o; }

template <typename T>
void launch_residual_tile(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, double *partial,
                          cudaStream_t st) {
    if (op.kind == OP_CONST) {
        if (op.cop.elastic) launch_res_tile_k<T, OP_CONST, true, false>(op, g, r, x, res, partial, st);
        else launch_res_tile_k<T, OP_CONST, false, false>(op, g, r, x, res, partial, st);
    } else {
        if (op.pop.sparse) launch_res_tile_k<T, OP_PLANE, false, true>(op, g, r, x, res, partial, st);
        else launch_res_tile_k<T, OP_PLANE, false, false>(op, g, r, x, res, partial, st);
    }
}

template bool residual_tile_applies<float>(const LevelOp<float> &, const Geom &);
template bool residual_tile_applies<double>(const LevelOp<double> &, const Geom &);
template void launch_residual_tile<float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *,
                                          double *, cudaStream_t);
template void launch_residual_tile<double>(const LevelOp<double> &, const Geom &, const double *, const double *,
                                           double *, double *, cudaStream_t);
template bool gs_tile_applies<float>(const LevelOp<float> &, const Geom &);
template bool gs_tile_applies<double>(const LevelOp<double> &, const Geom &);
template void launch_gs_sweep_tile<float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *,
                                          cudaStream_t);
template void launch_gs_sweep_tile<double>(const LevelOp<double> &, const Geom &, const double *, const double *,
                                           double *, cudaStream_t);

}  // namespace stzmg
