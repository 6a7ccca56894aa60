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
#include <type_traits>

#include "launch.h"
#include "ops.cuh"
#include "transfer.cuh"

namespace stzmg {

namespace {

constexpr int kTX = 32, kTY = 32, kHalo = 4;
constexpr int kSY = kTY + 2 * kHalo;
// Each half-row (one x-parity) is staged as the 16-byte-aligned window of
// kHW sub-grid slots starting 4 slots before the tile (the halo needs 2).
constexpr int kHW = kTX / 2 + 8, kHOff = 2;
constexpr int kTileThreads = 256;
// CTAs per SM the shared memory allows (3 in FP32, 1 in FP64): lets ptxas
// give each thread the registers those CTAs leave, for more loads in flight.
template <typename T>
constexpr int kTileMinBlocks = sizeof(T) == 4 ? 3 : 1;
// Threads of the tiled sweep: every phase (at most 19 x 19 nodes) in one round.
constexpr int kGsThreads = 384;
constexpr int RS = 2 * kHW;   // words per row (both x-parities) of one component plane

__device__ __forceinline__ int wrapn(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Three planes (k-1, k, k+1) of the widened tile, 3 components each, every
// component plane split by the parity of x so that a warp working on one
// colour reads consecutive words: node ii of row jj is at
// [..][ii & 1][jj][(ii >> 1) + kHOff].  Rows of one parity are kHW = 24 words
// apart, so two rows of one colour (2 kHW apart) fall on banks 16 apart.
template <typename T>
struct TileBuf {
    T v[3][3][2][kSY][kHW];
};

// Rows of one buffer component plane: the sweep stages rows 0 .. kSY - 1 of
// the widened tile, the residual rows kHalo - 1 .. kHalo + kTY (one beyond
// the tile) into buffer rows 0 .. kRowsRes - 1.
constexpr int kRowsRes = kTY + 2, kRes0 = kHalo - 1;

// A node's neighbours in one buffer plane are read relative to its "corner"
// word there: row jj - 1, slot (ii >> 1) + kHOff - 1 of the x-parity-0
// half-plane.  Neighbour (bdx, bdy)(b), component c, of a node of x-parity A is
// then at this non-negative compile-time word offset, in a buffer plane of
// NROWS rows per component (the node itself: b = 13, in its own plane).
template <int A, int NROWS>
__host__ __device__ constexpr int nb_off(int b, int c) {
    return c * NROWS * RS + ((A + bdx(b) + 2) & 1) * NROWS * kHW + (bdy(b) + 1) * kHW + ((A + bdx(b) + 2) >> 1);
}

// Corner word of node (ii, jj) in a buffer plane whose row 0 is tile row ROW0.
template <int ROW0>
__device__ __forceinline__ int corner_word(int ii, int jj) {
    return (jj - 1 - ROW0) * kHW + (ii >> 1) + kHOff - 1;
}

// Shared-memory load / store at a compile-time byte offset from a 32-bit
// shared address: one instruction per access, no per-access address arithmetic.
template <int OFF>
__device__ __forceinline__ void lds(unsigned a, float &v) {
    asm volatile("ld.shared.f32 %0, [%1+%2];" : "=f"(v) : "r"(a), "n"(OFF * 4));
}
template <int OFF>
__device__ __forceinline__ void lds(unsigned a, double &v) {
    asm volatile("ld.shared.f64 %0, [%1+%2];" : "=d"(v) : "r"(a), "n"(OFF * 8));
}
template <int OFF>
__device__ __forceinline__ void sts(unsigned a, float v) {
    asm volatile("st.shared.f32 [%0+%1], %2;" ::"r"(a), "n"(OFF * 4), "f"(v) : "memory");
}
template <int OFF>
__device__ __forceinline__ void sts(unsigned a, double v) {
    asm volatile("st.shared.f64 [%0+%1], %2;" ::"r"(a), "n"(OFF * 8), "d"(v) : "memory");
}

// Compile-time loop: f(std::integral_constant<int, I>) for I = B .. E - 1.
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// Asynchronous 16-byte global -> shared copy (cp.async, no register round
// trip): every copy of a tile is in flight at once.  Both addresses are
// 16-byte aligned (sub-grid rows and slot windows are multiples of 16 bytes).
__device__ __forceinline__ void copy16_async(unsigned d, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void copy_wait() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// The 16-byte copies that stage one plane of the widened tile (rows JLO ..
// JLO + NR - 1, the kHW-slot window from sub-grid column w0 of each half-row,
// periodic in x and y) into a buffer plane of NROWS rows per component whose
// row 0 is tile row ROW0.  Each thread works out its share once per CTA: the
// chunk's place in a buffer component plane and its offset inside a plane of
// one colour sub-grid, which is the same for every plane and component.
template <typename T, int JLO, int NR, int ROW0, int NROWS, int NT = kTileThreads>
struct Stager {
    static constexpr int E = 16 / sizeof(T), NC = kHW / E, NCH = NR * 2 * NC;
    static constexpr int ND = (NCH + NT - 1) / NT;
    unsigned soff[ND];   // bytes from the start of a buffer component plane
    int goff[ND];        // elements from the plane's start in colour sub-grid 0 (-1: none)

    __device__ __forceinline__ void init(const Geom &g, int w0, int j0) {
#pragma unroll
        for (int d = 0; d < ND; d++) {
            const int idx = (int)threadIdx.x + d * NT;
            goff[d] = -1;
            soff[d] = 0;
            if (idx < NCH) {
                const int cn = idx % NC, r1 = idx / NC;   // chunk fastest: consecutive sub-grid slots
                const int p = r1 & 1, jj = JLO + (r1 >> 1);
                const int j = wrapn(j0 + jj, g.n);
                const int I = wrapn(w0 + cn * E, g.M2);    // a chunk never straddles the wrap (M2 % E == 0)
                goff[d] = (((j & 1) << 1) + p) * g.S + (j >> 1) * g.M2 + I;
                soff[d] = (unsigned)(((p * NROWS + jj - ROW0) * kHW + cn * E) * (int)sizeof(T));
            }
        }
    }

    // Issue the copies of plane k of x into the buffer plane at shared byte
    // address dk; completed by a cp.async wait.
    __device__ __forceinline__ void stage(const Geom &g, const T *__restrict__ x, int k, unsigned dk) const {
        const T *xk = x + (size_t)((k & 1) << 2) * g.S + (size_t)(k >> 1) * g.N2 * g.M2;
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
            const T *xc = xk + (size_t)cc * g.npad;
            const unsigned dc = dk + (unsigned)(cc * NROWS * RS * (int)sizeof(T));
#pragma unroll
            for (int d = 0; d < ND; d++)
                if (goff[d] >= 0) copy16_async(dc + soff[d], xc + goff[d]);
        }
    }
};

// acc -= sum_b A_b x_b of the shared stencil in the order and arithmetic of
// const_row (ops.cuh): neighbour components first (those the stencil uses),
// then the products.  WITH_CENTRE: include the centre block (residual).
template <typename T, bool ELASTIC, bool WITH_CENTRE, int A, int NROWS>
__device__ __forceinline__ void tile_const_row(const ConstOp<T> &op, const unsigned (&cz)[3], T *acc) {
    if constexpr (!ELASTIC) {
        // a full-block stencil: each block's three values right before its
        // products (the same products in the same order; 81 values at once
        // would spill)
        static_for<0, 27>([&](auto bi) {
            constexpr int b = decltype(bi)::value;
            if constexpr (b != 13 || WITH_CENTRE) {
                asm volatile("" ::: "memory");
                T v[3];
                lds<nb_off<A, NROWS>(b, 0)>(cz[bdz(b) + 1], v[0]);
                lds<nb_off<A, NROWS>(b, 1)>(cz[bdz(b) + 1], v[1]);
                lds<nb_off<A, NROWS>(b, 2)>(cz[bdz(b) + 1], v[2]);
                if (b == 13 && op.centre_diag) {
                    acc[0] -= op.a[13][0] * v[0];
                    acc[1] -= op.a[13][4] * v[1];
                    acc[2] -= op.a[13][8] * v[2];
                } else {
                    matvec_sub(op.a[b], v, acc);
                }
            }
        });
        return;
    }
    T v[27][3];
    static_for<0, 27>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        if constexpr ((b != 13 || WITH_CENTRE) && !(ELASTIC && nnz_axes(b) == 3)) {
            static_for<0, 3>([&](auto ci) {
                constexpr int c = decltype(ci)::value;
                constexpr bool used = !ELASTIC || b == 13 || elastic_entry(b, c) || elastic_entry(b, 3 + c) ||
                                      elastic_entry(b, 6 + c);
                if constexpr (used) lds<nb_off<A, NROWS>(b, c)>(cz[bdz(b) + 1], v[b][c]);
                else v[b][c] = T(0);
            });
        }
    });
#pragma unroll
    for (int b = 0; b < 27; b++) {
        if (b == 13 && !WITH_CENTRE) continue;
        if (ELASTIC && nnz_axes(b) == 3) continue;
        if (ELASTIC && b != 13) {
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (elastic_entry(b, e)) acc[e / 3] -= op.a[b][e] * v[b][e % 3];
        } else if (b == 13 && op.centre_diag) {
            acc[0] -= op.a[13][0] * v[13][0];
            acc[1] -= op.a[13][4] * v[13][1];
            acc[2] -= op.a[13][8] * v[13][2];
        } else {
            matvec_sub(op.a[b], v[b], acc);
        }
    }
}

// acc -= sum_b A_b x_b with block b's entries in cf[9b ..] (shared memory):
// the order and arithmetic of plane_row_coef (ops.cuh); a neighbour beyond a
// Dirichlet z-boundary contributes nothing.  One block at a time: hoisting
// all 243 coefficient and 78 neighbour reads into registers would cost
// occupancy.
template <typename T, bool SPARSE, bool WITH_CENTRE, int A, int NROWS>
__device__ __forceinline__ void tile_plane_row(const T *cf, const unsigned (&cz)[3], bool has_lo, bool has_hi,
                                               T *acc) {
    static_for<0, 27>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        if constexpr (b != 13 || WITH_CENTRE) {
            asm volatile("" ::: "memory");
            const bool out = (bdz(b) < 0 && !has_lo) || (bdz(b) > 0 && !has_hi);
            T vv[3];
            lds<nb_off<A, NROWS>(b, 0)>(cz[bdz(b) + 1], vv[0]);
            lds<nb_off<A, NROWS>(b, 1)>(cz[bdz(b) + 1], vv[1]);
            lds<nb_off<A, NROWS>(b, 2)>(cz[bdz(b) + 1], vv[2]);
            if (out) vv[0] = vv[1] = vv[2] = T(0);
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (!SPARSE || coarse_entry(b, e)) acc[e / 3] -= cf[9 * b + e] * vv[e % 3];
        }
    });
}

// Phase N updates colour (a, b) = (N & 1, N >> 1) of the plane on the tile
// widened by 3 - N: nx x ny nodes, at most one per thread.  This thread's
// node (if any): its tile coordinates (ii, jj) and sub-grid slot s.
template <int N>
struct Phase {
    static constexpr int a = N & 1, b = N >> 1, ext = 3 - N;
    static constexpr int lox = kHalo - ext + ((kHalo - ext + a) & 1), loy = kHalo - ext + ((kHalo - ext + b) & 1);
    static constexpr int nx = (kHalo + kTX + ext - lox + 1) / 2, ny = (kHalo + kTY + ext - loy + 1) / 2;
    static_assert(nx * ny <= kGsThreads, "one node per thread");

    __device__ __forceinline__ static bool node(const Geom &g, int c, int k, int i0, int j0, int &ii, int &jj,
                                                int &s) {
        const int t = (int)threadIdx.x;
        if (t >= nx * ny) return false;
        const int yy = t / nx, xx = t - yy * nx;
        ii = lox + 2 * xx;
        jj = loy + 2 * yy;
        const int i = wrapn(i0 + ii, g.m), j = wrapn(j0 + jj, g.n);
        s = (N + 4 * c) * g.S + ((k >> 1) * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
        return true;
    }
};

// Phase N: every node of its colour in the widened tile, with r of this
// thread's nodes already in registers (rr).  All parities and widths are
// compile-time, so a neighbour read is one shared load at a fixed offset from
// the node's corner address.
template <typename T, int KIND, bool ELASTIC, bool SPARSE, int N>
__device__ __forceinline__ void tile_phase(const Geom &g, int c, int k, int i0, int j0, bool zin, bool has_lo,
                                           bool has_hi, const LevelOp<T> &op, const T *cf, unsigned sbase,
                                           const T (&rr)[3], T *__restrict__ xout) {
    constexpr int a = Phase<N>::a;
    const size_t np = (size_t)g.npad;
    int ii, jj, s;
    if (Phase<N>::node(g, c, k, i0, j0, ii, jj, s)) {
        T acc[3] = {rr[0], rr[1], rr[2]};
        constexpr unsigned PB = 3 * kSY * RS * sizeof(T);   // bytes per buffer plane
        const unsigned c1 = sbase + (unsigned)(corner_word<0>(ii, jj) * (int)sizeof(T));
        const unsigned cz[3] = {c1, c1 + PB, c1 + 2 * PB};
        T inv[9];
        if (KIND == OP_PLANE || zin) {
            if (KIND == OP_CONST) {
                tile_const_row<T, ELASTIC, false, a, kSY>(op.cop, cz, acc);
#pragma unroll
                for (int e = 0; e < 9; e++) inv[e] = op.cop.inv_int[e];
            } else {
                tile_plane_row<T, SPARSE, false, a, kSY>(cf, cz, has_lo, has_hi, acc);
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
        sts<nb_off<a, kSY>(13, 0)>(cz[1], n0);
        sts<nb_off<a, kSY>(13, 1)>(cz[1], n1);
        sts<nb_off<a, kSY>(13, 2)>(cz[1], n2);
        if (ii >= kHalo && ii < kHalo + kTX && jj >= kHalo && jj < kHalo + kTY) {
            xout[s] = n0;
            xout[s + np] = n1;
            xout[s + 2 * np] = n2;
        }
    }
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
__global__ void __launch_bounds__(kGsThreads, kTileMinBlocks<T>)
    gs_tile_kernel(Geom g, int c, const __grid_constant__ LevelOp<T> op, const T *__restrict__ r,
                   const T *__restrict__ xin, T *__restrict__ xout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
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
        for (int e = threadIdx.x; e < 252; e += kGsThreads)
            cf[e] = e < 243 ? op.pop.coef[e * op.pop.O + k] : op.pop.dinv[(e - 243) * op.pop.O + k];
    constexpr unsigned PB = 3 * kSY * RS * sizeof(T);   // bytes per buffer plane
    Stager<T, 0, kSY, 0, kSY, kGsThreads> st;
    st.init(g, (i0 >> 1) - kHOff, j0);   // first staged sub-grid column: a multiple of 4
    st.stage(g, xin, k, sbase + PB);
    if (has_lo) st.stage(g, xz, k == 0 ? g.o - 1 : k - 1, sbase);
    if (has_hi) st.stage(g, xz, k == g.o - 1 ? 0 : k + 1, sbase + 2 * PB);
    // r of every node this thread updates, loaded while the copies are in flight
    const size_t np = (size_t)g.npad;
    T rr[4][3];
    static_for<0, 4>([&](auto ni) {
        constexpr int N = decltype(ni)::value;
        int ii, jj, s;
        if (Phase<N>::node(g, c, k, i0, j0, ii, jj, s)) {
            rr[N][0] = r[s];
            rr[N][1] = r[s + np];
            rr[N][2] = r[s + 2 * np];
        }
    });
    copy_wait();
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 0>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, sbase, rr[0], xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 1>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, sbase, rr[1], xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 2>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, sbase, rr[2], xout);
    __syncthreads();
    tile_phase<T, KIND, ELASTIC, SPARSE, 3>(g, c, k, i0, j0, zin, has_lo, has_hi, op, cf, sbase, rr[3], xout);
}

// res = r - A x at one node of x-parity A (the arithmetic of the residual
// kernel: const_row / plane_row_coef with the centre block, ops.cuh).
template <typename T, int KIND, bool ELASTIC, bool SPARSE, int A>
__device__ __forceinline__ void res_node(const LevelOp<T> &op, const T *cf, const unsigned (&cz)[3], bool zin,
                                         bool has_lo, bool has_hi, T *acc) {
    if (KIND == OP_CONST) {
        if (zin) {
            tile_const_row<T, ELASTIC, true, A, kRowsRes>(op.cop, cz, acc);
        } else {
            T v[3];
            lds<nb_off<A, kRowsRes>(13, 0)>(cz[1], v[0]);
            lds<nb_off<A, kRowsRes>(13, 1)>(cz[1], v[1]);
            lds<nb_off<A, kRowsRes>(13, 2)>(cz[1], v[2]);
            matvec_sub(op.cop.fix, v, acc);
        }
    } else {
        tile_plane_row<T, SPARSE, true, A, kRowsRes>(cf, cz, has_lo, has_hi, acc);
    }
}

template <int N>
__device__ __forceinline__ void copy_wait_but() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void copy_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

// Ring slots of the marching residual: planes k-1, k, k+1 in use and k+2 in
// flight; r of planes k and k+1 in a second ring after them.
constexpr int kRing = 4;
constexpr int kRingSlot = 3 * kRowsRes * RS;   // words per slot
// r of one plane of the tile: per component and colour 16 rows of 16 slots,
// colours kRColour words apart (16 mod 32: the two half-warps of a warp, two
// colours apart, fall on disjoint banks in FP32)
constexpr int kRColour = 16 * 16 + 8;
constexpr int kRSlot = 3 * 4 * kRColour;
constexpr int kMarchSmemWords = kRing * kRingSlot + 2 * kRSlot;

// Issue the copies of r of plane k of tile (tx, ty) into the r slot at shared
// byte address d: 3 components x 4 colours x 16 rows x 4 chunks of 16 bytes.
template <typename T>
__device__ __forceinline__ void stage_r(const Geom &g, const T *__restrict__ r, int k, int tx, int ty, unsigned d) {
    constexpr int E = 16 / sizeof(T), CPR = 16 / E;   // elements per chunk, chunks per row
    for (int idx = threadIdx.x; idx < 3 * 4 * 16 * CPR; idx += kTileThreads) {
        const int ch = idx % CPR, row = (idx / CPR) % 16, n = (idx / (CPR * 16)) % 4, cc = idx / (CPR * 64);
        const size_t gs = (size_t)cc * g.npad + (size_t)(n + 4 * (k & 1)) * g.S +
                          (size_t)((k >> 1) * g.N2 + ty * 16 + row) * g.M2 + tx * 16 + ch * E;
        copy16_async(d + (unsigned)(((cc * 4 + n) * kRColour + row * 16 + ch * E) * (int)sizeof(T)), r + gs);
    }
}
template <typename T>
constexpr int kMarchMinBlocks = sizeof(T) == 4 ? 2 : 1;

// res = r - A x on one 32x32 tile column, planes k0 .. k0 + zlen - 1: the CTA
// marches up z with the planes in a ring of shared-memory slots, and the
// copies of plane k + 2 are in flight while plane k is computed.  With NORM
// each CTA writes the FP64 sum of |res|^2 over its nodes to
// partial[CTA index].
template <typename T, int KIND, bool ELASTIC, bool SPARSE, bool NORM>
__global__ void __launch_bounds__(kTileThreads, kMarchMinBlocks<T>)
    residual_tile_kernel(Geom g, const __grid_constant__ LevelOp<T> op, const T *__restrict__ r,
                         const T *__restrict__ x, T *__restrict__ res, double *__restrict__ partial, int zlen) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    __shared__ T cf[KIND == OP_PLANE ? 252 : 1];
    const int ntx = g.m / kTX;
    const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    const int k0 = (int)blockIdx.y * zlen, k1 = min(g.o, k0 + zlen);
    const int i0 = tx * kTX - kHalo, j0 = ty * kTY - kHalo;
    const size_t np = (size_t)g.npad;
    // plane kk (k0 - 1 <= kk <= k1) exists, its index, its slot
    auto exists = [&](int kk) { return g.zp || (kk >= 0 && kk < g.o); };
    auto wrapk = [&](int kk) { return kk < 0 ? kk + g.o : (kk >= g.o ? kk - g.o : kk); };
    auto slot = [&](int kk) { return sbase + (unsigned)(((kk + kRing) % kRing) * kRingSlot * (int)sizeof(T)); };

    auto rslot = [&](int kk) { return sbase + (unsigned)((kRing * kRingSlot + (kk & 1) * kRSlot) * (int)sizeof(T)); };

    // cp.async groups: {x of k0-1, k0, k0+1; r of k0}, {x of k0+2; r of k0+1},
    // then one per plane k: {x of k+3; r of k+2}
    Stager<T, kRes0, kRowsRes, kRes0, kRowsRes> st;
    st.init(g, (i0 >> 1) - kHOff, j0);
    for (int kk = k0 - 1; kk <= k0 + 1; kk++)
        if (kk <= k1 && exists(kk)) st.stage(g, x, wrapk(kk), slot(kk));
    stage_r(g, r, k0, tx, ty, rslot(k0));
    copy_commit();
    if (k0 + 2 <= k1 && exists(k0 + 2)) st.stage(g, x, wrapk(k0 + 2), slot(k0 + 2));
    if (k0 + 1 < k1) stage_r(g, r, k0 + 1, tx, ty, rslot(k0 + 1));
    copy_commit();

    // This thread's nodes: colour (a, b) and column xs are the same in every
    // plane; rows jj = kHalo + b + 2 R with R = h + 2 q2 + 4 it, it = 0 .. 3.
    // A warp takes 16 nodes of one colour in each of two rows 2 apart (2 kHW
    // words: the two half-warps fall on disjoint shared-memory banks in FP32).
    const int xs = threadIdx.x & 15, h = (threadIdx.x >> 4) & 1, a = (threadIdx.x >> 5) & 1;
    const int b = (threadIdx.x >> 6) & 1, pr0 = h + 2 * (threadIdx.x >> 7);
    const int ii = kHalo + a + 2 * xs, i = wrapn(i0 + ii, g.m);
    constexpr int NIT = kTX * kTY / kTileThreads;
    static_assert(kTileThreads == 256 && NIT == 4, "node mapping");
    double sq = 0.0;
    for (int k = k0; k < k1; k++) {
        if (KIND == OP_PLANE)
            for (int e = threadIdx.x; e < 252; e += kTileThreads)
                cf[e] = e < 243 ? op.pop.coef[e * op.pop.O + k] : op.pop.dinv[(e - 243) * op.pop.O + k];
        copy_wait_but<1>();   // every group but the newest ({x of k+2; r of k+1}) has landed
        __syncthreads();
        const bool has_lo = g.zp || k > 0, has_hi = g.zp || k < g.o - 1;
        const bool zin = g.zp || (k != 0 && k != g.o - 1);
        const unsigned rs = rslot(k) + (unsigned)(((a + 2 * b) * kRColour + xs) * (int)sizeof(T));
        const unsigned s0 = slot(k - 1), s1 = slot(k), s2 = slot(k + 1);
        auto node = [&](int it) {
            const int jj = kHalo + b + 2 * (pr0 + 4 * it);   // row R = pr0 + 4 it
            const int j = wrapn(j0 + jj, g.n);
            const int s = (a + 2 * b + 4 * (k & 1)) * g.S + ((k >> 1) * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
            T acc[3];
            const unsigned ra = rs + (unsigned)((pr0 + 4 * it) * 16 * (int)sizeof(T));
            lds<0>(ra, acc[0]);
            lds<4 * kRColour>(ra, acc[1]);
            lds<8 * kRColour>(ra, acc[2]);
            const unsigned cw = (unsigned)(corner_word<kRes0>(ii, jj) * (int)sizeof(T));
            const unsigned cz[3] = {s0 + cw, s1 + cw, s2 + cw};
            if (a == 0) res_node<T, KIND, ELASTIC, SPARSE, 0>(op, cf, cz, zin, has_lo, has_hi, acc);   // warp-uniform
            else res_node<T, KIND, ELASTIC, SPARSE, 1>(op, cf, cz, zin, has_lo, has_hi, acc);
            res[s] = acc[0];
            res[s + np] = acc[1];
            res[s + 2 * np] = acc[2];
            if (NORM)
                sq += (double)acc[0] * (double)acc[0] + (double)acc[1] * (double)acc[1] + (double)acc[2] * (double)acc[2];
        };
        if constexpr (KIND == OP_CONST && ELASTIC) {
#pragma unroll
            for (int it = 0; it < NIT; it++) node(it);
        } else {
            // a full-block row is long: unrolling the four nodes would spill
#pragma unroll 1
            for (int it = 0; it < NIT; it++) node(it);
        }
        __syncthreads();   // x slot of plane k - 1, r slot of plane k (and cf) free
        if (k + 3 <= k1 && exists(k + 3)) st.stage(g, x, wrapk(k + 3), slot(k + 3));
        if (k + 2 < k1) stage_r(g, r, k + 2, tx, ty, rslot(k + 2));
        copy_commit();
    }
    copy_wait_but<0>();
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

// The shared-memory attribute of a kernel is set per device: true the first
// time this is asked on the current device (setting it twice is harmless).
bool first_use_on_device(unsigned long long &devices) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (devices & bit) return false;
    devices |= bit;
    return true;
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
void launch_tile_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    const int tiles = (g.m / kTX) * (g.n / kTY);
    auto kern = gs_tile_kernel<T, KIND, ELASTIC, SPARSE>;
    const int smem = (int)sizeof(TileBuf<T>);
    static unsigned long long attr_devices = 0;   // per instantiation
    if (first_use_on_device(attr_devices))
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    for (int c = 0; c < 2; c++) {
        const int planes = c == 0 ? (g.o + 1) / 2 : g.o / 2;
        if (planes > 0) kern<<<dim3(tiles, planes), kGsThreads, smem, st>>>(g, c, op, r, xin, xout);
    }
}

// Planes per CTA of the marching residual: about four waves of CTAs over the
// SMs (each CTA also stages the two planes beyond its chunk), 4 .. 32 planes.
template <typename T>
int march_zlen(const Geom &g) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long tiles = (long)(g.m / kTX) * (g.n / kTY);
    const long per = 4L * sms * kMarchMinBlocks<T>;
    const long z = (g.o * tiles + per - 1) / per;
    return (int)std::min<long>(32, std::max<long>(4, z));
}

template <typename T, int KIND, bool ELASTIC, bool SPARSE>
void launch_res_tile_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, double *partial,
                       cudaStream_t st) {
    const int smem = kMarchSmemWords * (int)sizeof(T);
    const int zlen = march_zlen<T>(g);
    const dim3 grid((g.m / kTX) * (g.n / kTY), (g.o + zlen - 1) / zlen);
    static unsigned long long attr_devices = 0;   // per instantiation
    if (first_use_on_device(attr_devices)) {
        cudaFuncSetAttribute(residual_tile_kernel<T, KIND, ELASTIC, SPARSE, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(residual_tile_kernel<T, KIND, ELASTIC, SPARSE, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }
    if (partial)
        residual_tile_kernel<T, KIND, ELASTIC, SPARSE, true>
            <<<grid, kTileThreads, smem, st>>>(g, op, r, x, res, partial, zlen);
    else
        residual_tile_kernel<T, KIND, ELASTIC, SPARSE, false>
            <<<grid, kTileThreads, smem, st>>>(g, op, r, x, res, partial, zlen);
}

// ------------------------------------------- residual fused with restriction
// The descent of the V-cycle computes res = r - A x on a level and restricts
// it at once (multigrid.cc:253-297: region::compute_rats residual, then
// region::restrict, region.cc:2129-2186); res itself is read by nothing else.
// The fused kernel never writes it: each CTA takes a 32 x 32 tile of the fine
// level (16 x 16 coarse columns) and marches up z through a chunk of coarse
// planes, computing the residual of every fine plane on the tile widened by
// one node towards lower x and y (the children 2I - 1 of its first coarse
// row and column) into shared memory and adding it, with the restriction's
// weights, to the coarse nodes it belongs to.  A coarse node collects its
// fine planes 2K - 1, 2K, 2K + 1 in that order, and within a plane the rows
// and nodes in the restriction kernel's order, so its sum is the restriction
// kernel's bit for bit; the residual values are residual_tile_kernel's.
//
// Staged x rows: tile rows -2 .. 32 (buffer rows 0 .. 34), in the ring slots
// of the marching residual; the residual plane is [component][y + 1][x + 1]
// for tile nodes x, y = -1 .. 31, rows kRP words apart.
constexpr int kRR0 = kHalo - 2, kRowsRR = kTY + 3;
constexpr int kRRSlot = 3 * kRowsRR * RS;
constexpr int kRP = kTX + 2, kRPlane = (kTY + 1) * kRP;
constexpr int kRRSmemWords = kRing * kRRSlot + 3 * kRPlane;

// res = r - A x at one staged node of x-parity A (residual_tile_kernel's
// arithmetic: the shared stencil with its centre block, or r - fix x on a
// Dirichlet plate).
template <typename T, bool ELASTIC, int A>
__device__ __forceinline__ void rr_node(const ConstOp<T> &op, const unsigned (&cz)[3], bool zin, T *acc) {
    if (zin) {
        tile_const_row<T, ELASTIC, true, A, kRowsRR>(op, cz, acc);
    } else {
        T v[3];
        lds<nb_off<A, kRowsRR>(13, 0)>(cz[1], v[0]);
        lds<nb_off<A, kRowsRR>(13, 1)>(cz[1], v[1]);
        lds<nb_off<A, kRowsRR>(13, 2)>(cz[1], v[2]);
        matvec_sub(op.fix, v, acc);
    }
}

// One residual node (tile coordinates ii, jj of the widened tile) of plane k
// into the residual plane; r of the node in rv.
template <typename T, bool ELASTIC>
__device__ __forceinline__ void rr_store(const ConstOp<T> &op, unsigned s0, unsigned s1, unsigned s2, int ii, int jj,
                                         bool zin, const T (&rv)[3], T *resp) {
    const unsigned cw = (unsigned)(corner_word<kRR0>(ii, jj) * (int)sizeof(T));
    const unsigned cz[3] = {s0 + cw, s1 + cw, s2 + cw};
    T acc[3] = {rv[0], rv[1], rv[2]};
    if (ii & 1) rr_node<T, ELASTIC, 1>(op, cz, zin, acc);
    else rr_node<T, ELASTIC, 0>(op, cz, zin, acc);
    const int w = (jj - kHalo + 1) * kRP + (ii - kHalo + 1);
    resp[w] = acc[0];
    resp[kRPlane + w] = acc[1];
    resp[2 * kRPlane + w] = acc[2];
}

// Add fine plane kk's residual to the coarse nodes of this thread it is a
// child of along z: with weight w0 to acc0 (if w0 != 0) and w1 to acc1 (if
// w1 != 0; an odd plane closes one coarse plane and opens the next).  The 9
// children in the plane go in the restriction's order (rows, then nodes),
// weights 1/8 (1/2, 1, 1/2) in x and y times the z weight; each row's three
// values per component come in one 8- or 16-byte and one scalar shared load
// and serve both sums.
template <typename T>
__device__ __forceinline__ void rr_add(const T *resp, int ci, int cj, T w0, T *acc0, T w1, T *acc1) {
    using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
    const bool d0 = w0 != T(0), d1 = w1 != T(0);
#pragma unroll
    for (int b = 0; b < 3; b++) {
        T v[3][3];
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
            const T *row = resp + cc * kRPlane + (2 * cj + b) * kRP + 2 * ci;
            const V2 p = *reinterpret_cast<const V2 *>(row);
            v[cc][0] = p.x;
            v[cc][1] = p.y;
            v[cc][2] = row[2];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const T wxy = T(0.125) * (c == 1 ? T(1) : T(0.5)) * (b == 1 ? T(1) : T(0.5));
            if (d0) {
                const T w = wxy * w0;
                acc0[0] += w * v[0][c];
                acc0[1] += w * v[1][c];
                acc0[2] += w * v[2][c];
            }
            if (d1) {
                const T w = wxy * w1;
                acc1[0] += w * v[0][c];
                acc1[1] += w * v[1][c];
                acc1[2] += w * v[2][c];
            }
        }
    }
}

// Threads of the fused kernel: the marching residual's 256 (four nodes of the
// tile each, and one coarse node each) and a ninth warp for the 65 nodes of
// the widened row and column (three each), so that no thread has more than
// four residual nodes per plane.
constexpr int kRRThreads = kTileThreads + 32;
constexpr int kRRExtra = kTY + 1 + kTX;   // nodes of the column x = -1 and the row y = -1
constexpr int kRRPer = (kRRExtra + 31) / 32;

// rc = R (r - A x) for the coarse planes K0 .. K0 + zc - 1 of one tile; the
// level is periodic in x and y, its operator the shared stencil.
template <typename T, bool ELASTIC>
__global__ void __launch_bounds__(kRRThreads, kMarchMinBlocks<T>)
    res_restrict_kernel(Geom g, Geom gc, const __grid_constant__ LevelOp<T> op, const T *__restrict__ r,
                        const T *__restrict__ x, T *__restrict__ rc, int zc) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    T *resp = reinterpret_cast<T *>(smem_raw) + kRing * kRRSlot;
    const int ntx = g.m / kTX;
    const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    const int K0 = (int)blockIdx.y * zc, K1 = min(gc.o, K0 + zc);
    const int i0 = tx * kTX - kHalo, j0 = ty * kTY - kHalo;
    const size_t np = (size_t)g.npad;
    // fine planes 2 K0 - 1 .. 2 K1 - 1, unwrapped (outside a Dirichlet z: none)
    const int kf0 = 2 * K0 - 1, kf1 = 2 * K1 - 1;
    auto exists = [&](int kk) { return g.zp || (kk >= 0 && kk < g.o); };
    auto wrapk = [&](int kk) { return kk < 0 ? kk + g.o : (kk >= g.o ? kk - g.o : kk); };
    auto xslot = [&](int kk) { return sbase + (unsigned)(((kk + 2 * kRing) % kRing) * kRRSlot * (int)sizeof(T)); };

    // cp.async groups: {x of kf0-1, kf0, kf0+1}, {x of kf0+2}, then one per plane kk: {x of kk+3}
    Stager<T, kRR0, kRowsRR, kRR0, kRowsRR, kRRThreads> st;
    st.init(g, (i0 >> 1) - kHOff, j0);
    for (int kk = kf0 - 1; kk <= kf0 + 1; kk++)
        if (kk <= kf1 + 1 && exists(kk)) st.stage(g, x, wrapk(kk), xslot(kk));
    copy_commit();
    if (kf0 + 2 <= kf1 + 1 && exists(kf0 + 2)) st.stage(g, x, wrapk(kf0 + 2), xslot(kf0 + 2));
    copy_commit();

    // residual nodes of this thread: threads 0 .. 255 four of the tile
    // (residual_tile_kernel's mapping), the ninth warp up to three of the
    // widened column x = -1 (e = 0 .. 32: y = e - 1) and row y = -1
    // (e = 33 .. 64: x = e - 33), e = lane + 32 u
    const int te = (int)threadIdx.x;
    const bool main = te < kTileThreads;
    const int xs = te & 15, h = (te >> 4) & 1, a = (te >> 5) & 1;
    const int b = (te >> 6) & 1, pr0 = h + 2 * ((te >> 7) & 1);
    const int ii = kHalo + a + 2 * xs, i = wrapn(i0 + ii, g.m);
    const int lane = te & 31;
    auto enode = [&](int u, int &eii, int &ejj) {
        const int e = lane + 32 * u;
        eii = e <= kTY ? kHalo - 1 : kHalo + e - (kTY + 1);
        ejj = e <= kTY ? kHalo - 1 + e : kHalo - 1;
        return e < kRRExtra;
    };
    // this thread's coarse node (threads 0 .. 255)
    const int ci = te & 15, cj = (te >> 4) & 15;
    const int Ic = tx * (kTX / 2) + ci, Jc = ty * (kTY / 2) + cj;
    // r of this thread's nodes of plane kk (unwrapped), loaded a plane ahead
    constexpr int NV = 4 > kRRPer ? 4 : kRRPer;
    auto load_r = [&](int kk, T (&rv)[NV][3]) {
        if (!exists(kk)) return;
        const int k = wrapk(kk);
        if (main) {
#pragma unroll
            for (int it = 0; it < 4; it++) {
                const int j = wrapn(j0 + kHalo + b + 2 * (pr0 + 4 * it), g.n);
                const int s = (a + 2 * b + 4 * (k & 1)) * g.S + ((k >> 1) * g.N2 + (j >> 1)) * g.M2 + (i >> 1);
                rv[it][0] = __ldcs(r + s);
                rv[it][1] = __ldcs(r + s + np);
                rv[it][2] = __ldcs(r + s + 2 * np);
            }
        } else {
#pragma unroll
            for (int u = 0; u < kRRPer; u++) {
                int eii, ejj;
                if (enode(u, eii, ejj)) {
                    const int ei = wrapn(i0 + eii, g.m), ej = wrapn(j0 + ejj, g.n);
                    const int s = ((ei & 1) + 2 * (ej & 1) + 4 * (k & 1)) * g.S +
                                  ((k >> 1) * g.N2 + (ej >> 1)) * g.M2 + (ei >> 1);
                    rv[u][0] = r[s];
                    rv[u][1] = r[s + np];
                    rv[u][2] = r[s + 2 * np];
                }
            }
        }
    };
    T acc[3] = {T(0), T(0), T(0)};
    T rv[NV][3], rn[NV][3];
    load_r(kf0, rv);
    for (int kk = kf0; kk <= kf1; kk++) {
        const bool ex = exists(kk);
        const int k = wrapk(kk);
        if (kk + 1 <= kf1) load_r(kk + 1, rn);   // in flight while plane kk is computed
        copy_wait_but<1>();   // every group but the newest ({x of kk+2}) has landed
        __syncthreads();      // ... for every thread; the residual plane is free
        if (ex) {
            const bool zin = g.zp || (k != 0 && k != g.o - 1);
            const unsigned s0 = xslot(kk - 1), s1 = xslot(kk), s2 = xslot(kk + 1);
            if (main) {
#pragma unroll
                for (int it = 0; it < 4; it++)
                    rr_store<T, ELASTIC>(op.cop, s0, s1, s2, ii, kHalo + b + 2 * (pr0 + 4 * it), zin, rv[it], resp);
            } else {
#pragma unroll
                for (int u = 0; u < kRRPer; u++) {
                    int eii, ejj;
                    if (enode(u, eii, ejj)) rr_store<T, ELASTIC>(op.cop, s0, s1, s2, eii, ejj, zin, rv[u], resp);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < NV; u++)
#pragma unroll
            for (int e = 0; e < 3; e++) rv[u][e] = rn[u][e];
        __syncthreads();      // residual plane complete; x slot of plane kk - 1 free
        if (kk + 3 <= kf1 + 1 && exists(kk + 3)) st.stage(g, x, wrapk(kk + 3), xslot(kk + 3));
        copy_commit();
        if (!main) continue;
        if (kk & 1) {
            // plane kk = 2K + 1 closes coarse plane K = (kk - 1) / 2 and opens K + 1
            const int K = (kk - 1) >> 1;
            const T w0 = ex && K >= K0 ? child_w<T>(K, kk, g.o, g.zp) : T(0);
            const T w1 = ex && K + 1 < K1 ? child_w<T>(K + 1, kk, g.o, g.zp) : T(0);
            T nxt[3] = {T(0), T(0), T(0)};
            rr_add<T>(resp, ci, cj, w0, acc, w1, nxt);
            if (K >= K0) {
                const int p = slot(gc, Ic, Jc, K);
                rc[p] = acc[0];
                rc[p + gc.npad] = acc[1];
                rc[p + 2 * gc.npad] = acc[2];
            }
            acc[0] = nxt[0];
            acc[1] = nxt[1];
            acc[2] = nxt[2];
        } else {
            const T w0 = ex ? child_w<T>(kk >> 1, kk, g.o, g.zp) : T(0);
            rr_add<T>(resp, ci, cj, w0, acc, T(0), acc);
        }
    }
    copy_wait_but<0>();
}

// Coarse planes per CTA of the fused kernel: about four waves of CTAs over
// the SMs, 2 .. 16 coarse planes (each CTA also computes the fine plane below
// its chunk).
template <typename T>
int rr_zc(const Geom &g, const Geom &gc) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long tiles = (long)(g.m / kTX) * (g.n / kTY);
    const long per = 4L * sms * kMarchMinBlocks<T>;
    const long z = (gc.o * tiles + per - 1) / per;
    return (int)std::min<long>(16, std::max<long>(2, z));
}

template <typename T, bool ELASTIC>
void launch_rr_k(const LevelOp<T> &op, const Geom &g, const Geom &gc, const T *r, const T *x, T *rc,
                 cudaStream_t st) {
    const int smem = kRRSmemWords * (int)sizeof(T);
    const int zc = rr_zc<T>(g, gc);
    const dim3 grid((g.m / kTX) * (g.n / kTY), (gc.o + zc - 1) / zc);
    static unsigned long long attr_devices = 0;   // per instantiation
    if (first_use_on_device(attr_devices))
        cudaFuncSetAttribute(res_restrict_kernel<T, ELASTIC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    res_restrict_kernel<T, ELASTIC><<<grid, kRRThreads, smem, st>>>(g, gc, op, r, x, rc, zc);
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
// FP32): 167 vs 223 us on the fine shared-stencil level and 72 vs 166 us on
// the plane-invariant level 1 against the colour-interleaved residual kernel,
// so by default it runs on FP32 levels of at least 64x64 nodes per plane.
// STZ_MG_TILE=0 disables it, STZ_MG_TILE=1 uses it in FP64 too.
template <typename T>
bool residual_tile_applies(const LevelOp<T> &op, const Geom &g) {
    int mode = -1;
    if (const char *e = std::getenv("STZ_MG_TILE")) mode = std::atoi(e) != 0;
    if (mode == 0) return false;
    if (op.kind != OP_CONST && op.kind != OP_PLANE) return false;
    if (mode < 0 && sizeof(T) != 4) return false;
    return g.xp && g.yp && g.m % kTX == 0 && g.n % kTY == 0 && g.m * g.n >= 64 * 64;
}

int residual_tile_blocks(const Geom &g, bool fp64) {
    const int zlen = fp64 ? march_zlen<double>(g) : march_zlen<float>(g);
    return (g.m / kTX) * (g.n / kTY) * ((g.o + zlen - 1) / zlen);
}

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

// The descent's residual and restriction in one pass (res_restrict_kernel)
// where the tiled residual runs on a shared-stencil level periodic in x and y
// (an even z extent if z is periodic): rc = R (r - A x), res not written.
// Opt-in (STZ_MG_FUSED_RESTRICT=1): measured on a GB300 at 256x256x257 it
// saves the 404 MB of res traffic per cycle but is slower than the two
// kernels (about 238 against 226 us per cycle, the mixed solve 23.0 against
// 22.9 ms), because the marching residual is bound by the shared-memory pipe,
// not by DRAM, and the restriction's loads (and the widened row and column)
// add to that pipe.  False where it does not apply or is not enabled (the
// caller runs the two kernels).
template <typename T>
bool launch_residual_restrict(const LevelOp<T> &op, const Geom &g, const Geom &gc, const T *r, const T *x, T *rc,
                              cudaStream_t st) {
    const char *e = std::getenv("STZ_MG_FUSED_RESTRICT");
    if (!e || std::atoi(e) == 0) return false;
    if (op.kind != OP_CONST || !residual_tile_applies(op, g)) return false;
    if (g.zp && (g.o & 1)) return false;
    if (gc.m * 2 != g.m || gc.n * 2 != g.n || !gc.xp || !gc.yp || gc.zp != g.zp) return false;
    if (op.cop.elastic) {
        launch_rr_k<T, true>(op, g, gc, r, x, rc, st);
        return true;
    }
    if constexpr (sizeof(T) == 4) {   // a full-block row in FP64 would spill: the two kernels run instead
        launch_rr_k<T, false>(op, g, gc, r, x, rc, st);
        return true;
    }
    return false;
}
template bool launch_residual_restrict<float>(const LevelOp<float> &, const Geom &, const Geom &, const float *,
                                              const float *, float *, cudaStream_t);
template bool launch_residual_restrict<double>(const LevelOp<double> &, const Geom &, const Geom &, const double *,
                                               const double *, double *, cudaStream_t);

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
