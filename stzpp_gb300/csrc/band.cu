// Band Gauss-Seidel sweep of the levels periodic in x and y -- the fine
// level's shared elasticity stencil and the plane-invariant coarse operators
// below it -- two launches per sweep, every CTA staging its planes with the
// tensor-memory-access (TMA) engine; and the band residual of the
// plane-invariant levels from the same staging.
//
// Replaces, on those levels, the eight colour launches of smooth.cu
// (region::gauss_seidel, region.cc:1557-1762,
// in the 8-colour order q = (i&1) + 2(j&1) + 4(k&1)).  Colours 0-3 live on
// even z-planes and 4-7 on odd ones, and a colour couples only to its own
// plane and the planes above and below.  So a sweep is two launches (even
// planes, then odd planes) reading x_in and writing x_out; each CTA takes one
// band of 8 node rows spanning the whole periodic x range of one plane and
// runs the plane's four colours in order from shared memory:
//
//  * the in-plane chain of the colour order needs only one row of halo: the
//    colours (a, b) = (0,0), (1,0), (0,1), (1,1) depend on each other
//    through x-faces (0->1, 2->3), y-faces (0->2, 1->3) and xy-edges (0->3,
//    1->2), so colours 0 and 1 are computed on the band plus the first row of
//    the next band, colours 2 and 3 on the band itself, from old values on
//    the band widened by one row on each side;
//  * the whole x range is in the CTA, so the periodic wrap in x is an index
//    wrap in shared memory and there is no x halo at all;
//  * planes k-1, k, k+1 of the widened band (3 components each) arrive by
//    cp.async.bulk.tensor boxes completing on one mbarrier; at the periodic
//    wrap in y a box is split in two (rows N2-1 and 0.. or ..N2-1 and 0);
//  * the planes above and below are old (x_in, even launch) or new (x_out,
//    odd launch) values, as in the colour order.
//
// Each node update has the arithmetic of const_row (ops.cuh) in the same
// order, so the sweep is bit-identical to the eight colour launches.  Every
// wait is an mbarrier wait with a time limit; a CTA whose copies do not
// arrive in time records the fact (band_take_error) and returns.
#include <cuda.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "launch.h"
#include "ops.cuh"

namespace stzmg {

__device__ int g_band_err = 0;

namespace {

// Node rows of a band: 8 on every level.  Measured at 256x256x257 (mixed
// solve, one box): 16-row bands on the 128x128 level 1 take its two sweeps
// from 123 to 108 us timed alone, yet the solve from 22.79 to 22.85 ms (the
// level's residual, and the launches around it, lose more); on the fine
// level 16 rows leave one CTA per SM (371 against 337 us), on levels of
// 16-32 columns they halve the CTAs of a launch (the solve 23.0 -> 23.6 ms);
// 4 rows are slower everywhere (fine level 366 us).
__host__ __device__ constexpr int band_rows(int) { return 8; }
template <int M2>
constexpr int kOwnSub = band_rows(M2) / 2;      // sub-grid rows per parity owned by a band
template <int M2>
constexpr int kStageRows = kOwnSub<M2> + 2;     // staged sub-rows J0-1 .. J0+kOwnSub

// Shared-memory layout of the staged band: plane p (0: k-1, 1: k, 2: k+1),
// component c, sub-row Jr (staged row 0 is sub-row J0-1), colour ab = a + 2b
// of the plane, sub-grid column I: Jr outside ab, so one TMA box brings a
// plane's component (all four colours of the staged sub-rows).
template <int M2>
__host__ __device__ constexpr int woff(int p, int c, int Jr, int ab, int I) {
    return (((p * 3 + c) * kStageRows<M2> + Jr) * 4 + ab) * M2 + I;
}
template <int M2>
constexpr int kBandWords = 3 * 3 * kStageRows<M2> * 4 * M2;

template <int B, int E, typename F>
__device__ __forceinline__ void sfor(F &&f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor<B + 1, E>(f);
    }
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    return ok != 0;
}

// Wait for phase `phase` of the barrier for at most `limit_ns`.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned phase, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (!mbar_try(bar, phase))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

// One box of a 5-d tensor map into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load5(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                          int c4, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

// The tensor maps of one field (x_in or x_out): boxes of kStageRows,
// kStageRows - 1 and 1 sub-rows.
struct BandMaps {
    CUtensorMap full, less1, one;
};

struct BandArgs {
    Geom g;
    int c;          // plane parity of this launch
    int nbands;     // n / band_rows(M2)
    int nplanes;    // planes of parity c
    int rev;        // planes taken from the top down
    const void *xz; // the residual's x (read directly on Dirichlet plates)
};

// Stage plane kk of a field (three components) into buffer plane p: boxes
// cover sub-rows J0-1 .. J0+kOwnSub, split where they cross the periodic
// wrap in y.  Every plane delivers a third of kBandWords<M2> elements.
template <typename T, int M2>
__device__ __forceinline__ void stage_plane(const BandMaps &mp, const Geom &g, int kk, int J0, int p,
                                                unsigned sbase, unsigned bar) {
    const int K = kk >> 1, cpar = kk & 1;
    constexpr unsigned rowb = 4 * M2 * sizeof(T);   // bytes per staged sub-row (four colours)
    for (int comp = 0; comp < 3; comp++) {
        const unsigned dst = sbase + (unsigned)(woff<M2>(p, comp, 0, 0, 0) * (int)sizeof(T));
        const int cc = 2 * comp + cpar;
        // coordinates (I, ab, J, K, cc)
        if (J0 == 0) {   // rows N2-1 | 0 .. kOwnSub
            tma_load5(dst, &mp.one, 0, 0, g.N2 - 1, K, cc, bar);
            tma_load5(dst + rowb, &mp.less1, 0, 0, 0, K, cc, bar);
        } else if (J0 + kOwnSub<M2> == g.N2) {   // rows J0-1 .. N2-1 | 0
            tma_load5(dst, &mp.less1, 0, 0, J0 - 1, K, cc, bar);
            tma_load5(dst + (kStageRows<M2> - 1) * rowb, &mp.one, 0, 0, 0, K, cc, bar);
        } else {
            tma_load5(dst, &mp.full, 0, 0, J0 - 1, K, cc, bar);
        }
    }
}

// Plane k's coarse row in shared memory: block b's 9 coefficients at
// kCoefPad * b (padded to 16-byte boundaries), the inverse centre block at
// kCoefPad * 27.
constexpr int kCoefPad = 12;
constexpr int kCoefWords = kCoefPad * 28;

// The 9 entries of one padded block (the 16-byte loads cover 12).
template <typename T>
__device__ __forceinline__ void load_block_coef(const T *p, T (&c)[kCoefPad]) {
    if constexpr (sizeof(T) == 4) {
        const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float4 w = q[i];
            c[4 * i] = w.x; c[4 * i + 1] = w.y; c[4 * i + 2] = w.z; c[4 * i + 3] = w.w;
        }
    } else {
        const double2 *q = reinterpret_cast<const double2 *>(p);
#pragma unroll
        for (int i = 0; i < 5; i++) {
            const double2 w = q[i];
            c[2 * i] = w.x; c[2 * i + 1] = w.y;
        }
        c[10] = c[11] = T(0);
    }
}

// Plane k's row into the padded shared layout (all threads of the CTA).
template <typename T>
__device__ __forceinline__ void stage_coef(const PlaneOp<T> &pop, int k, T *cfs, int tid, int nthreads) {
    for (int e = tid; e < 252; e += nthreads) {
        const int b = e / 9, i = e % 9;
        cfs[kCoefPad * b + i] = e < 243 ? pop.coef[e * pop.O + k] : pop.dinv[(e - 243) * pop.O + k];
    }
}

// One colour (A, B) of plane k (buffer plane 1) on up to NR sub-rows
// T0 .. T0+NR-1 (those below NT) of this thread's sub-grid column I: new
// values from r (rr) and the staged neighbours, in the arithmetic and order
// of const_row<T, true, false>, then the centre solve.  Neighbour
// (dx, dy, dz) of a node of parity (A, B) lies in colour ((A+dx)&1, (B+dy)&1)
// at column I + floor((A+dx)/2) (wrapped: base index ib[0..2] for shifts -1,
// 0, +1, which already include the rows T0) and staged row
// Jr + floor((B+dy)/2), Jr = t + 1.
// KIND: OP_CONST (the elasticity stencil shared by every interior node, op.cop)
// or OP_PLANE (the row of coefficients of plane k, cf: 243 entries and the 9
// of the inverse centre block, in shared memory; SPARSE: the structural
// zeros of the coarse elasticity operators), with the arithmetic of
// const_row<T, true, false> or plane_row_coef<T, SPARSE, false>.
template <typename T, int M2, int KIND, bool SPARSE, int A, int B, int NR>
__device__ __forceinline__ void band_colour(const T *__restrict__ s, const int (&ib)[3], const LevelOp<T> &op,
                                            const T *cf, int nvalid, const T (&rr)[NR][3], T (&out)[NR][3]) {
    constexpr bool CONST = KIND == OP_CONST;
    constexpr int rowstep = woff<M2>(0, 0, 1, 0, 0);
    if constexpr (!CONST) {
        // plane k's coarse row, one block at a time: its 9 coefficients
        // (16-byte shared loads of the padded row, the same for every thread)
        // serve all of this thread's rows, then each row takes its three
        // neighbour values and its products in plane_row_coef's order
        if (nvalid <= 0) return;
        // rows past this thread's last repeat its last row (no branch inside
        // the block loop; their results are not stored)
        int roff[NR];
#pragma unroll
        for (int u = 0; u < NR; u++) roff[u] = (1 + min(u, nvalid - 1)) * rowstep;
        T acc[NR][3];
#pragma unroll
        for (int u = 0; u < NR; u++)
#pragma unroll
            for (int e = 0; e < 3; e++) acc[u][e] = rr[u][e];
        // one block: its coefficients at cf + kCoefPad * b, its neighbours in
        // buffer plane 1 + dz (shared-memory offset pz of that plane)
        auto block = [&](auto bi, int b, int pz) {
            constexpr int bxy = decltype(bi)::value;   // dx + 1 + 3 (dy + 1)
            constexpr int dx = bxy % 3 - 1, dy = bxy / 3 - 1;
            constexpr int ap = (A + dx + 2) & 1, sI = (A + dx + 2) / 2 - 1;
            constexpr int bp = (B + dy + 2) & 1, sJ = (B + dy + 2) / 2 - 1;
            asm volatile("" ::: "memory");
            T cb[kCoefPad];
            load_block_coef<T>(cf + kCoefPad * b, cb);
#pragma unroll
            for (int u = 0; u < NR; u++) {
                const int base = ib[sI + 1] + roff[u] + sJ * rowstep + pz;
                T v[3];
                v[0] = s[base + woff<M2>(0, 0, 0, ap + 2 * bp, 0)];
                v[1] = s[base + woff<M2>(0, 1, 0, ap + 2 * bp, 0)];
                v[2] = s[base + woff<M2>(0, 2, 0, ap + 2 * bp, 0)];
#pragma unroll
                for (int e = 0; e < 9; e++)
                    if (!SPARSE || coarse_entry(b, e)) acc[u][e / 3] -= cb[e] * v[e % 3];
            }
        };
        if constexpr (SPARSE) {
            // the structural zeros depend on the block: every block unrolled
            sfor<0, 27>([&](auto bi) {
                constexpr int b = decltype(bi)::value;
                if constexpr (b != 13)
                    block(std::integral_constant<int, b % 9>{}, b, (bdz(b) + 1) * woff<M2>(1, 0, 0, 0, 0));
            });
        } else {
            // the three planes of blocks in turn (blocks in ascending order,
            // as plane_row_coef takes them), the nine of a plane unrolled: a
            // third of the code of the whole unrolled row, which stalled on
            // instruction fetch (level 1, two sweeps: 123 -> 115 us; the
            // mixed solve 22.64 -> 22.03 ms)
#pragma unroll 1
            for (int dz = 0; dz < 3; dz++) {
                const int pz = dz * woff<M2>(1, 0, 0, 0, 0);
                sfor<0, 9>([&](auto bi) {
                    constexpr int bxy = decltype(bi)::value;
                    if (dz != 1 || bxy != 4) block(bi, 9 * dz + bxy, pz);   // not the centre
                });
            }
        }
        T inv[kCoefPad];
        load_block_coef<T>(cf + kCoefPad * 27, inv);
#pragma unroll
        for (int u = 0; u < NR; u++) {
            if (u >= nvalid) break;
            out[u][0] = dot3(inv[0], acc[u][0], inv[1], acc[u][1], inv[2], acc[u][2]);
            out[u][1] = dot3(inv[3], acc[u][0], inv[4], acc[u][1], inv[5], acc[u][2]);
            out[u][2] = dot3(inv[6], acc[u][0], inv[7], acc[u][1], inv[8], acc[u][2]);
        }
        return;
    }
#pragma unroll
    for (int u = 0; u < NR; u++) {
        if (u >= nvalid) break;   // warp-uniform
        const int Jr = u + 1;
        T v[27][3];
        sfor<0, 27>([&](auto bi) {
            constexpr int b = decltype(bi)::value;
            if constexpr (b != 13 && nnz_axes(b) != 3) {
                constexpr int dx = bdx(b), dy = bdy(b), dz = bdz(b);
                constexpr int ap = (A + dx + 2) & 1, sI = (A + dx + 2) / 2 - 1;
                constexpr int bp = (B + dy + 2) & 1, sJ = (B + dy + 2) / 2 - 1;
                sfor<0, 3>([&](auto ci) {
                    constexpr int c = decltype(ci)::value;
                    constexpr bool used = elastic_entry(b, c) || elastic_entry(b, 3 + c) || elastic_entry(b, 6 + c);
                    if constexpr (used) v[b][c] = s[ib[sI + 1] + woff<M2>(1 + dz, c, 0, ap + 2 * bp, 0) +
                                                    (Jr + sJ) * woff<M2>(0, 0, 1, 0, 0)];
                    else v[b][c] = T(0);
                });
            }
        });
        T acc[3] = {rr[u][0], rr[u][1], rr[u][2]};
#pragma unroll
        for (int b = 0; b < 27; b++) {
            if (b == 13 || nnz_axes(b) == 3) continue;
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (elastic_entry(b, e)) acc[e / 3] -= op.cop.a[b][e] * v[b][e % 3];
        }
        const T *inv = op.cop.inv_int;
        out[u][0] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
        out[u][1] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
        out[u][2] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
    }
}

// Slot (component 0) of colour ab of plane parity c, sub-grid row J (wrapped), column I.
__device__ __forceinline__ size_t band_slot(const Geom &g, int ab, int c, int K, int J, int I) {
    return (size_t)(ab + 4 * c) * g.S + ((size_t)K * g.N2 + J) * g.M2 + I;
}

// Rows of a colour per thread: colours 0 and 1 run on kOwnSub + 1 sub-rows,
// 2 and 3 on kOwnSub; NH threads share a column, thread h taking rows
// h * per .. (the rest of the column when fewer).
template <int NRT, int NH>
constexpr int kPer = (NRT + NH - 1) / NH;

// One work item of a launch: band `band` of plane k (parity args.c).
struct BandItem {
    int band, k, K, J0;
    bool zin, has_lo, has_hi;
};

template <int M2>
__device__ __forceinline__ BandItem band_item(const BandArgs &args, int item) {
    const Geom &g = args.g;
    BandItem it;
    it.band = item % args.nbands;
    const int kraw = item / args.nbands;
    it.K = args.rev ? args.nplanes - 1 - kraw : kraw;
    it.k = 2 * it.K + args.c;
    it.J0 = it.band * kOwnSub<M2>;
    it.zin = g.zp || (it.k != 0 && it.k != g.o - 1);
    // planes k-1, k+1 exist (a Dirichlet z ends at the plates)
    it.has_lo = g.zp || it.k > 0;
    it.has_hi = g.zp || it.k < g.o - 1;
    return it;
}

// Whether an item stages planes (a plate of the shared stencil does not).
template <int KIND>
__device__ __forceinline__ bool band_stages(const BandItem &it) {
    return KIND == OP_PLANE || it.zin;
}

// Thread 0: the boxes of an item's planes into the buffer at sbuf,
// completing on bar (every byte announced before any box is issued).
template <typename T, int M2>
__device__ __forceinline__ void band_issue(const BandArgs &args, const BandMaps &in, const BandMaps &out_maps,
                                           const BandItem &it, unsigned sbuf, unsigned bar) {
    const Geom &g = args.g;
    const unsigned plane_bytes = (unsigned)(kBandWords<M2> / 3 * sizeof(T));
    mbar_expect_tx(bar, plane_bytes * (1u + it.has_lo + it.has_hi));
    // the z-neighbour planes: old values (x_in) under the even launch, new
    // ones (x_out) under the odd launch; plane k itself from x_in
    const BandMaps &zm = args.c == 0 ? in : out_maps;
    const int klo = it.k == 0 ? g.o - 1 : it.k - 1, khi = it.k == g.o - 1 ? 0 : it.k + 1;
    if (it.has_lo) stage_plane<T, M2>(zm, g, klo, it.J0, 0, sbuf, bar);
    stage_plane<T, M2>(in, g, it.k, it.J0, 1, sbuf, bar);
    if (it.has_hi) stage_plane<T, M2>(zm, g, khi, it.J0, 2, sbuf, bar);
}

// A Dirichlet plate of the shared stencil: x = fix^-1 r, no neighbours.
template <typename T, int M2, int NH>
__device__ __forceinline__ void band_plate(const Geom &g, const ConstOp<T> &op, const BandItem &it, int c,
                                           const T *__restrict__ r, T *__restrict__ xout) {
    const int tid = threadIdx.x, I = tid % M2, hh = tid / M2;
    const size_t np = (size_t)g.npad;
    const T *inv = op.inv_fix;
#pragma unroll 1
    for (int w = hh; w < 4 * kOwnSub<M2>; w += NH) {
        const int ab = w / kOwnSub<M2>, t = w % kOwnSub<M2>;
        const size_t sl = band_slot(g, ab, c, it.K, it.J0 + t, I);
        const T a0 = r[sl], a1 = r[sl + np], a2 = r[sl + 2 * np];
        xout[sl] = dot3(inv[0], a0, inv[1], a1, inv[2], a2);
        xout[sl + np] = dot3(inv[3], a0, inv[4], a1, inv[5], a2);
        xout[sl + 2 * np] = dot3(inv[6], a0, inv[7], a1, inv[8], a2);
    }
}

// All threads: one staged item -- r of this thread's nodes (loaded while the
// boxes are in flight), the wait for the boxes (phase `phase` of bar, at
// most 0.2 s), then the plane's four colours.  False if the boxes did not
// arrive (recorded; every thread returns false).
template <typename T, int M2, int NH, int KIND, bool SPARSE>
__device__ __forceinline__ bool band_compute(const BandArgs &args, const LevelOp<T> &op, const BandItem &it, T *s,
                                             T *cfs, unsigned bar, unsigned phase, const T *__restrict__ r,
                                             T *__restrict__ xout) {
    const Geom &g = args.g;
    const int tid = threadIdx.x, I = tid % M2, hh = tid / M2;
    const int c = args.c, K = it.K, J0 = it.J0, k = it.k;
    const size_t np = (size_t)g.npad;
    // this thread's rows of each colour
    constexpr int OWN = kOwnSub<M2>;
    constexpr int P0 = kPer<OWN + 1, NH>, P1 = kPer<OWN, NH>;
    const int t0a = hh * P0, t0b = hh * P1;
    const int na = min(P0, OWN + 1 - t0a), nb = min(P1, OWN - t0b);
    T r0[P0][3], r1[P0][3], r2[P1][3], r3[P1][3];
#pragma unroll
    for (int u = 0; u < P0; u++) {
        if (u >= na) break;
        const int J = J0 + t0a + u == g.N2 ? 0 : J0 + t0a + u;
        const size_t s0 = band_slot(g, 0, c, K, J, I), s1 = band_slot(g, 1, c, K, J, I);
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
            r0[u][cc] = __ldcs(r + s0 + cc * np);
            r1[u][cc] = __ldcs(r + s1 + cc * np);
        }
    }
#pragma unroll
    for (int u = 0; u < P1; u++) {
        if (u >= nb) break;
        const size_t s2 = band_slot(g, 2, c, K, J0 + t0b + u, I), s3 = band_slot(g, 3, c, K, J0 + t0b + u, I);
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
            r2[u][cc] = __ldcs(r + s2 + cc * np);
            r3[u][cc] = __ldcs(r + s3 + cc * np);
        }
    }
    if (KIND == OP_PLANE) stage_coef<T>(op.pop, k, cfs, tid, NH * M2);   // plane k's row of coefficients
    const bool ok = mbar_wait(bar, phase, 200000000ull);   // 0.2 s: copies that never arrive
    if (!__syncthreads_and(ok)) {
        if (tid == 0) {
            atomicExch(&g_band_err, 1);
            mbar_wait(bar, phase, 200000000ull);   // let copies still in flight land before the CTA leaves
        }
        __syncthreads();
        return false;
    }
    if (KIND == OP_PLANE && !(it.has_lo && it.has_hi)) {
        // a missing neighbour plane reads as zeros (the colour kernels'
        // neighbour outside the grid)
        constexpr int PW = kBandWords<M2> / 3;
        if (!it.has_lo)
            for (int w = tid; w < PW; w += NH * M2) s[w] = T(0);
        if (!it.has_hi)
            for (int w = tid; w < PW; w += NH * M2) s[2 * PW + w] = T(0);
        __syncthreads();
    }
    constexpr int rowstep = woff<M2>(0, 0, 1, 0, 0);
    const int ibx[3] = {I == 0 ? M2 - 1 : I - 1, I, I == M2 - 1 ? 0 : I + 1};
    const int iba[3] = {ibx[0] + t0a * rowstep, ibx[1] + t0a * rowstep, ibx[2] + t0a * rowstep};
    const int ibb[3] = {ibx[0] + t0b * rowstep, ibx[1] + t0b * rowstep, ibx[2] + t0b * rowstep};
    // store a colour's new values: shared memory for the later colours, x_out
    // for the rows this band owns
    auto emit = [&](auto A_, auto B_, auto NR_, int t0, int nv, const auto &o, bool to_smem) {
        constexpr int A = decltype(A_)::value, B = decltype(B_)::value, NR = decltype(NR_)::value;
#pragma unroll
        for (int u = 0; u < NR; u++) {
            if (u >= nv) break;
            const int t = t0 + u;
            if (to_smem)
#pragma unroll
                for (int cc = 0; cc < 3; cc++) s[I + woff<M2>(1, cc, 0, A + 2 * B, 0) + (t + 1) * rowstep] = o[u][cc];
            if (t < OWN) {
                const size_t sl = band_slot(g, A + 2 * B, c, K, J0 + t, I);
#pragma unroll
                for (int cc = 0; cc < 3; cc++) xout[sl + cc * np] = o[u][cc];
            }
        }
    };
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using NR0 = std::integral_constant<int, P0>;
    using NR1 = std::integral_constant<int, P1>;
    {
        T o[P0][3];
        band_colour<T, M2, KIND, SPARSE, 0, 0, P0>(s, iba, op, cfs, na, r0, o);
        emit(I0{}, I0{}, NR0{}, t0a, na, o, true);
    }
    __syncthreads();
    {
        T o[P0][3];
        band_colour<T, M2, KIND, SPARSE, 1, 0, P0>(s, iba, op, cfs, na, r1, o);
        emit(I1{}, I0{}, NR0{}, t0a, na, o, true);
    }
    __syncthreads();
    {
        T o[P1][3];
        band_colour<T, M2, KIND, SPARSE, 0, 1, P1>(s, ibb, op, cfs, nb, r2, o);
        emit(I0{}, I1{}, NR1{}, t0b, nb, o, true);
    }
    __syncthreads();
    {
        T o[P1][3];
        band_colour<T, M2, KIND, SPARSE, 1, 1, P1>(s, ibb, op, cfs, nb, r3, o);
        emit(I1{}, I1{}, NR1{}, t0b, nb, o, false);
    }
    return true;
}

// One CTA per work item.
// CTAs per SM the sweep's registers must allow: on the widest FP32 level as
// many as the staging buffer lets share an SM's 228 KB (two of 110.6 KB with
// 8-row bands); one elsewhere (ptxas then keeps every value in registers).
template <typename T, int M2, int KIND>
constexpr int kBandMinBlocks =
    sizeof(T) == 4 && M2 >= 128 ? (KIND == OP_CONST ? 233472 / (kBandWords<M2> * 4 + 2048) : 2) : 1;

template <typename T, int M2, int NH, int KIND, bool SPARSE>
__global__ void __launch_bounds__(NH * M2, (kBandMinBlocks<T, M2, KIND>))
    gs_band_kernel(const BandArgs args, const __grid_constant__ LevelOp<T> op, const __grid_constant__ BandMaps in,
                   const __grid_constant__ BandMaps out_maps, const T *__restrict__ r, T *__restrict__ xout) {
    extern __shared__ __align__(128) unsigned char band_smem[];
    __shared__ __align__(8) unsigned long long bar_store;
    __shared__ __align__(16) T cfs[KIND == OP_PLANE ? kCoefWords : 4];
    const int tid = threadIdx.x;
    const BandItem it = band_item<M2>(args, blockIdx.x);
    if (!band_stages<KIND>(it)) {
        band_plate<T, M2, NH>(args.g, op.cop, it, args.c, r, xout);
        return;
    }
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(band_smem);
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&bar_store);
    if ((sbase & 127u) != 0) {   // TMA boxes land at 128-byte aligned shared addresses only
        if (tid == 0) atomicExch(&g_band_err, 2);
        return;
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) band_issue<T, M2>(args, in, out_maps, it, sbase, bar);
    band_compute<T, M2, NH, KIND, SPARSE>(args, op, it, reinterpret_cast<T *>(band_smem), cfs, bar, 0, r, xout);
}

// ------------------------------------------------------------ residual
// res = r - A x on one band of plane k: the same staging, every colour on the
// band's own rows (no chain between colours, so no halo row and no barrier
// between them), in the arithmetic and order of residual_kernel
// (const_row<T, ELASTIC, true> / plane_row_coef<T, SPARSE, true>).
template <typename T, int M2, int KIND, bool SPARSE, int A, int B, int NR>
__device__ __forceinline__ void band_res_colour(const T *__restrict__ s, const int (&ib)[3], const LevelOp<T> &op,
                                                const T *cf, int t0, int nv, const Geom &g, int c, int K, int J0,
                                                int I, const T *__restrict__ r, T *__restrict__ res) {
    constexpr int rowstep = woff<M2>(0, 0, 1, 0, 0);
    const size_t np = (size_t)g.npad;
    if constexpr (KIND != OP_CONST) {
        // plane k's coarse row, one block at a time: its 9 coefficients
        // (16-byte shared loads) serve all of this thread's rows, each row
        // taking its three values and its products in plane_row_coef's order
        if (nv <= 0) return;
        // rows past this thread's last repeat its last row (no branch inside
        // the block loop; their results are not stored)
        int roff[NR];
        T acc[NR][3];
#pragma unroll
        for (int u = 0; u < NR; u++) {
            const int t = t0 + min(u, nv - 1);
            roff[u] = (t + 1) * rowstep;
            const size_t sl = band_slot(g, A + 2 * B, c, K, J0 + t, I);
            acc[u][0] = r[sl];
            acc[u][1] = r[sl + np];
            acc[u][2] = r[sl + 2 * np];
        }
        // one block (as in band_colour), the planes of blocks rolled where
        // no structural zeros are skipped
        auto block = [&](auto bi, int b, int pz) {
            constexpr int bxy = decltype(bi)::value;
            constexpr int dx = bxy % 3 - 1, dy = bxy / 3 - 1;
            constexpr int ap = (A + dx + 2) & 1, sI = (A + dx + 2) / 2 - 1;
            constexpr int bp = (B + dy + 2) & 1, sJ = (B + dy + 2) / 2 - 1;
            asm volatile("" ::: "memory");
            T cb[kCoefPad];
            load_block_coef<T>(cf + kCoefPad * b, cb);
#pragma unroll
            for (int u = 0; u < NR; u++) {
                const int base = ib[sI + 1] + roff[u] + sJ * rowstep + pz;
                T v[3];
                v[0] = s[base + woff<M2>(0, 0, 0, ap + 2 * bp, 0)];
                v[1] = s[base + woff<M2>(0, 1, 0, ap + 2 * bp, 0)];
                v[2] = s[base + woff<M2>(0, 2, 0, ap + 2 * bp, 0)];
#pragma unroll
                for (int e = 0; e < 9; e++)
                    if (!SPARSE || coarse_entry(b, e)) acc[u][e / 3] -= cb[e] * v[e % 3];
            }
        };
        if constexpr (SPARSE) {
            sfor<0, 27>([&](auto bi) {
                constexpr int b = decltype(bi)::value;
                block(std::integral_constant<int, b % 9>{}, b, (bdz(b) + 1) * woff<M2>(1, 0, 0, 0, 0));
            });
        } else {
#pragma unroll 1
            for (int dz = 0; dz < 3; dz++) {
                const int pz = dz * woff<M2>(1, 0, 0, 0, 0);
                sfor<0, 9>([&](auto bi) { block(bi, 9 * dz + decltype(bi)::value, pz); });
            }
        }
#pragma unroll
        for (int u = 0; u < NR; u++)
            if (u < nv) {
                const size_t sl = band_slot(g, A + 2 * B, c, K, J0 + t0 + u, I);
                res[sl] = acc[u][0];
                res[sl + np] = acc[u][1];
                res[sl + 2 * np] = acc[u][2];
            }
        return;
    }
#pragma unroll 1
    for (int u = 0; u < NR; u++) {
        if (u >= nv) break;
        const int t = t0 + u, Jr = t + 1;
        const size_t sl = band_slot(g, A + 2 * B, c, K, J0 + t, I);
        T acc[3] = {r[sl], r[sl + np], r[sl + 2 * np]};
        {
            T v[27][3];
            sfor<0, 27>([&](auto bi) {
                constexpr int b = decltype(bi)::value;
                if constexpr (nnz_axes(b) != 3) {
                    constexpr int dx = bdx(b), dy = bdy(b), dz = bdz(b);
                    constexpr int ap = (A + dx + 2) & 1, sI = (A + dx + 2) / 2 - 1;
                    constexpr int bp = (B + dy + 2) & 1, sJ = (B + dy + 2) / 2 - 1;
                    sfor<0, 3>([&](auto ci) {
                        constexpr int cc = decltype(ci)::value;
                        constexpr bool used =
                            b == 13 || elastic_entry(b, cc) || elastic_entry(b, 3 + cc) || elastic_entry(b, 6 + cc);
                        if constexpr (used) v[b][cc] = s[ib[sI + 1] + woff<M2>(1 + dz, cc, 0, ap + 2 * bp, 0) +
                                                         (Jr + sJ) * rowstep];
                        else v[b][cc] = T(0);
                    });
                }
            });
#pragma unroll
            for (int b = 0; b < 27; b++) {
                if (nnz_axes(b) == 3) continue;
                if (b != 13) {
#pragma unroll
                    for (int e = 0; e < 9; e++)
                        if (elastic_entry(b, e)) acc[e / 3] -= op.cop.a[b][e] * v[b][e % 3];
                } else if (op.cop.centre_diag) {
                    acc[0] -= op.cop.a[13][0] * v[13][0];
                    acc[1] -= op.cop.a[13][4] * v[13][1];
                    acc[2] -= op.cop.a[13][8] * v[13][2];
                } else {
                    matvec_sub(op.cop.a[13], v[13], acc);
                }
            }
        }
        res[sl] = acc[0];
        res[sl + np] = acc[1];
        res[sl + 2 * np] = acc[2];
    }
}

template <typename T, int M2, int NH, int KIND, bool SPARSE>
__global__ void __launch_bounds__(NH * M2, sizeof(T) == 4 && M2 >= 128 ? 2 : 1)
    residual_band_kernel(const BandArgs args, const __grid_constant__ LevelOp<T> op,
                         const __grid_constant__ BandMaps xm, const T *__restrict__ r, T *__restrict__ res) {
    extern __shared__ __align__(128) unsigned char band_smem[];
    __shared__ __align__(8) unsigned long long bar_store;
    __shared__ __align__(16) T cfs[KIND == OP_PLANE ? kCoefWords : 4];
    const Geom &g = args.g;
    const int tid = threadIdx.x, I = tid % M2, hh = tid / M2;
    const int band = blockIdx.x % args.nbands, k = blockIdx.x / args.nbands;
    const int c = k & 1, K = k >> 1, J0 = band * kOwnSub<M2>;
    const size_t np = (size_t)g.npad;
    const bool has_lo = g.zp || k > 0, has_hi = g.zp || k < g.o - 1;
    if (KIND == OP_CONST && !(has_lo && has_hi)) {   // a Dirichlet plate: r - fix x
#pragma unroll 1
        for (int w = hh; w < 4 * kOwnSub<M2>; w += NH) {
            const int ab = w / kOwnSub<M2>, t = w % kOwnSub<M2>;
            const size_t sl = band_slot(g, ab, c, K, J0 + t, I);
            T acc[3] = {r[sl], r[sl + np], r[sl + 2 * np]};
            const T *xp = static_cast<const T *>(args.xz);
            const T v[3] = {xp[sl], xp[sl + np], xp[sl + 2 * np]};
            matvec_sub(op.cop.fix, v, acc);
            res[sl] = acc[0];
            res[sl + np] = acc[1];
            res[sl + 2 * np] = acc[2];
        }
        return;
    }
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(band_smem);
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&bar_store);
    if ((sbase & 127u) != 0) {
        if (tid == 0) atomicExch(&g_band_err, 2);
        return;
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        const unsigned plane_bytes = (unsigned)(kBandWords<M2> / 3 * sizeof(T));
        mbar_expect_tx(bar, plane_bytes * (1u + has_lo + has_hi));
        const int klo = k == 0 ? g.o - 1 : k - 1, khi = k == g.o - 1 ? 0 : k + 1;
        if (has_lo) stage_plane<T, M2>(xm, g, klo, J0, 0, sbase, bar);
        stage_plane<T, M2>(xm, g, k, J0, 1, sbase, bar);
        if (has_hi) stage_plane<T, M2>(xm, g, khi, J0, 2, sbase, bar);
    }
    if (KIND == OP_PLANE) stage_coef<T>(op.pop, k, cfs, tid, NH * M2);
    const bool ok = mbar_wait(bar, 0, 200000000ull);
    if (!__syncthreads_and(ok)) {
        if (tid == 0) {
            atomicExch(&g_band_err, 1);
            mbar_wait(bar, 0, 200000000ull);
        }
        __syncthreads();
        return;
    }
    T *s = reinterpret_cast<T *>(band_smem);
    if (KIND == OP_PLANE && !(has_lo && has_hi)) {
        constexpr int PW = kBandWords<M2> / 3;
        if (!has_lo)
            for (int w = tid; w < PW; w += NH * M2) s[w] = T(0);
        if (!has_hi)
            for (int w = tid; w < PW; w += NH * M2) s[2 * PW + w] = T(0);
        __syncthreads();
    }
    constexpr int P = kPer<kOwnSub<M2>, NH>;
    const int t0 = hh * P, nv = min(P, kOwnSub<M2> - t0);
    const int ib[3] = {I == 0 ? M2 - 1 : I - 1, I, I == M2 - 1 ? 0 : I + 1};
    // the four colours as the branches of a loop that is not unrolled: the
    // colours share no barrier, and in one straight run the instruction
    // scheduler would start every colour's shared loads at once
#pragma unroll 1
    for (int q = 0; q < 4; q++) {
        switch (q) {
            case 0: band_res_colour<T, M2, KIND, SPARSE, 0, 0, P>(s, ib, op, cfs, t0, nv, g, c, K, J0, I, r, res); break;
            case 1: band_res_colour<T, M2, KIND, SPARSE, 1, 0, P>(s, ib, op, cfs, t0, nv, g, c, K, J0, I, r, res); break;
            case 2: band_res_colour<T, M2, KIND, SPARSE, 0, 1, P>(s, ib, op, cfs, t0, nv, g, c, K, J0, I, r, res); break;
            default: band_res_colour<T, M2, KIND, SPARSE, 1, 1, P>(s, ib, op, cfs, t0, nv, g, c, K, J0, I, r, res);
        }
    }
}

// ------------------------------------------------------------------ host
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// The tensor maps of one colour-blocked field of level g: a 5-d view with
// column I innermost, then colour ab, sub-row J, plane K, component x plane
// parity, and boxes of the whole row of M2 columns, 4 colours and 6, 5 or 1
// sub-rows.  False if the driver does not accept them (the caller then runs
// the colour launches).
template <typename T>
bool make_band_maps(const Geom &g, const T *field, BandMaps &mp) {
    EncodeTiled enc = encoder();
    if (!enc) return false;
    const cuuint64_t e = sizeof(T);
    const cuuint64_t M2 = g.M2, N2 = g.N2, O2 = g.O2, S = g.S;
    const cuuint64_t dims[5] = {M2, 4, N2, O2, 6}, strides[4] = {S * e, M2 * e, M2 * N2 * e, 4 * S * e};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    CUtensorMap *maps[3] = {&mp.full, &mp.less1, &mp.one};
    const cuuint32_t stage = (cuuint32_t)(band_rows(g.M2) / 2 + 2);
    const cuuint32_t rows[3] = {stage, stage - 1, 1};
    for (int i = 0; i < 3; i++) {
        const cuuint32_t box[5] = {(cuuint32_t)M2, 4, rows[i], 1, 1};
        if (enc(maps[i], dt, 5, const_cast<T *>(field), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

bool first_band_use(unsigned long long &devices) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (devices & bit) return false;
    devices |= bit;
    return true;
}

// Threads per column of the residual kernel: two (each thread two of the
// band's four sub-rows, which share each coefficient load; four threads with
// one row each measured slower: level 1 59.5 against 43.9 us).
template <typename T, int M2>
constexpr int kResNH = 2;

template <typename T, int M2, int NH, int KIND, bool SPARSE>
bool launch_band_kn(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    BandMaps min_, mout;
    if (!make_band_maps<T>(g, xin, min_) || !make_band_maps<T>(g, xout, mout)) return false;
    auto kern = gs_band_kernel<T, M2, NH, KIND, SPARSE>;
    const int smem = kBandWords<M2> * (int)sizeof(T);
    static unsigned long long attr_devices = 0;
    if (first_band_use(attr_devices)) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    BandArgs a;
    a.g = g;
    a.nbands = g.n / band_rows(g.M2);
    a.xz = nullptr;
    for (int c = 0; c < 2; c++) {
        const int planes = c == 0 ? (g.o + 1) / 2 : g.o / 2;
        if (planes <= 0) continue;
        a.c = c;
        a.nplanes = planes;
        // the odd launch walks down from where the even one ended, so its
        // first planes (and the even planes they read) are still in L2; the
        // next sweep's even launch starts at the bottom, where this one ends
        a.rev = c;
        kern<<<a.nbands * planes, NH * M2, smem, st>>>(a, op, min_, mout, r, xout);
    }
    return true;
}

// Threads per column of the sweep: in FP32 two on wide levels (64 or 128
// sub-grid columns; four, with twice the warps, measured no faster: 350 vs
// 347 us for two fine sweeps with 8-row bands, 131 vs 126 us on level 1,
// where a thread's rows share each coefficient load) and eight on narrow
// ones, one row per thread: those levels have few CTAs and are bound by the
// latency of each thread's chain (mixed solve 21.99 -> 21.65 ms against four
// on the 16- and 8-column levels, 21.73 -> 21.68 ms on the 32-column one);
// one or two in FP64 (registers).
template <typename T, int M2, int KIND, bool SPARSE>
bool launch_band_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    constexpr int NH = sizeof(T) == 4 ? (M2 >= 64 ? 2 : 8) : (M2 >= 64 ? 1 : 2);
    return launch_band_kn<T, M2, NH, KIND, SPARSE>(op, g, r, xin, xout, st);
}

template <typename T, int KIND, bool SPARSE>
bool launch_band_m(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    switch (g.M2) {
        case 8: return launch_band_k<T, 8, KIND, SPARSE>(op, g, r, xin, xout, st);
        case 16: return launch_band_k<T, 16, KIND, SPARSE>(op, g, r, xin, xout, st);
        case 32: return launch_band_k<T, 32, KIND, SPARSE>(op, g, r, xin, xout, st);
        case 64: return launch_band_k<T, 64, KIND, SPARSE>(op, g, r, xin, xout, st);
        case 128: return launch_band_k<T, 128, KIND, SPARSE>(op, g, r, xin, xout, st);
        default: return false;
    }
}

template <typename T>
bool launch_band_op(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    if (op.kind == OP_CONST) return launch_band_m<T, OP_CONST, false>(op, g, r, xin, xout, st);
    if (op.pop.sparse) return launch_band_m<T, OP_PLANE, true>(op, g, r, xin, xout, st);
    return launch_band_m<T, OP_PLANE, false>(op, g, r, xin, xout, st);
}

}  // namespace

// Where the band sweep runs: the elasticity stencil shared by every interior
// node or a plane-invariant coarse operator, a level periodic in x and y
// with 8, 16, 32, 64 or 128 sub-grid columns (16 .. 256 nodes) and whole
// bands of 8 rows (at least two), an even z extent if z is periodic.  FP32 levels by default;
// STZ_MG_BAND=0 turns it off, STZ_MG_BAND=1 uses it in FP64 too.
template <typename T>
bool gs_band_applies(const LevelOp<T> &op, const Geom &g) {
    int mode = -1;
    if (const char *e = std::getenv("STZ_MG_BAND")) mode = std::atoi(e) != 0;
    if (mode == 0) return false;
    if (mode < 0 && sizeof(T) != 4) return false;
    if (!((op.kind == OP_CONST && op.cop.elastic) || op.kind == OP_PLANE)) return false;
    const int rows = band_rows(g.M2);
    if (!g.xp || !g.yp || (g.m & 1) || g.n % rows != 0 || g.n < 2 * rows) return false;
    if (g.M2 != 8 && g.M2 != 16 && g.M2 != 32 && g.M2 != 64 && g.M2 != 128) return false;
    if (g.zp && (g.o & 1)) return false;
    return true;
}

// One sweep x_in -> x_out; false when the tensor maps cannot be made (the
// caller then sweeps with the colour launches).
template <typename T>
bool launch_gs_sweep_band(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st) {
    return launch_band_op<T>(op, g, r, xin, xout, st);
}

namespace {

template <typename T, int M2, int KIND, bool SPARSE>
bool launch_res_band_k(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, cudaStream_t st) {
    BandMaps xm;
    if (!make_band_maps<T>(g, x, xm)) return false;
    constexpr int NH = kResNH<T, M2>;
    auto kern = residual_band_kernel<T, M2, NH, KIND, SPARSE>;
    const int smem = kBandWords<M2> * (int)sizeof(T);
    static unsigned long long attr_devices = 0;
    if (first_band_use(attr_devices)) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    BandArgs a;
    a.g = g;
    a.nbands = g.n / band_rows(g.M2);
    a.c = 0;
    a.nplanes = g.o;
    a.rev = 0;
    a.xz = x;
    kern<<<a.nbands * g.o, NH * M2, smem, st>>>(a, op, xm, r, res);
    return true;
}

template <typename T, int KIND, bool SPARSE>
bool launch_res_band_m(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, cudaStream_t st) {
    switch (g.M2) {
        case 8: return launch_res_band_k<T, 8, KIND, SPARSE>(op, g, r, x, res, st);
        case 16: return launch_res_band_k<T, 16, KIND, SPARSE>(op, g, r, x, res, st);
        case 32: return launch_res_band_k<T, 32, KIND, SPARSE>(op, g, r, x, res, st);
        case 64: return launch_res_band_k<T, 64, KIND, SPARSE>(op, g, r, x, res, st);
        case 128: return launch_res_band_k<T, 128, KIND, SPARSE>(op, g, r, x, res, st);
        default: return false;
    }
}

template <typename T>
bool launch_res_band_op(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, cudaStream_t st) {
    if (op.kind == OP_CONST) return launch_res_band_m<T, OP_CONST, false>(op, g, r, x, res, st);
    if (op.pop.sparse) return launch_res_band_m<T, OP_PLANE, true>(op, g, r, x, res, st);
    return launch_res_band_m<T, OP_PLANE, false>(op, g, r, x, res, st);
}

}  // namespace

// res = r - A x by the band kernel on the plane-invariant levels the band
// sweep serves; false (the caller falls back) elsewhere or when the tensor
// maps cannot be made.  On the shared-stencil fine level the marching tiled
// residual is faster (each plane staged once instead of three times: 169 vs
// 232 us at 256x256x257), so the band residual runs there only with
// STZ_MG_BAND_RES=1; STZ_MG_BAND_RES=0 turns it off everywhere.
template <typename T>
bool launch_residual_band(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, cudaStream_t st) {
    if (!gs_band_applies(op, g)) return false;
    int mode = -1;
    if (const char *e = std::getenv("STZ_MG_BAND_RES")) mode = std::atoi(e) != 0;
    if (mode == 0 || (mode < 0 && op.kind != OP_PLANE)) return false;
    return launch_res_band_op<T>(op, g, r, x, res, st);
}
template bool launch_residual_band<float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *,
                                          cudaStream_t);
template bool launch_residual_band<double>(const LevelOp<double> &, const Geom &, const double *, const double *,
                                           double *, cudaStream_t);

// Whether the tensor maps of the band sweep can be made for this level.
template <typename T>
bool gs_band_ready(const Geom &g, const T *field) {
    BandMaps mp;
    return make_band_maps<T>(g, field, mp);
}
template bool gs_band_ready<float>(const Geom &, const float *);
template bool gs_band_ready<double>(const Geom &, const double *);

// 1 if a band CTA gave up waiting for its copies since the last call, 2 if
// one found its shared memory misaligned for TMA (and clears the record);
// -1 if the record cannot be read.
int band_take_error(cudaStream_t st) {
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_band_err, sizeof v, 0, cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
    if (cudaMemcpyToSymbolAsync(g_band_err, &z, sizeof z, 0, cudaMemcpyHostToDevice, st) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    return v;
}

template bool gs_band_applies<float>(const LevelOp<float> &, const Geom &);
template bool gs_band_applies<double>(const LevelOp<double> &, const Geom &);
template bool launch_gs_sweep_band<float>(const LevelOp<float> &, const Geom &, const float *, const float *, float *,
                                          cudaStream_t);
template bool launch_gs_sweep_band<double>(const LevelOp<double> &, const Geom &, const double *, const double *,
                                           double *, cudaStream_t);

}  // namespace stzmg
