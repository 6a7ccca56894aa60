// Top-level residual of the mixed solver in double-float arithmetic.
//
// The defect-correction step needs r = b - A x of the FP64 solution, rounded
// to FP32 for the next correction solve, and |r|^2 for the stopping test.
// Near convergence r is ten digits below the terms of A x, so FP32 alone
// cannot form it; FP64 can, but GB300's FP64 pipe makes the pass take 2.2 ms
// on the 256x256x257 problem, 12 % of the solve.  Here every FP64 value is
// carried as a pair of floats (hi + lo, about 47 significant bits):
//
//  * x is split once per residual into float pairs (split_kernel; one 8-byte
//    load per neighbour component), b per node as it is read, the shared
//    stencil on the host;
//  * a product a x = (ah + al)(xh + xl) is ah*xh exactly -- its rounded value
//    p and its error fma(ah, xh, -p) (Dekker, "A floating-point technique for
//    extending the available precision", 1971) -- plus the two cross terms
//    ah*xl + al*xh (the al*xl term, 2^-48 of the product, is dropped; a
//    stencil exact in FP32 has al = 0 and a kernel without the al terms);
//  * the running sum keeps its high part exact with Knuth's two-sum (The Art
//    of Computer Programming vol. 2, 4.2.2) and gathers every rounding error
//    and small term in a float low part.
//
// The result carries an absolute error of a few 2^-47 of sum |a x| over the
// row -- on the benchmark problem sum |a x| is about 6 |b|, so relative
// residuals near 1e-13 stay resolved, three orders of magnitude below the
// usual 1e-10 tolerance -- and uses only the FP32 pipe.  The squares for |r|^2 are formed in FP32 from r scaled by a
// power of two near 1/rms(b), so they stay in FP32's range while the solve
// converges, and each warp's sum is accumulated in FP64.
//
// Values are split within FP32's normal range: |x| below 2^-126 counts as 0
// and |x| of 2^128 or more as infinite -- the FP32 correction solve needs
// that range in any case.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "launch.h"
#include "ops.cuh"

namespace stzmg {

namespace {

constexpr int kDfThreads = 256;

// The shared stencil and the Dirichlet block with every FP64 entry split
// into hi + lo floats.
struct DfConst {
    float ah[27][9], al[27][9];
    float fh[9], fl[9];
};

__host__ __device__ inline float bits_to_float(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}

// x = hi + lo: hi is x with its mantissa cut to FP32's 24 bits (rounding
// toward zero), lo the remaining 29 bits rounded to a float, so hi + lo is
// within 2^-48 |x| of x for 2^-78 <= |x| < 2^128 (below, lo meets FP32's
// subnormal range; the absolute error stays under 2^-149).  Integer
// operations and one integer-to-float conversion: no FP64 arithmetic.
__host__ __device__ inline void split_double(double x, float &hi, float &lo) {
    unsigned long long u;
#ifdef __CUDA_ARCH__
    u = (unsigned long long)__double_as_longlong(x);
#else
    std::memcpy(&u, &x, sizeof u);
#endif
    const unsigned uh = (unsigned)(u >> 32), ul = (unsigned)u;
    const unsigned sign = uh & 0x80000000u;
    const int e = (int)((uh >> 20) & 0x7FFu) - 1023;
    if (e < -126) {   // zero, FP64 subnormal, or below FP32's normal range
        hi = lo = bits_to_float(sign);
        return;
    }
    if (e > 127) {   // beyond FP32's range, infinite or NaN: hi infinite
        hi = bits_to_float(sign | 0x7F800000u);
        lo = 0.0f;
        return;
    }
    // the implicit bit and the top 23 of the 52 mantissa bits
    hi = bits_to_float(sign | ((unsigned)(e + 127) << 23) | ((uh & 0xFFFFFu) << 3) | (ul >> 29));
    // the remaining 29 bits are worth 2^(e-52) each: rounded to a float
    // (24 bits), then scaled by 2^(e-52) in two exact steps
    const unsigned m = ul & 0x1FFFFFFFu;
#ifdef __CUDA_ARCH__
    const float f = __uint2float_rn(m);
#else
    const float f = (float)m;
#endif
    const int s = e - 52, s1 = s / 2, s2 = s - s1;   // each in [-89, 38]
    const float v = (f * bits_to_float((unsigned)(s1 + 127) << 23)) * bits_to_float((unsigned)(s2 + 127) << 23);
    lo = sign ? -v : v;
}

// (sh, sl) -= (ah + al)(xh + xl); AL false: al is 0
template <bool AL>
__device__ __forceinline__ void df_sub_prod(float &sh, float &sl, float ah, float al, float xh, float xl) {
    const float p = __fmul_rn(ah, xh);
    const float ep = __fmaf_rn(ah, xh, -p);   // ah*xh = p + ep exactly
    const float s = __fsub_rn(sh, p);          // two-sum of sh and -p
    const float bv = __fsub_rn(s, sh);
    const float err = __fsub_rn(__fsub_rn(sh, __fsub_rn(s, bv)), __fadd_rn(p, bv));
    sh = s;
    const float cross = AL ? __fmaf_rn(ah, xl, __fmul_rn(al, xh)) : __fmul_rn(ah, xl);
    sl = __fsub_rn(__fadd_rn(sl, __fsub_rn(err, ep)), cross);
}

// (sh, sl) = (ah, al)-free sum of two pairs: (xh1 + xl1) + (xh2 + xl2) with
// the high parts' sum exact (two-sum) and every rounding error in the low part.
__device__ __forceinline__ void df_add(float xh1, float xl1, float xh2, float xl2, float &sh, float &sl) {
    const float s = __fadd_rn(xh1, xh2);
    const float bv = __fsub_rn(s, xh1);
    const float err = __fadd_rn(__fsub_rn(xh1, __fsub_rn(s, bv)), __fsub_rn(xh2, bv));
    sh = s;
    sl = __fadd_rn(__fadd_rn(xl1, xl2), err);
}

// xs = x split into pairs; with e non-null x += e first (the defect
// correction's update, add_correction_kernel's arithmetic) and written back.
__global__ void split_kernel(double *__restrict__ x, const float *__restrict__ e, float2 *__restrict__ xs,
                             size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        double xv = x[t];
        if (e) {
            xv += (double)e[t];
            x[t] = xv;
        }
        float2 v;
        split_double(xv, v.x, v.y);
        xs[t] = v;
    }
}

// r32 = b - A x over every slot of the top level (unused slots get 0) and,
// per block, the FP64 sum of (scale * r32)^2 into partial; xs: x as
// (hi, lo) pairs.  Thread layout of residual_kernel: block (32, 8), lanes
// along x, threadIdx.y the colour.
template <bool ELASTIC, bool AL, bool PAIRED>
__global__ void __launch_bounds__(kDfThreads) residual_df_kernel(Geom g, const __grid_constant__ DfConst op,
                                                                 int centre_diag, const double *__restrict__ b,
                                                                 const float2 *__restrict__ xs,
                                                                 float *__restrict__ r32, float scale,
                                                                 double *__restrict__ partial) {
    const int q = threadIdx.y;
    const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y, K = blockIdx.z;
    const int a = q & 1, bq = (q >> 1) & 1, c = q >> 2;
    const int i = 2 * I + a, j = 2 * J + bq, k = 2 * K + c;
    const size_t np = (size_t)g.npad;
    float sq = 0.0f;
    if (I < g.M2) {
        const int p = q * g.S + (K * g.N2 + J) * g.M2 + I;
        float out[3] = {0.0f, 0.0f, 0.0f};
        if (i < g.m && j < g.n && k < g.o) {
            float sh[3], sl[3];
#pragma unroll
            for (int cc = 0; cc < 3; cc++) split_double(b[p + cc * np], sh[cc], sl[cc]);
            if (PAIRED && is_interior(g, i, j, k)) {
                // blocks d and -d carry the same coefficients: one product per
                // pair, of the neighbours' double-float sum
                const NbrOffsets nb = nbr_offsets_sub(g, I, J, K, a, bq, c);
#pragma unroll
                for (int blk = 0; blk < 27; blk++) {
                    if (blk > 13 || (ELASTIC && nnz_axes(blk) == 3)) continue;
                    const int mblk = 26 - blk;
                    const int s0 = nb.ox[bdx(blk) + 1] + nb.oy[bdy(blk) + 1] + nb.oz[bdz(blk) + 1];
                    const int s1 = nb.ox[bdx(mblk) + 1] + nb.oy[bdy(mblk) + 1] + nb.oz[bdz(mblk) + 1];
                    float vh[3], vl[3];
#pragma unroll
                    for (int cc = 0; cc < 3; cc++) {
                        bool used = !ELASTIC || blk == 13;
#pragma unroll
                        for (int rr = 0; rr < 3; rr++) used = used || elastic_entry(blk, 3 * rr + cc);
                        if (!used) {
                            vh[cc] = vl[cc] = 0.0f;
                        } else if (blk == 13) {
                            const float2 v = xs[s0 + cc * np];
                            vh[cc] = v.x;
                            vl[cc] = v.y;
                        } else {
                            const float2 v0 = xs[s0 + cc * np], v1 = xs[s1 + cc * np];
                            df_add(v0.x, v0.y, v1.x, v1.y, vh[cc], vl[cc]);
                        }
                    }
#pragma unroll
                    for (int e = 0; e < 9; e++) {
                        if (ELASTIC && blk != 13 && !elastic_entry(blk, e)) continue;
                        if (blk == 13 && centre_diag && e % 4 != 0) continue;   // warp-uniform
                        if (!ELASTIC && op.ah[blk][e] == 0.0f) continue;      // warp-uniform
                        df_sub_prod<AL>(sh[e / 3], sl[e / 3], op.ah[blk][e], op.al[blk][e], vh[e % 3], vl[e % 3]);
                    }
                }
            } else if (is_interior(g, i, j, k)) {
                const NbrOffsets nb = nbr_offsets_sub(g, I, J, K, a, bq, c);
#pragma unroll
                for (int blk = 0; blk < 27; blk++) {
                    if (ELASTIC && nnz_axes(blk) == 3) continue;
                    const int s = nb.ox[bdx(blk) + 1] + nb.oy[bdy(blk) + 1] + nb.oz[bdz(blk) + 1];
                    float vh[3], vl[3];
#pragma unroll
                    for (int cc = 0; cc < 3; cc++) {
                        bool used = !ELASTIC || blk == 13;
#pragma unroll
                        for (int rr = 0; rr < 3; rr++) used = used || elastic_entry(blk, 3 * rr + cc);
                        const float2 v = used ? xs[s + cc * np] : make_float2(0.0f, 0.0f);
                        vh[cc] = v.x;
                        vl[cc] = v.y;
                    }
#pragma unroll
                    for (int e = 0; e < 9; e++) {
                        if (ELASTIC && blk != 13 && !elastic_entry(blk, e)) continue;
                        if (blk == 13 && centre_diag && e % 4 != 0) continue;   // warp-uniform
                        if (!ELASTIC && op.ah[blk][e] == 0.0f) continue;      // warp-uniform
                        df_sub_prod<AL>(sh[e / 3], sl[e / 3], op.ah[blk][e], op.al[blk][e], vh[e % 3], vl[e % 3]);
                    }
                }
            } else {
                float vh[3], vl[3];
#pragma unroll
                for (int cc = 0; cc < 3; cc++) {
                    const float2 v = xs[p + cc * np];
                    vh[cc] = v.x;
                    vl[cc] = v.y;
                }
#pragma unroll
                for (int e = 0; e < 9; e++)
                    df_sub_prod<AL>(sh[e / 3], sl[e / 3], op.fh[e], op.fl[e], vh[e % 3], vl[e % 3]);
            }
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                out[cc] = __fadd_rn(sh[cc], sl[cc]);
                const float v = out[cc] * scale;
                sq = __fmaf_rn(v, v, sq);
            }
        }
#pragma unroll
        for (int cc = 0; cc < 3; cc++) r32[p + cc * np] = out[cc];
    }
    // per warp in FP32 (at most 96 squares), across the block in FP64
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
    __shared__ double red[kDfThreads / 32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if ((tid & 31) == 0) red[tid >> 5] = (double)sq;
    __syncthreads();
    if (tid == 0) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < kDfThreads / 32; w++) v += red[w];
        partial[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = v;
    }
}

// The stencil split into float pairs; *exact: every low half is 0.
DfConst split_stencil(const ConstOp<double> &op, bool *exact) {
    DfConst d;
    *exact = true;
    for (int blk = 0; blk < 27; blk++)
        for (int e = 0; e < 9; e++) {
            split_double(op.a[blk][e], d.ah[blk][e], d.al[blk][e]);
            *exact = *exact && d.al[blk][e] == 0.0f;
        }
    for (int e = 0; e < 9; e++) {
        split_double(op.fix[e], d.fh[e], d.fl[e]);
        *exact = *exact && d.fl[e] == 0.0f;
    }
    return d;
}

template <bool ELASTIC, bool AL>
void launch_df(const Geom &g, const DfConst &d, bool paired, int centre_diag, const double *b, const float2 *xs,
               float *r32, float scale, double *partial, cudaStream_t st) {
    const dim3 blocks((g.M2 + 31) / 32, g.N2, g.O2), blk(32, 8);
    if (paired)
        residual_df_kernel<ELASTIC, AL, true><<<blocks, blk, 0, st>>>(g, d, centre_diag, b, xs, r32, scale, partial);
    else
        residual_df_kernel<ELASTIC, AL, false><<<blocks, blk, 0, st>>>(g, d, centre_diag, b, xs, r32, scale, partial);
}

// Whether every block d of the stencil equals block -d (a symmetric shared
// stencil whose blocks are symmetric, as the elasticity stencil's are):
// then the residual forms one product per pair of opposite neighbours.
// STZ_MG_DF_PAIRS=0 turns the pairing off.
bool stencil_paired(const ConstOp<double> &op) {
    if (const char *e = std::getenv("STZ_MG_DF_PAIRS"))
        if (std::atoi(e) == 0) return false;
    for (int blk = 0; blk < 13; blk++)
        for (int e = 0; e < 9; e++)
            if (op.a[blk][e] != op.a[26 - blk][e]) return false;
    return true;
}

}  // namespace

// The double-float residual serves shared-stencil top levels; STZ_MG_DF=0
// turns it off (the FP64 residual kernel then runs).
bool residual_df_applies(const LevelOp<double> &op) {
    if (const char *e = std::getenv("STZ_MG_DF"))
        if (std::atoi(e) == 0) return false;
    return op.kind == OP_CONST;
}

// A power of two near 1 / rms of a field with sum of squares bsq over n
// values (1 for a zero field).
double df_norm_scale(double bsq, size_t n) {
    if (!(bsq > 0) || n == 0) return 1.0;
    const double rms = std::sqrt(bsq / (double)n);
    const int e = std::ilogb(rms);
    return std::ldexp(1.0, -(e < -120 ? -120 : (e > 120 ? 120 : e)));   // a normal float
}

void launch_residual_df(const LevelOp<double> &op, const Geom &g, const double *b, double *x, const float *corr,
                        float2 *xs, float *r32, double scale, double *partial, double *out, cudaStream_t st) {
    const size_t n = 3 * (size_t)g.npad;
    const unsigned sb = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32);
    split_kernel<<<sb, 256, 0, st>>>(x, corr, xs, n);
    bool exact = false;
    const DfConst d = split_stencil(op.cop, &exact);
    const int cd = op.cop.centre_diag;
    const float sc = (float)scale;
    const bool pr = stencil_paired(op.cop);
    if (op.cop.elastic) {
        if (exact) launch_df<true, false>(g, d, pr, cd, b, xs, r32, sc, partial, st);
        else launch_df<true, true>(g, d, pr, cd, b, xs, r32, sc, partial, st);
    } else {
        if (exact) launch_df<false, false>(g, d, pr, cd, b, xs, r32, sc, partial, st);
        else launch_df<false, true>(g, d, pr, cd, b, xs, r32, sc, partial, st);
    }
    if (out) launch_sum_partials(partial, residual_blocks(g), out, st);
}

}  // namespace stzmg
