// Galerkin (RAT) coarse operators and their box bounds.
//
// Reference: region::fill_rat_bounds / compute_rats (mg_3d_template/
// region.cc:1848-1966) with rat_bound_*/rat_fill_* (2275-2466), A_red
// (2485-2538), A_add (2545-2578), grid_map/igrid_map (2587-2647) and the
// driver multigrid::compute_rats (multigrid.cc:330-344).
//
// The reference builds A_c = (1/8) P^T A P by scattering, for every fine row
// f, the row of A P (A_red) into the rows of f's coarse parents.  Here one
// thread owns one coarse entry (coarse node I, offset J - I) and gathers
//     A_c[I,J] = sum_{f child of I} sum_{g child of J, g in box(f)}
//                (1/8 A[f,g]) w_P(g,J) w_P(f,I).
// All weights are powers of two, so every term is bit-identical to the
// reference's; only the order of the additions differs.  Entries are kept in
// the unwrapped offset convention of the reference's boxes (on a periodic
// dimension of size 2 or 1, offsets -1 and +1 are separate entries).
#include "launch.h"
#include "ops.cuh"

namespace stzmg {

constexpr int kRB = 128;

// Children of coarse index I along one dimension: fine range [lo, hi) and
// the fine index that coincides with I (igrid_map without the cropping);
// returns false when I is outside a non-periodic grid.
__device__ inline bool children(int I, int mf, int mc, int prd, int &lo, int &hi, int &c) {
    if (!prd && (I < 0 || I >= mc)) return false;
    int j = 2 * I;
    if (prd) { lo = j - 1; hi = j + 2; c = j; return true; }
    if (mf & 1) { lo = j == 0 ? 0 : j - 1; hi = j == mf - 1 ? mf : j + 2; c = j; }
    else if (j == mf) { lo = mf - 1; hi = mf; c = mf - 1; }
    else { lo = j == 0 ? 0 : j - 1; hi = j == mf - 2 ? mf - 1 : j + 2; c = j; }
    return true;
}

__device__ inline int wrapd(int a, int len) {
    a %= len;
    return a < 0 ? a + len : a;
}

// Block (d) of fine row f for the three operator kinds.
template <int KIND>
__device__ inline void fine_block(const LevelOp<double> &op, const Geom &g, int fs, bool interior,
                                  const double *mu_nb, const double *lam_nb, const LameRow<double> &L, int b,
                                  double *a) {
#pragma unroll
    for (int e = 0; e < 9; e++) a[e] = 0.0;
    if (KIND == OP_CONST) {
        const double *src = interior ? op.cop.a[b] : op.cop.fix;
        for (int e = 0; e < 9; e++) a[e] = src[e];
    } else if (KIND == OP_LAME) {
        if (!interior) {
            double f = lame_fix(op.lop, fs);
            a[0] = a[4] = a[8] = f;
            return;
        }
        int dx = bdx(b), dy = bdy(b), dz = bdz(b), nz = nnz_axes(b);
        if (nz == 0) {
            a[0] = L.centre[0]; a[4] = L.centre[1]; a[8] = L.centre[2];
        } else if (nz == 1) {
            int f = dx ? (dx > 0 ? 1 : 0) : dy ? (dy > 0 ? 3 : 2) : (dz > 0 ? 5 : 4);
            a[0] = L.face[f][0]; a[4] = L.face[f][1]; a[8] = L.face[f][2];
        } else if (nz == 2) {
            int d[3] = {dx, dy, dz};
            int r = dz == 0 ? 0 : (dy == 0 ? 0 : 1), c = dz == 0 ? 1 : 2;
            int sr = d[r], sc = d[c];
            const double ie = op.lop.iedge[r + c - 1], sgn = (double)(sr * sc);
            const double lam_r = lam_nb[2 * r + (sr > 0)], mu_r = mu_nb[2 * r + (sr > 0)];
            const double lam_c = lam_nb[2 * c + (sc > 0)], mu_c = mu_nb[2 * c + (sc > 0)];
            a[3 * r + c] = -op.lop.dt * ((sgn * (lam_r + mu_c)) * ie);
            a[3 * c + r] = -op.lop.dt * ((sgn * (lam_c + mu_r)) * ie);
        }
    } else if (KIND == OP_PLANE) {
        const int k = fs;   // callers pass the plane index for plane operators
        for (int e = 0; e < 9; e++) a[e] = op.pop.coef[(9 * b + e) * op.pop.O + k];
    } else {
        const size_t np = (size_t)g.npad;
        for (int e = 0; e < 9; e++) a[e] = op.dop.coef[(size_t)(9 * b + e) * np + fs];
    }
}

template <int KIND, bool OUT_PLANE>
__global__ void __launch_bounds__(kRB) rat_kernel(Geom gf, Geom gc, const __grid_constant__ LevelOp<double> op,
                                                  double *__restrict__ coef_c) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x, off = blockIdx.y;
    int I, J, K;
    if (OUT_PLANE) {
        // one coarse node per plane: the column i = j = 0
        if (p >= gc.o) return;
        I = 0; J = 0; K = p;
    } else if (p >= gc.npad || !slot_node(gc, p, I, J, K)) {
        return;
    }
    const int ox = bdx(off), oy = bdy(off), oz = bdz(off);
    const int TI = I + ox, TJ = J + oy, TK = K + oz;   // target coarse node (unwrapped)
    int tlo[3], thi[3], tc[3];
    if (!children(TI, gf.m, gc.m, gf.xp, tlo[0], thi[0], tc[0]) ||
        !children(TJ, gf.n, gc.n, gf.yp, tlo[1], thi[1], tc[1]) ||
        !children(TK, gf.o, gc.o, gf.zp, tlo[2], thi[2], tc[2]))
        return;   // entry stays zero
    int slo[3], shi[3], sc[3];
    children(I, gf.m, gc.m, gf.xp, slo[0], shi[0], sc[0]);
    children(J, gf.n, gc.n, gf.yp, slo[1], shi[1], sc[1]);
    children(K, gf.o, gc.o, gf.zp, slo[2], shi[2], sc[2]);
    double acc[9];
#pragma unroll
    for (int e = 0; e < 9; e++) acc[e] = 0.0;
    for (int fz = slo[2]; fz < shi[2]; fz++) {
        const double wfz = fz == sc[2] ? 1.0 : 0.5;
        const int fzw = wrapd(fz, gf.o);
        for (int fy = slo[1]; fy < shi[1]; fy++) {
            const double wfy = fy == sc[1] ? wfz : 0.5 * wfz;
            const int fyw = wrapd(fy, gf.n);
            for (int fx = slo[0]; fx < shi[0]; fx++) {
                const double wf = fx == sc[0] ? wfy : 0.5 * wfy;
                const int fxw = wrapd(fx, gf.m);
                const int fs = KIND == OP_PLANE ? fzw : slot(gf, fxw, fyw, fzw);
                const bool interior = (KIND == OP_DENSE || KIND == OP_PLANE) ? true : is_interior(gf, fxw, fyw, fzw);
                // box of f: [-1,1]^3 for interior rows (and every dense row), centre only otherwise
                const int r0 = interior ? -1 : 0, r1 = interior ? 1 : 0;
                LameRow<double> L;
                double mu_nb[6], lam_nb[6];
                if (KIND == OP_LAME && interior) {
                    NbrOffsets nb = nbr_offsets(gf, fxw, fyw, fzw);
                    lame_faces(op.lop, gf, nb, fs, L, mu_nb, lam_nb);
                }
                for (int dz = r0; dz <= r1; dz++) {
                    const int gz = fz + dz;
                    if (gz < tlo[2] || gz >= thi[2]) continue;
                    const double wgz = gz == tc[2] ? 1.0 : 0.5;
                    for (int dy = r0; dy <= r1; dy++) {
                        const int gy = fy + dy;
                        if (gy < tlo[1] || gy >= thi[1]) continue;
                        const double wgy = gy == tc[1] ? wgz : 0.5 * wgz;
                        for (int dx = r0; dx <= r1; dx++) {
                            const int gx = fx + dx;
                            if (gx < tlo[0] || gx >= thi[0]) continue;
                            const double wg = gx == tc[0] ? wgy : 0.5 * wgy;
                            const int b = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                            double a[9];
                            fine_block<KIND>(op, gf, fs, interior, mu_nb, lam_nb, L, b, a);
#pragma unroll
                            for (int e = 0; e < 9; e++) acc[e] += ((0.125 * a[e]) * wg) * wf;
                        }
                    }
                }
            }
        }
    }
    const size_t np = OUT_PLANE ? (size_t)gc.o : (size_t)gc.npad;
#pragma unroll
    for (int e = 0; e < 9; e++) coef_c[(size_t)(9 * off + e) * np + p] = acc[e];
}

template <typename T>
__global__ void plane_dinv_kernel(int O, const T *__restrict__ coef, T *__restrict__ dinv, int *bad) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= O) return;
    T a[9], inv[9];
    for (int e = 0; e < 9; e++) a[e] = coef[(9 * 13 + e) * O + k];
    if (!inverse3(a, inv)) atomicExch(bad, 1);
    for (int e = 0; e < 9; e++) dinv[e * O + k] = inv[e];
}

template <typename T>
__global__ void dinv_kernel(Geom g, const T *__restrict__ coef, T *__restrict__ dinv, int *bad) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (p >= g.npad) return;
    const size_t np = (size_t)g.npad;
    T a[9], inv[9];
    if (!slot_node(g, p, i, j, k)) {
        for (int e = 0; e < 9; e++) dinv[(size_t)e * np + p] = T(0);
        return;
    }
    for (int e = 0; e < 9; e++) a[e] = coef[(size_t)(9 * 13 + e) * np + p];
    bool ok = inverse3(a, inv);
    if (!ok) atomicExch(bad, 1);
    for (int e = 0; e < 9; e++) dinv[(size_t)e * np + p] = inv[e];
}

// grid_map (region.cc:2587-2604), with the reference's range checks
// reported through *bad.
__device__ inline void grid_map(int &lo, int &hi, int ma, int prd, int *bad) {
    if (prd) {
        if (lo < -ma || lo > ma - 1 || hi < 1 || hi > 2 * ma) atomicExch(bad, 2);
        lo = lo < 0 ? (lo - (ma & 1 ? 2 : 1)) / 2 : lo >> 1;
        hi = (hi + ((ma & 1) && hi > ma ? 1 : 2)) >> 1;
    } else {
        if (lo < 0 || lo > ma - 1 || hi < 1 || hi > ma) atomicExch(bad, 2);
        lo = (!(ma & 1) && lo == ma - 1 ? lo + 1 : lo) >> 1;
        hi = (hi + 2) >> 1;
    }
}

__global__ void top_bounds_kernel(Geom g, int *S) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, i, j, k;
    if (p >= g.npad) return;
    bool used = slot_node(g, p, i, j, k);
    bool in = used && is_interior(g, i, j, k);
    for (int d = 0; d < 3; d++) {
        S[(size_t)(2 * d) * g.npad + p] = in ? -1 : 0;
        S[(size_t)(2 * d + 1) * g.npad + p] = in ? 2 : 1;
    }
}

// Coarse bounds: union over the children f of I of grid_map(box(f)) - I
// (fill_rat_bounds, region.cc:1848-1905).  Bounds are stored SoA, 6 x npad.
__global__ void rat_bounds_kernel(Geom gf, const int *__restrict__ Sf, Geom gc, int *__restrict__ Sc, int *bad) {
    int p = blockIdx.x * blockDim.x + threadIdx.x, I, J, K;
    if (p >= gc.npad) return;
    int box[6] = {0, 1, 0, 1, 0, 1};
    if (slot_node(gc, p, I, J, K)) {
        int lo[3], hi[3], c[3];
        children(I, gf.m, gc.m, gf.xp, lo[0], hi[0], c[0]);
        children(J, gf.n, gc.n, gf.yp, lo[1], hi[1], c[1]);
        children(K, gf.o, gc.o, gf.zp, lo[2], hi[2], c[2]);
        const int C[3] = {I, J, K};
        const int dims[3] = {gf.m, gf.n, gf.o}, prd[3] = {gf.xp, gf.yp, gf.zp};
        for (int fz = lo[2]; fz < hi[2]; fz++)
            for (int fy = lo[1]; fy < hi[1]; fy++)
                for (int fx = lo[0]; fx < hi[0]; fx++) {
                    const int f[3] = {fx, fy, fz};
                    const int fs = slot(gf, wrapd(fx, gf.m), wrapd(fy, gf.n), wrapd(fz, gf.o));
                    for (int d = 0; d < 3; d++) {
                        int l = f[d] + Sf[(size_t)(2 * d) * gf.npad + fs];
                        int h = f[d] + Sf[(size_t)(2 * d + 1) * gf.npad + fs];
                        // the reference maps boxes in the parent's global frame of the
                        // unwrapped fine index; wrapping f by whole periods shifts the
                        // coarse box by whole coarse periods, so map the wrapped box and
                        // shift back
                        int shift = 0;
                        if (prd[d]) {
                            int fw = wrapd(f[d], dims[d]);
                            shift = f[d] - fw;   // multiple of the fine period
                            l -= shift; h -= shift;
                        }
                        grid_map(l, h, dims[d], prd[d], bad);
                        if (prd[d] && shift) {
                            const int cper = d == 0 ? gc.m : d == 1 ? gc.n : gc.o;
                            l += (shift / dims[d]) * cper;
                            h += (shift / dims[d]) * cper;
                        }
                        if (l - C[d] < box[2 * d]) box[2 * d] = l - C[d];
                        if (h - C[d] > box[2 * d + 1]) box[2 * d + 1] = h - C[d];
                    }
                }
    }
    for (int e = 0; e < 6; e++) Sc[(size_t)e * gc.npad + p] = box[e];
}

__global__ void bounds_cb_to_nat_kernel(Geom g, const int *__restrict__ S, int *__restrict__ nat) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long npts = (long)g.m * g.n * g.o;
    if (t >= npts) return;
    int i = t % g.m, j = (t / g.m) % g.n, k = t / ((long)g.m * g.n);
    int s = slot(g, i, j, k);
    for (int e = 0; e < 6; e++) nat[6 * t + e] = S[(size_t)e * g.npad + s];
}

// Dense 27-block form of a top-level operator (for export and checks).
template <int KIND>
__global__ void expand_dense_kernel(Geom g, const __grid_constant__ LevelOp<double> op, double *__restrict__ coef) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    int i, j, k;
    if (p >= g.npad || !slot_node(g, p, i, j, k)) return;
    const bool interior = (KIND == OP_DENSE || KIND == OP_PLANE) ? true : is_interior(g, i, j, k);
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (interior || b == 13) {
        LameRow<double> L;
        double mu_nb[6], lam_nb[6];
        if (KIND == OP_LAME && interior) {
            NbrOffsets nb = nbr_offsets(g, i, j, k);
            lame_faces(op.lop, g, nb, p, L, mu_nb, lam_nb);
        }
        fine_block<KIND>(op, g, KIND == OP_PLANE ? k : p, interior, mu_nb, lam_nb, L, b, a);
    }
    const size_t np = (size_t)g.npad;
    for (int e = 0; e < 9; e++) coef[(size_t)(9 * b + e) * np + p] = a[e];
}

void launch_expand_dense(const LevelOp<double> &op, const Geom &g, double *coef, cudaStream_t st) {
    cudaMemsetAsync(coef, 0, sizeof(double) * 243 * (size_t)g.npad, st);
    dim3 grid((g.npad + kRB - 1) / kRB, 27);
    switch (op.kind) {
        case OP_CONST: expand_dense_kernel<OP_CONST><<<grid, kRB, 0, st>>>(g, op, coef); break;
        case OP_LAME: expand_dense_kernel<OP_LAME><<<grid, kRB, 0, st>>>(g, op, coef); break;
        case OP_PLANE: expand_dense_kernel<OP_PLANE><<<grid, kRB, 0, st>>>(g, op, coef); break;
        default: expand_dense_kernel<OP_DENSE><<<grid, kRB, 0, st>>>(g, op, coef); break;
    }
}

void launch_rat(const LevelOp<double> &fine, const Geom &gf, const Geom &gc, double *coef_c, bool plane,
                cudaStream_t st) {
    if (plane) {
        cudaMemsetAsync(coef_c, 0, sizeof(double) * 243 * (size_t)gc.o, st);
        dim3 grid((gc.o + kRB - 1) / kRB, 27);
        if (fine.kind == OP_CONST) rat_kernel<OP_CONST, true><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c);
        else rat_kernel<OP_PLANE, true><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c);
        return;
    }
    cudaMemsetAsync(coef_c, 0, sizeof(double) * 243 * (size_t)gc.npad, st);
    dim3 grid((gc.npad + kRB - 1) / kRB, 27);
    switch (fine.kind) {
        case OP_CONST: rat_kernel<OP_CONST, false><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c); break;
        case OP_LAME: rat_kernel<OP_LAME, false><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c); break;
        case OP_PLANE: rat_kernel<OP_PLANE, false><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c); break;
        default: rat_kernel<OP_DENSE, false><<<grid, kRB, 0, st>>>(gf, gc, fine, coef_c); break;
    }
}

template <typename T>
void launch_plane_dinv(int O, const T *coef, T *dinv, int *bad, cudaStream_t st) {
    plane_dinv_kernel<T><<<(O + 127) / 128, 128, 0, st>>>(O, coef, dinv, bad);
}
template void launch_plane_dinv<float>(int, const float *, float *, int *, cudaStream_t);
template void launch_plane_dinv<double>(int, const double *, double *, int *, cudaStream_t);

template <typename T>
void launch_dense_dinv(const Geom &g, const T *coef, T *dinv, int *bad, cudaStream_t st) {
    dinv_kernel<T><<<(g.npad + 255) / 256, 256, 0, st>>>(g, coef, dinv, bad);
}
template void launch_dense_dinv<float>(const Geom &, const float *, float *, int *, cudaStream_t);
template void launch_dense_dinv<double>(const Geom &, const double *, double *, int *, cudaStream_t);

void launch_top_bounds(const Geom &g, int *S, cudaStream_t st) {
    top_bounds_kernel<<<(g.npad + 255) / 256, 256, 0, st>>>(g, S);
}
void launch_rat_bounds(const Geom &gf, const int *fine_S, const Geom &gc, int *S_c, int *bad, cudaStream_t st) {
    rat_bounds_kernel<<<(gc.npad + 255) / 256, 256, 0, st>>>(gf, fine_S, gc, S_c, bad);
}
void launch_bounds_cb_to_nat(const Geom &g, const int *S, int *nat, cudaStream_t st) {
    bounds_cb_to_nat_kernel<<<(int)(((long)g.m * g.n * g.o + 255) / 256), 256, 0, st>>>(g, S, nat);
}

}  // namespace stzmg
