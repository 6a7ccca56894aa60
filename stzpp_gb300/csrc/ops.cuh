// Row evaluation of the three operator kinds: acc -= sum_{blocks} A x over a
// node's 3x3x3 box, with or without the centre block, plus the centre solve.
// Reference: region::gauss_seidel (mg_3d_template/region.cc:1557-1762) and
// region::residual (region.cc:1008-1055); the constant stencil is the one of
// shear_sim_3d::set_up_stencil_base (src/shear_sim_3d.cpp:215-331).
#pragma once

#include "common.cuh"

namespace stzmg {

// Offsets (dx,dy,dz) of block b.
__host__ __device__ constexpr int bdx(int b) { return b % 3 - 1; }
__host__ __device__ constexpr int bdy(int b) { return (b / 3) % 3 - 1; }
__host__ __device__ constexpr int bdz(int b) { return b / 9 - 1; }
__host__ __device__ constexpr int nnz_axes(int b) {
    return (bdx(b) != 0) + (bdy(b) != 0) + (bdz(b) != 0);
}
// Whether entry e (row*3+col) of block b can be non-zero in the elasticity
// stencil: faces are diagonal, edges couple the two components of their
// plane symmetrically, corners are zero, the centre is full.
__host__ __device__ constexpr bool elastic_entry(int b, int e) {
    return b == 13 ? true
         : nnz_axes(b) == 1 ? (e == 0 || e == 4 || e == 8)
         : nnz_axes(b) == 2 ? (bdz(b) == 0 ? (e == 1 || e == 3)
                             : bdy(b) == 0 ? (e == 2 || e == 6)
                                           : (e == 5 || e == 7))
         : false;
}

// COH: the field is written by other blocks of the same launch (the
// persistent small-level kernel), so read it through L2 (ld.global.cg), not
// from a possibly stale L1 line.
template <typename T, bool COH = false>
__device__ inline void load3(const T *__restrict__ f, int npad, int s, T *v) {
    if (COH) {
        v[0] = __ldcg(f + s);
        v[1] = __ldcg(f + s + npad);
        v[2] = __ldcg(f + s + 2 * npad);
    } else {
        v[0] = f[s];
        v[1] = f[s + npad];
        v[2] = f[s + 2 * npad];
    }
}

// ---------------------------------------------------------------- constant
// acc -= sum_{b (!= 13 unless WITH_CENTRE)} a[b] x_b   for an interior node.
template <typename T, bool ELASTIC, bool WITH_CENTRE>
__device__ inline void const_row(const ConstOp<T> &op, const Geom &g, const NbrOffsets &t,
                                 const T *__restrict__ x, T *acc) {
    // neighbour components first (only those the stencil uses), then arithmetic
    T v[27][3];
#pragma unroll
    for (int b = 0; b < 27; b++) {
        if (b == 13 && !WITH_CENTRE) continue;
        if (ELASTIC && nnz_axes(b) == 3) continue;
        int s = t.ox[bdx(b) + 1] + t.oy[bdy(b) + 1] + t.oz[bdz(b) + 1];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            bool used = !ELASTIC || b == 13;
#pragma unroll
            for (int r = 0; r < 3; r++) used = used || elastic_entry(b, 3 * r + c);
            v[b][c] = used ? x[s + c * g.npad] : T(0);
        }
    }
#pragma unroll
    for (int b = 0; b < 27; b++) {
        if (b == 13 && !WITH_CENTRE) continue;
        if (ELASTIC && nnz_axes(b) == 3) continue;
        if (ELASTIC && b != 13) {
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (elastic_entry(b, e)) acc[e / 3] -= op.a[b][e] * v[b][e % 3];
        } else if (b == 13 && op.centre_diag) {
            // a diagonal centre block (the elasticity stencil): only its three
            // non-zero products are formed
            acc[0] -= op.a[13][0] * v[13][0];
            acc[1] -= op.a[13][4] * v[13][1];
            acc[2] -= op.a[13][8] * v[13][2];
        } else {
            matvec_sub(op.a[b], v[b], acc);
        }
    }
}

// ---------------------------------------------------------------- Lame
// Stencil of the variable-coefficient operator -dt*div(mu(grad u + grad u^T)
// + lam div(u) I): face blocks from midpoint-averaged coefficients, edge
// blocks from node values (block (+1,+1,0): a12 = (lam[i+1,j] + mu[i,j+1])/(4dxdy)).
// Reduces to the constant stencil for constant mu, lam.
template <typename T>
struct LameRow {
    T face[6][3];     // face diagonal, order x-, x+, y-, y+, z-, z+
    T centre[3];      // diagonal of the centre block
};

template <typename T>
__device__ inline void lame_faces(const LameOp<T> &op, const Geom &g, const NbrOffsets &t, int p,
                                  LameRow<T> &L, T mu_nb[6], T lam_nb[6]) {
    const T mu0 = op.mu[p], lam0 = op.lam[p];
    const int ctr_x = t.ox[1], ctr_y = t.oy[1], ctr_z = t.oz[1];
    const int sl[6] = {t.ox[0] + ctr_y + ctr_z, t.ox[2] + ctr_y + ctr_z, ctr_x + t.oy[0] + ctr_z,
                       ctr_x + t.oy[2] + ctr_z, ctr_x + ctr_y + t.oz[0], ctr_x + ctr_y + t.oz[2]};
    T cen[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int f = 0; f < 6; f++) {
        mu_nb[f] = op.mu[sl[f]];
        lam_nb[f] = op.lam[sl[f]];
        const int ax = f / 2;
        T mu_f = T(0.5) * (mu0 + mu_nb[f]);
        T lam_f = T(0.5) * (lam0 + lam_nb[f]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            T v = (c == ax ? (lam_f + T(2) * mu_f) : mu_f) * op.ih2[ax];
            L.face[f][c] = -op.dt * v;
            cen[c] -= v;
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) L.centre[c] = -op.dt * cen[c];
}

// acc -= sum over the 18 non-zero off-centre blocks (and the centre if asked).
template <typename T, bool WITH_CENTRE>
__device__ inline void lame_row(const LameOp<T> &op, const Geom &g, const NbrOffsets &t, int p,
                                const T *__restrict__ x, T *acc, T *centre_out) {
    LameRow<T> L;
    T mu_nb[6], lam_nb[6];
    lame_faces(op, g, t, p, L, mu_nb, lam_nb);
    const int npad = g.npad;
    // faces
#pragma unroll
    for (int f = 0; f < 6; f++) {
        const int ax = f / 2, s = (f & 1) ? 2 : 0;
        int sl = (ax == 0 ? t.ox[s] : t.ox[1]) + (ax == 1 ? t.oy[s] : t.oy[1]) + (ax == 2 ? t.oz[s] : t.oz[1]);
        T v[3];
        load3(x, npad, sl, v);
#pragma unroll
        for (int c = 0; c < 3; c++) acc[c] -= L.face[f][c] * v[c];
    }
    // edges: component pair (r, c) in the plane of axes (r, c)
#pragma unroll
    for (int pr = 0; pr < 3; pr++) {
        const int r = pr == 2 ? 1 : 0, c = pr == 0 ? 1 : 2;
        const T ie = op.iedge[pr];
#pragma unroll
        for (int sr = -1; sr <= 1; sr += 2)
#pragma unroll
            for (int sc = -1; sc <= 1; sc += 2) {
                int d[3] = {0, 0, 0};
                d[r] = sr;
                d[c] = sc;
                int sl = t.ox[d[0] + 1] + t.oy[d[1] + 1] + t.oz[d[2] + 1];
                const T sgn = T(sr * sc);
                // neighbour coefficient values: lam/mu at p + sr e_r and p + sc e_c
                const T lam_r = lam_nb[2 * r + (sr > 0)], mu_r = mu_nb[2 * r + (sr > 0)];
                const T lam_c = lam_nb[2 * c + (sc > 0)], mu_c = mu_nb[2 * c + (sc > 0)];
                const T a_rc = -op.dt * ((sgn * (lam_r + mu_c)) * ie);
                const T a_cr = -op.dt * ((sgn * (lam_c + mu_r)) * ie);
                acc[r] -= a_rc * x[sl + c * npad];
                acc[c] -= a_cr * x[sl + r * npad];
            }
    }
    if (WITH_CENTRE) {
        T v[3];
        load3(x, npad, p, v);
#pragma unroll
        for (int c = 0; c < 3; c++) acc[c] -= L.centre[c] * v[c];
    }
    if (centre_out) {
#pragma unroll
        for (int c = 0; c < 3; c++) centre_out[c] = L.centre[c];
    }
}

template <typename T>
__device__ inline T lame_fix(const LameOp<T> &op, int p) {
    const T mu0 = op.mu[p], lam0 = op.lam[p];
    return (-op.dt * T(2)) * ((lam0 + T(2) * mu0) * op.ih2[0] + mu0 * op.ih2[1] + mu0 * op.ih2[2]);
}

// ---------------------------------------------------------------- dense
template <typename T, bool WITH_CENTRE, bool COH = false>
__device__ inline void dense_row(const DenseOp<T> &op, const Geom &g, const NbrOffsets &t, int p,
                                 const T *__restrict__ x, T *acc) {
    const size_t np = (size_t)g.npad;
#pragma unroll
    for (int b = 0; b < 27; b++) {
        if (b == 13 && !WITH_CENTRE) continue;
        int s = t.ox[bdx(b) + 1] + t.oy[bdy(b) + 1] + t.oz[bdz(b) + 1];
        if (s < 0) continue;   // outside a non-periodic grid: coefficients are zero there
        T v[3], a[9];
        load3<T, COH>(x, g.npad, s, v);
        const T *cb = op.coef + (size_t)(9 * b) * np + p;
#pragma unroll
        for (int e = 0; e < 9; e++) a[e] = __ldg(cb + (size_t)e * np);
        matvec_sub(a, v, acc);
    }
}

// ---------------------------------------------------------------- plane
// Structural non-zeros of the coarse elasticity operators: entry (r,c) of the
// block at offset d can be non-zero only if r == c or d_r, d_c are both non-zero.
__host__ __device__ constexpr bool coarse_entry(int b, int e) {
    return (e / 3 == e % 3) ||
           ((e / 3 == 0 ? bdx(b) : e / 3 == 1 ? bdy(b) : bdz(b)) != 0 &&
            (e % 3 == 0 ? bdx(b) : e % 3 == 1 ? bdy(b) : bdz(b)) != 0);
}

// acc -= sum_b A_b x_b with entry e of block b read from cf[(9b + e) * stride]
// (shared memory with stride 1, or plane storage in global memory).
template <typename T, bool SPARSE, bool WITH_CENTRE, bool COH = false>
__device__ inline void plane_row_coef(const T *cf, int stride, const Geom &g, const NbrOffsets &t,
                                      const T *__restrict__ x, T *acc) {
    if constexpr (sizeof(T) == 8) {
        // FP64: arithmetic bound; load each neighbour right before its block
#pragma unroll
        for (int b = 0; b < 27; b++) {
            if (b == 13 && !WITH_CENTRE) continue;
            int s = t.ox[bdx(b) + 1] + t.oy[bdy(b) + 1] + t.oz[bdz(b) + 1];
            if (s < 0) continue;
            T v[3];
            load3<T, COH>(x, g.npad, s, v);
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (!SPARSE || coarse_entry(b, e)) acc[e / 3] -= cf[(9 * b + e) * stride] * v[e % 3];
        }
    } else {
        // FP32: all neighbour loads are issued before the arithmetic so that
        // they are in flight together (one memory latency per node, not one per block)
        T v[27][3];
#pragma unroll
        for (int b = 0; b < 27; b++) {
            if (b == 13 && !WITH_CENTRE) continue;
            int s = t.ox[bdx(b) + 1] + t.oy[bdy(b) + 1] + t.oz[bdz(b) + 1];
            const int sc = s < 0 ? 0 : s;
            load3<T, COH>(x, g.npad, sc, v[b]);
            if (s < 0) v[b][0] = v[b][1] = v[b][2] = T(0);
        }
#pragma unroll
        for (int b = 0; b < 27; b++) {
            if (b == 13 && !WITH_CENTRE) continue;
#pragma unroll
            for (int e = 0; e < 9; e++)
                if (!SPARSE || coarse_entry(b, e)) acc[e / 3] -= cf[(9 * b + e) * stride] * v[b][e % 3];
        }
    }
}

}  // namespace stzmg
