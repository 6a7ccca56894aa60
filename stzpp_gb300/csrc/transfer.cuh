// Per-node grid-transfer arithmetic shared by the transfer kernels and the
// persistent small-level kernel.  See transfer.cu for the definitions of P
// (interpolation) and R (restriction) and their reference counterparts.
#pragma once

#include "ops.cuh"

namespace stzmg {

// Weight of fine index f (unwrapped, f in {2I-1, 2I, 2I+1}) as a child of
// coarse index I along one dimension: 1, 0.5, or 0 when f is not a child.
template <typename T>
__host__ __device__ inline T child_w(int I, int f, int mf, int prd) {
    if (!prd && (f < 0 || f >= mf)) return T(0);
    const bool collapse_dim = !prd && !(mf & 1);   // last fine node coincides with last coarse node
    if (f == 2 * I) return T(1);                    // (2I < mf guaranteed by the range test above)
    if (f == 2 * I - 1) return (collapse_dim && f == mf - 1) ? T(1) : T(0.5);
    /* f == 2I + 1 */
    return (collapse_dim && f == mf - 1) ? T(0) : T(0.5);
}

__device__ inline int wrapi(int a, int len) {
    if (a < 0) return a + len;
    if (a >= len) return a - len;
    return a;
}

// Coarse r at slot p (node I,J,K) = sum of (1/8) P-weighted fine residuals,
// including the restrict_partial mask-145 quirk (see transfer.cu).
template <typename T, bool COH = false>
__device__ inline void restrict_node(const Geom &gf, const Geom &gc, const T *__restrict__ res, int p, int I, int J,
                                     int K, T *acc) {
    acc[0] = acc[1] = acc[2] = T(0);
    const bool xs = !gf.xp && !(gf.m & 1) && I == gc.m - 2;
    for (int dz = -1; dz <= 1; dz++) {
        int fz = 2 * K + dz;
        T wz = child_w<T>(K, fz, gf.o, gf.zp);
        if (wz == T(0)) continue;
        int fzw = wrapi(fz, gf.o);
        for (int dy = -1; dy <= 1; dy++) {
            int fy = 2 * J + dy;
            T wy = child_w<T>(J, fy, gf.n, gf.yp);
            if (!gf.yp && (fy < 0 || fy >= gf.n)) continue;
            int fyw = wrapi(fy, gf.n);
            for (int dx = -1; dx <= 1; dx++) {
                int fx = 2 * I + dx;
                T wx = child_w<T>(I, fx, gf.m, gf.xp);
                if (wx == T(0)) continue;
                T wyy = wy;
                if (dx == 0 && (fy & 1) && (fz & 1)) wyy = xs ? (dy < 0 ? T(1) : T(0)) : T(0.5);
                if (wyy == T(0)) continue;
                int s = slot(gf, wrapi(fx, gf.m), fyw, fzw);
                T w = T(0.125) * wx * wyy * wz;
                T v[3];
                load3<T, COH>(res, gf.npad, s, v);
                acc[0] += w * v[0];
                acc[1] += w * v[1];
                acc[2] += w * v[2];
            }
        }
    }
}

// Parents of fine index f (wrapped coarse indices).
__device__ inline int parents(int f, int mf, int mc, int prd, int *c) {
    if ((f & 1) == 0) { c[0] = f >> 1; return 1; }
    if (!prd && !(mf & 1) && f == mf - 1) { c[0] = (f >> 1) + 1; return 1; }
    c[0] = f >> 1;
    c[1] = wrapi((f >> 1) + 1, mc);
    return 2;
}

// (P x_c) at fine node (i,j,k).
template <typename T, bool COH = false>
__device__ inline void interp_node(const Geom &gf, const Geom &gc, const T *__restrict__ xc, int i, int j, int k,
                                   T *s) {
    int cx[2], cy[2], cz[2];
    int nx = parents(i, gf.m, gc.m, gf.xp, cx);
    int ny = parents(j, gf.n, gc.n, gf.yp, cy);
    int nz = parents(k, gf.o, gc.o, gf.zp, cz);
    s[0] = s[1] = s[2] = T(0);
    for (int a = 0; a < nz; a++)
        for (int b = 0; b < ny; b++)
            for (int c = 0; c < nx; c++) {
                T v[3];
                load3<T, COH>(xc, gc.npad, slot(gc, cx[c], cy[b], cz[a]), v);
                s[0] += v[0];
                s[1] += v[1];
                s[2] += v[2];
            }
    // every parent of a node carries the same weight 1/2^(number of split dimensions)
    const T w = T(1) / T(nx * ny * nz);
    s[0] *= w;
    s[1] *= w;
    s[2] *= w;
}

}  // namespace stzmg
