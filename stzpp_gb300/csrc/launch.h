// Host-side declarations of the kernel launchers of the GB300 multigrid.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace stzmg {

constexpr int kMaxLevels = 16;

// One level's operator as the kernels see it.
template <typename T>
struct LevelOp {
    OpKind kind;
    ConstOp<T> cop;
    LameOp<T> lop;
    DenseOp<T> dop;
    PlaneOp<T> pop;
};

// smooth.cu
template <typename T>
void launch_gs_colour(const LevelOp<T> &op, const Geom &g, int q, const T *r, T *x, cudaStream_t st);
template <typename T>
void launch_gs_sweep(const LevelOp<T> &op, const Geom &g, const T *r, T *x, cudaStream_t st);
// `sweeps` in-place sweeps of x; tmp (3*npad, may be null) lets large levels
// use the tiled two-buffer sweep of tile.cu, with the same result
template <typename T>
void launch_gs_sweeps(const LevelOp<T> &op, const Geom &g, const T *r, T *x, T *tmp, int sweeps, cudaStream_t st);
// tile.cu: one sweep reading xin and writing xout (levels periodic in x, y
// with whole 32x32 tiles, shared-stencil or plane-invariant operators)
template <typename T>
bool gs_tile_applies(const LevelOp<T> &op, const Geom &g);
template <typename T>
void launch_gs_sweep_tile(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st);
// band.cu: one sweep reading xin and writing xout on the top level of a
// shared elasticity stencil periodic in x, y (full-width bands of 8 rows,
// planes staged by TMA); false if the tensor maps cannot be made
template <typename T>
bool gs_band_applies(const LevelOp<T> &op, const Geom &g);
template <typename T>
bool launch_gs_sweep_band(const LevelOp<T> &op, const Geom &g, const T *r, const T *xin, T *xout, cudaStream_t st);
template <typename T>
bool gs_band_ready(const Geom &g, const T *field);
// band.cu: res = r - A x by full-width bands staged by TMA where the band
// sweep applies (no norm); false where it does not
template <typename T>
bool launch_residual_band(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, cudaStream_t st);
// tile.cu: rc = R (r - A x) in one pass on the levels the tiled residual
// serves with a shared stencil (the fine level's residual never written;
// opt-in, STZ_MG_FUSED_RESTRICT=1); false where it does not apply
template <typename T>
bool launch_residual_restrict(const LevelOp<T> &op, const Geom &g, const Geom &gc, const T *r, const T *x, T *rc,
                              cudaStream_t st);
// How launch_gs_sweeps smooths a level: 0 eight colour launches per sweep,
// 1 the tiled two-buffer sweep, 2 the band sweep, 3 the plane-phase kernels
// (two launches per sweep each but the first)
template <typename T>
int gs_sweep_kind(const LevelOp<T> &op, const Geom &g, const T *x, bool has_tmp);
// 1 if a band CTA gave up waiting for its copies since the last call, 2 if
// one found its shared memory misaligned for TMA (the record is cleared),
// 0 if none did, -1 if the record cannot be read
int band_take_error(cudaStream_t st);
// tile.cu: res = r - A x by plane tiles staged in shared memory; with
// partial non-null, per-CTA sums of |res|^2
template <typename T>
bool residual_tile_applies(const LevelOp<T> &op, const Geom &g);
// the tiled residual's CTA count (its number of norm partials)
int residual_tile_blocks(const Geom &g, bool fp64);
template <typename T>
void launch_residual_tile(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, T *res, double *partial,
                          cudaStream_t st);
// output.cu: a z-slice of a top-level vec3 field (colour-blocked) as floats
// of |v|^2 (|v|^2 |v|^2 with quartic), m x n natural order; the file of
// region::output_internal for one process
void launch_slice(const Geom &g, const double *f, int k, bool quartic, float *out, cudaStream_t st);
bool write_slice_file(const float *vals, int m, int n, double ax, double bx, double ay, double by,
                      const char *filename);
int residual_blocks(const Geom &g);
// out[0] = the fixed-order sum of partial[0 .. n-1]
void launch_sum_partials(const double *partial, int n, double *out, cudaStream_t st);
// residual_df.cu: r32 = b - A x of a shared-stencil top level in double-float
// arithmetic (x split first into the (hi, lo) float pairs xs, 3*npad of
// them; with corr non-null x += corr first, in the same pass); per-block
// sums of (scale * r32)^2 into partial and, when out is non-null, their sum
// to out[0]
bool residual_df_applies(const LevelOp<double> &op);
double df_norm_scale(double bsq, size_t n);
void launch_residual_df(const LevelOp<double> &op, const Geom &g, const double *b, double *x, const float *corr,
                        float2 *xs, float *r32, double scale, double *partial, double *out, cudaStream_t st);
// res = r - A x (res may be null); when partial is non-null, per-block sums of
// |res|^2 go to partial[residual_blocks(g)] and, when out is non-null, their
// total to out[0].
template <typename T, typename R>
void launch_residual(const LevelOp<T> &op, const Geom &g, const T *r, const T *x, R *res, double *partial,
                     double *out, cudaStream_t st);

// transfer.cu
template <typename T>
void launch_restriction(const Geom &gf, const Geom &gc, const T *res_f, T *r_c, cudaStream_t st);
template <typename T>
void launch_interpolation(const Geom &gf, const Geom &gc, const T *x_c, T *x_f, cudaStream_t st);
// natural-order AoS vec3 (double) <-> colour-blocked SoA
template <typename T>
void launch_nat_to_cb(const Geom &g, const double *nat, T *cb, cudaStream_t st);
template <typename T>
void launch_cb_to_nat(const Geom &g, const T *cb, double *nat, cudaStream_t st);
// natural-order scalar (double) -> colour-blocked scalar
template <typename T>
void launch_scalar_nat_to_cb(const Geom &g, const double *nat, T *cb, cudaStream_t st);
// natural-order dense coefficients (npts x 243 doubles) -> colour-blocked SoA (243 x npad)
void launch_coef_nat_to_cb(const Geom &g, const double *nat, double *cb, cudaStream_t st);
void launch_coef_cb_to_nat(const Geom &g, const double *cb, double *nat, cudaStream_t st);
void launch_convert(const double *src, float *dst, size_t n, cudaStream_t st);
// x64 += e32 over n elements
void launch_add_correction(double *x, const float *e, size_t n, cudaStream_t st);
// x = Ainv r on the bottom level: Ainv is (3N)^2 row-major in natural node
// order (3 rows per node); nat_slot maps natural node index -> slot.
template <typename T>
void launch_bottom_direct(int nrow, const double *ainv_t, const int *nat_slot, int npad, const T *r, T *x,
                          cudaStream_t st);
void launch_scale(double *v, double s, size_t n, cudaStream_t st);
// inverse of the n x n matrix in the left half of the augmented n x 2n matrix
// [M | I] (row-major, overwritten) into inv (row-major); bad[0] set when singular
void launch_gauss_jordan(double *aug, int n, double *inv, int *piv, double *col, int *bad, cudaStream_t st);

// field.cu
// r (colour-blocked, 3 x npad) = node divergence of the cell tensor field eps
void launch_rhs_divergence(const Geom &g, const double *eps, double dx, double dy, double dz, double *r,
                           cudaStream_t st);
// sigma (6 doubles per cell, natural order) += the projection-step stress
// increment of the solution u (colour-blocked FP64); per-block sums of
// modsq(increment) to partial[0 .. nblocks)
void launch_stress_update(const Geom &g, const double *u, double *sigma, double lam, double mu, double dt, double dx,
                          double dy, double dz, double *partial, int nblocks, cudaStream_t st);

// adjoint.cu (natural-order vec3 fields, 3 doubles per node)
// dst = src with the rows of Dirichlet nodes zeroed
void launch_mask_dirichlet(const Geom &g, const double *src, double *dst, cudaStream_t st);
// w_D = F^{-T} (g_D - A_ID^T w_I) on the Dirichlet nodes of the top level
// (OP_CONST or OP_LAME), given w on the interior nodes
void launch_adjoint_dirichlet(const LevelOp<double> &top, const Geom &g, const double *gv, double *w,
                              cudaStream_t st);
// dmu, dlam = -w^T (dA/dmu, dA/dlam) u per node of the Lame operator; C is
// scratch of 14 doubles per node
void launch_lame_grad(const LameOp<double> &op, const Geom &g, const double *w, const double *u, double *C,
                      double *dmu, double *dlam, cudaStream_t st);

// tail.cu: persistent cluster kernels for the small levels lo..hi (hi+1 is
// the bottom level).  Levels must be OP_PLANE or OP_DENSE.
constexpr int kTailThreads = 1024;
template <typename T>
struct TailLev {
    Geom g;
    int kind;
    const T *coef, *dinv;
    int O, sparse;
    T *x, *r, *res;
};
template <typename T>
struct TailDesc {
    int lo, hi, v_down, v_up, growth, cap_planes;
    TailLev<T> L[kMaxLevels];
};
template <typename T>
cudaError_t launch_tail_down(const TailDesc<T> &d, int cluster, cudaStream_t st);
template <typename T>
cudaError_t launch_tail_up(const TailDesc<T> &d, int cluster, cudaStream_t st);
// cluster size (16 or 8) the device can run with this shared memory, or 0
template <typename T>
int tail_cluster_size(int smem_bytes);

// rat.cu
// Galerkin coarse operator A_c = (1/8) P^T A P into a dense SoA field (243 x npad_c),
// or, when plane is set, into plane storage (243 x o_c) from the column i = j = 0.
void launch_rat(const LevelOp<double> &fine, const Geom &gf, const Geom &gc, double *coef_c, bool plane,
                cudaStream_t st);
// inverse centre blocks of plane storage
template <typename T>
void launch_plane_dinv(int O, const T *coef, T *dinv, int *bad, cudaStream_t st);
// dense 27-block SoA copy of any operator (top level export)
void launch_expand_dense(const LevelOp<double> &op, const Geom &g, double *coef, cudaStream_t st);
// inverse of every centre block; bad[0] set to 1 on a singular/non-finite block
template <typename T>
void launch_dense_dinv(const Geom &g, const T *coef, T *dinv, int *bad, cudaStream_t st);
// RAT box bounds (6 ints per slot) of the coarse level from the fine bounds
// (fill_rat_bounds); fine_S null means the top level's interior/boundary boxes.
void launch_rat_bounds(const Geom &gf, const int *fine_S, const Geom &gc, int *S_c, int *bad, cudaStream_t st);
void launch_top_bounds(const Geom &g, int *S, cudaStream_t st);
void launch_bounds_cb_to_nat(const Geom &g, const int *S, int *nat, cudaStream_t st);

}  // namespace stzmg
