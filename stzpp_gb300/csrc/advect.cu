// Quasi-static advection step of shear_sim_3d (src/shear_sim_3d.cpp:393-525)
// on the device: the part of step_forward_qs before the projection solve.
//
// Fields are device arrays of the reference's ghosted grid ((nx+4) x (ny+4)
// x (nz+4) points, 2 ghost layers, x fastest), one array per Field member
// (src/field.hh:11-22), the ghosts filled by the caller as the reference's
// set_up_ghost_regions / set_boundary_conditions do.  Three launches:
//
//  1. plastic_kernel: per interior cell, sbar (Field::dev) and, above the
//     yield stress, the adaptive sub-stepping of the STZ plastic rate
//     (adaptive_plastic_term, shear_sim_3d.cpp:108-147), which adds the
//     plastic change of chi to cchi; the new ad_Dpl into scratch;
//  2. update_kernel: the ENO2 advection of the stresses and chi, the
//     Truesdell terms and the chi diffusion (shear_sim_3d.cpp:413-525);
//  3. the new ad_Dpl copied over the old.
//
// The reference updates the points in place in z, y, x order, so a point's
// chi diffusion reads the new ad_Dpl of its interior -x, -y, -z neighbours
// and the previous step's value of the others; update_kernel reads the same.
// Every operation is an explicitly rounded one (no contraction into FMAs), in
// the reference's order, so the results equal the reference's except where
// they depend on exp (the plastic rate), which is CUDA's.
#include <cuda_runtime.h>

#include "stz_mg.h"

namespace {

constexpr int kG = 2;   // ghost layers
// Bound on the adaptive sub-steps of one cell (the reference loops until its
// remaining time is spent; an infinite or NaN-free but huge plastic rate
// would never end): a cell that reaches it stops and the step reports
// STZ_MG_ERR_NONFINITE.
constexpr int kMaxSubsteps = 1 << 22;

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }

struct AdvGrid {
    int nx, ny, nz;
    long sx, sy, sz;   // strides of the ghosted grid: 1, nx + 4, (nx + 4)(ny + 4)
    long npts;
};

// The step's loop-invariant factors, each the reference's own rounded value
// (a correctly rounded division or product gives the same double wherever it
// is computed), worked out once on the host instead of per use: the FP64
// pipe bounds these kernels and a division costs it about ten operations.
struct AdvConst {
    double dxi, dyi, dzi;   // dx_inv = 1./dx (shear_sim_3d.cpp:46)
    double qx, qy, qz;      // .25*dx_inv (calculate_first_order_velocities)
    double hx, hy, hz;      // .5/h of eno2 with h = dx/dt (advection_grid_step)
    double gx, gy, gz;      // .5*dx_inv (chi_diffusion)
    double lx, ly, lz;      // dx_inv*dx_inv (chi_diffusion)
    double third;           // 1./3. (also Field::pressure's 1/3.)
    double dl2;             // diff_l*diff_l
};

__device__ __forceinline__ bool cell_of(const AdvGrid &g, int &i, int &j, int &k, long &p) {
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return false;
    p = (i + kG) + g.sy * (j + kG) + g.sz * (k + kG);
    return true;
}

// Field::dev (field.hh:147-184)
__device__ __forceinline__ double devstress(double s11, double s12, double s13, double s22, double s23, double s33,
                                            double third) {
    const double p = ml(-ad(ad(s11, s22), s33), third);
    const double t11 = ad(s11, p), t22 = ad(s22, p), t33 = ad(s33, p);
    double q = ml(0.5, ad(ad(ml(t11, t11), ml(t22, t22)), ml(t33, t33)));
    q = ad(ad(ad(q, ml(s12, s12)), ml(s13, s13)), ml(s23, s23));
    return __dsqrt_rn(q);
}

// calc_Dpl with calc_Lambda and calc_curly_c (shear_sim_3d.cpp:1170-1188)
__device__ __forceinline__ double plastic_rate(const stz_adv_params &P, double sbar, double chi) {
    if (!(sbar >= P.sy)) return 0.0;
    const double lam = exp(dv(-P.ez, chi));
    const double oe = ml(ml(P.omega, P.eps0), sbar);
    const double c1 = exp(dv(sb(oe, P.delta), P.bath_temp));
    const double c2 = exp(dv(-ad(oe, P.delta), P.bath_temp));
    const double cc = ml(0.5, ad(c1, c2));
    return dv(ml(ml(lam, cc), sb(1.0, dv(P.sy, sbar))), P.tau0);
}

__global__ void plastic_kernel(AdvGrid g, stz_adv_params P, AdvConst C, double dt, const double *__restrict__ s11,
                               const double *__restrict__ s12, const double *__restrict__ s13,
                               const double *__restrict__ s22, const double *__restrict__ s23,
                               const double *__restrict__ s33, const double *__restrict__ chi,
                               double *__restrict__ cchi, double *__restrict__ sbar_out,
                               double *__restrict__ adapt_out, double *__restrict__ adnew, double *__restrict__ flag) {
    int i, j, k;
    long p;
    if (!cell_of(g, i, j, k, p)) return;
    const double sbar0 = devstress(s11[p], s12[p], s13[p], s22[p], s23[p], s33[p], C.third);
    sbar_out[p] = sbar0;
    double adapt = 0.0;
    if (sbar0 > P.sy) {
        // adaptive_plastic_term: sub-steps of at most eta in the scaled plastic strain
        const double eta = .0005;
        double tr = dt, ts;
        const double chi0 = chi[p];
        double sa = sbar0, ca = chi0;
        for (int it = 0;; it++) {
            if (it == kMaxSubsteps) {
                flag[1] = 1.0;
                break;
            }
            const double d = plastic_rate(P, sa, ca);
            const double dp = dv(ml(ml(2.0, P.mu), d), P.sy);
            // calc_chi_F (shear_sim_3d.cpp:1240-1244)
            const double F = dv(ml(ml(ml(2.0, d), sa), sb(P.chi_inf, ca)), ml(P.sy, P.c0));
            bool last = false;
            if (ml(dp, tr) > eta) {
                ts = dv(eta, fabs(dp));
                tr = sb(tr, ts);
            } else {
                ts = tr;
                last = true;
            }
            sa = sb(sa, ml(ml(ts, dp), P.sy));
            ca = ad(ca, ml(ts, F));
            if (last) break;
        }
        cchi[p] = ad(cchi[p], sb(ca, chi0));
        adapt = sb(1.0, dv(sa, sbar0));
        if (adapt > 0) *flag = 1.0;
    }
    adapt_out[p] = adapt;
    adnew[p] = ml(dv(ml(adapt, 0.5), P.mu), sbar0);   // adapt/2. is exactly adapt*0.5
}

// eno2 (shear_sim_3d.cpp:1256-1266) along stride st from point p of field f;
// half_h = .5/h
__device__ __forceinline__ double eno2(double half_h, double vel, const double *__restrict__ f, long p, long st) {
    const double f2p = f[p + 2 * st], fp = f[p + st], f0 = f[p], fm = f[p - st], f2m = f[p - 2 * st];
    const double c2 = fabs(ad(sb(fp, ml(2.0, f0)), fm));
    double d;
    // only the second difference on the upwind side enters the comparison
    if (vel < 0) {
        const double fw2 = fabs(ad(sb(f2p, ml(2.0, fp)), f0));
        d = c2 > fw2 ? sb(ad(-f2p, ml(4.0, fp)), ml(3.0, f0)) : sb(fp, fm);
    } else {
        const double bk2 = fabs(ad(sb(f0, ml(2.0, fm)), f2m));
        d = c2 > bk2 ? ad(sb(ml(3.0, f0), ml(4.0, fm)), f2m) : sb(fp, fm);
    }
    return ml(half_h, d);
}

// the alternating sum a - b + c - d + e - f + g - h of calculate_first_order_velocities
__device__ __forceinline__ double alt8(const double *__restrict__ f, long p, long a, long b, long c, long d, long e,
                                       long f_, long g, long h) {
    return sb(ad(sb(ad(sb(ad(sb(f[p + a], f[p + b]), f[p + c]), f[p + d]), f[p + e]), f[p + f_]), f[p + g]), f[p + h]);
}

// the cell's 8 nodes, in the order of the staggered velocities (shear_sim_3d.cpp:432-434)
__device__ __forceinline__ double node_mean(const double *__restrict__ f, long p, long X, long Y, long Z) {
    double t = ad(f[p], f[p + X]);
    t = ad(t, f[p + Z]);
    t = ad(t, f[p + X + Z]);
    t = ad(t, f[p + Y]);
    t = ad(t, f[p + X + Y]);
    t = ad(t, f[p + Y + Z]);
    t = ad(t, f[p + X + Y + Z]);
    return ml(0.125, t);
}

__device__ __forceinline__ double dot3r(double a, double x, double b, double y, double c, double z) {
    return ad(ad(ml(a, x), ml(b, y)), ml(c, z));
}

__global__ void update_kernel(AdvGrid g, stz_adv_params P, AdvConst C, double dt, const double *__restrict__ u,
                              const double *__restrict__ v, const double *__restrict__ w,
                              const double *__restrict__ s11, const double *__restrict__ s12,
                              const double *__restrict__ s13, const double *__restrict__ s22,
                              const double *__restrict__ s23, const double *__restrict__ s33,
                              const double *__restrict__ chi, const double *__restrict__ adold,
                              const double *__restrict__ adapt_in, const double *__restrict__ adnew,
                              double *__restrict__ cs11, double *__restrict__ cs12, double *__restrict__ cs13,
                              double *__restrict__ cs22, double *__restrict__ cs23, double *__restrict__ cs33,
                              double *__restrict__ cchi) {
    int i, j, k;
    long p;
    if (!cell_of(g, i, j, k, p)) return;
    const long X = g.sx, Y = g.sy, Z = g.sz;
    // calculate_first_order_velocities (shear_sim_3d.cpp:900-917)
    const double qx = C.qx, qy = C.qy, qz = C.qz;
    const double du_dx = ml(qx, alt8(u, p, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z));
    const double dv_dx = ml(qx, alt8(v, p, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z));
    const double dw_dx = ml(qx, alt8(w, p, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z));
    const double du_dy = ml(qy, alt8(u, p, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z));
    const double dv_dy = ml(qy, alt8(v, p, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z));
    const double dw_dy = ml(qy, alt8(w, p, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z));
    const double du_dz = ml(qz, alt8(u, p, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y));
    const double dv_dz = ml(qz, alt8(v, p, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y));
    const double dw_dz = ml(qz, alt8(w, p, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y));
    const double adapt = adapt_in[p];
    const double uc = node_mean(u, p, X, Y, Z), vc = node_mean(v, p, X, Y, Z), wc = node_mean(w, p, X, Y, Z);
    const double *sf[6] = {s11, s12, s13, s22, s23, s33};
    double gd[6];
#pragma unroll
    for (int n = 0; n < 6; n++) {
        const double a = eno2(C.hx, uc, sf[n], p, X);
        const double b = eno2(C.hy, vc, sf[n], p, Y);
        const double c = eno2(C.hz, wc, sf[n], p, Z);
        gd[n] = dot3r(uc, a, vc, b, wc, c);
    }
    const double a11 = s11[p], a12 = s12[p], a13 = s13[p], a22 = s22[p], a23 = s23[p], a33 = s33[p];
    // the Truesdell terms (shear_sim_3d.cpp:476-481)
    const double t11 = ad(ad(ml(a11, sb(sb(du_dx, dv_dy), dw_dz)), ml(ml(2.0, a13), du_dz)), ml(ml(2.0, a12), du_dy));
    const double t12 = ad(ad(sb(ad(ml(a23, du_dz), ml(a13, dv_dz)), ml(a12, dw_dz)), ml(a22, du_dy)), ml(a11, dv_dx));
    const double t13 = sb(ad(ad(ad(ml(a33, du_dz), ml(a11, dw_dx)), ml(a23, du_dy)), ml(a12, dw_dy)), ml(a13, dv_dy));
    const double t22 = ad(ad(ml(ml(2.0, a23), dv_dz), ml(a22, sb(sb(dv_dy, du_dx), dw_dz))), ml(ml(2.0, a12), dv_dx));
    const double t23 = ad(sb(ad(ad(ml(a33, dv_dz), ml(a22, dw_dy)), ml(a13, dv_dx)), ml(a23, du_dx)), ml(a12, dw_dx));
    const double t33 = ad(ad(ml(a33, sb(sb(dw_dz, dv_dy), du_dx)), ml(ml(2.0, a23), dw_dy)), ml(ml(2.0, a13), dw_dx));
    const double at = ml(adapt, C.third), na = -adapt;
    cs11[p] = ad(sb(ml(at, sb(ad(a33, a22), ml(2.0, a11))), gd[0]), ml(dt, t11));
    cs12[p] = ad(sb(ml(na, a12), gd[1]), ml(dt, t12));
    cs13[p] = ad(sb(ml(na, a13), gd[2]), ml(dt, t13));
    cs22[p] = ad(sb(ml(at, ad(sb(a11, ml(2.0, a22)), a33)), gd[3]), ml(dt, t22));
    cs23[p] = ad(sb(ml(na, a23), gd[4]), ml(dt, t23));
    cs33[p] = ad(sb(ml(at, sb(ad(a11, a22), ml(2.0, a33))), gd[5]), ml(dt, t33));
    // chi: advection, then the diffusion (chi_diffusion, shear_sim_3d.cpp:1216-1236)
    const double dchi_dx = eno2(C.hx, uc, chi, p, X);
    const double dchi_dy = eno2(C.hy, vc, chi, p, Y);
    const double dchi_dz = eno2(C.hz, wc, chi, p, Z);
    double c = sb(cchi[p], dot3r(uc, dchi_dx, vc, dchi_dy, wc, dchi_dz));
    // ad_Dpl as the reference's in-place sweep sees it
    const double a0 = adnew[p];
    const double axm = i > 0 ? adnew[p - X] : adold[p - X], axp = adold[p + X];
    const double aym = j > 0 ? adnew[p - Y] : adold[p - Y], ayp = adold[p + Y];
    const double azm = k > 0 ? adnew[p - Z] : adold[p - Z], azp = adold[p + Z];
    const double c0 = chi[p];
    const double cxm = chi[p - X], cxp = chi[p + X], cym = chi[p - Y], cyp = chi[p + Y], czm = chi[p - Z], czp = chi[p + Z];
    const double dD_dx = ml(C.gx, sb(axp, axm)), dD_dy = ml(C.gy, sb(ayp, aym));
    const double dD_dz = ml(C.gz, sb(azp, azm));
    const double gx = ml(C.gx, sb(cxp, cxm)), gy = ml(C.gy, sb(cyp, cym));
    const double gz = ml(C.gz, sb(czp, czm));
    const double lx = ml(C.lx, ad(sb(cxp, ml(2.0, c0)), cxm));
    const double ly = ml(C.ly, ad(sb(cyp, ml(2.0, c0)), cym));
    const double lz = ml(C.lz, ad(sb(czp, ml(2.0, c0)), czm));
    const double ddx = ad(ml(dD_dx, gx), ml(a0, lx));
    const double ddy = ad(ml(dD_dy, gy), ml(a0, ly));
    const double ddz = ad(ml(dD_dz, gz), ml(a0, lz));
    const double diff = ml(C.dl2, ad(ad(ddx, ddy), ddz));
    cchi[p] = ad(c, dv(diff, P.c0));
}

__global__ void copy_interior_kernel(AdvGrid g, const double *__restrict__ src, double *__restrict__ dst) {
    int i, j, k;
    long p;
    if (!cell_of(g, i, j, k, p)) return;
    dst[p] = src[p];
}

}  // namespace

extern "C" int stz_mg_advection_step(const stz_adv_params *P, const stz_adv_fields *f, double dt, void *stream,
                            int *yielded) {
    if (!P || !f) return STZ_MG_ERR_ARG;
    if (P->nx < 1 || P->ny < 1 || P->nz < 1 || !(dt > 0)) return STZ_MG_ERR_ARG;
    const double *in[] = {f->u, f->v, f->w, f->s11, f->s12, f->s13, f->s22, f->s23, f->s33, f->chi};
    double *out[] = {f->ad_dpl, f->sbar, f->cs11, f->cs12, f->cs13, f->cs22, f->cs23, f->cs33, f->cchi, f->work};
    for (const double *q : in)
        if (!q) return STZ_MG_ERR_ARG;
    for (double *q : out)
        if (!q) return STZ_MG_ERR_ARG;
    AdvGrid g;
    g.nx = P->nx;
    g.ny = P->ny;
    g.nz = P->nz;
    g.sx = 1;
    g.sy = P->nx + 2 * kG;
    g.sz = g.sy * (P->ny + 2 * kG);
    g.npts = g.sz * (P->nz + 2 * kG);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    AdvConst C;
    C.dxi = 1. / P->dx;
    C.dyi = 1. / P->dy;
    C.dzi = 1. / P->dz;
    C.qx = .25 * C.dxi;
    C.qy = .25 * C.dyi;
    C.qz = .25 * C.dzi;
    C.hx = .5 / (P->dx / dt);
    C.hy = .5 / (P->dy / dt);
    C.hz = .5 / (P->dz / dt);
    C.gx = .5 * C.dxi;
    C.gy = .5 * C.dyi;
    C.gz = .5 * C.dzi;
    C.lx = C.dxi * C.dxi;
    C.ly = C.dyi * C.dyi;
    C.lz = C.dzi * C.dzi;
    C.third = 1. / 3.;
    C.dl2 = P->diff_l * P->diff_l;
    // work: adaptive terms, new ad_Dpl, then flags {a cell yielded, a cell hit kMaxSubsteps}
    double *adapt = f->work, *adnew = f->work + g.npts, *flag = f->work + 2 * g.npts;
    if (cudaMemsetAsync(flag, 0, 2 * sizeof(double), st) != cudaSuccess) return STZ_MG_ERR_CUDA;
    const dim3 blk(32, 8), grd((P->nx + 31) / 32, (P->ny + 7) / 8, P->nz);
    plastic_kernel<<<grd, blk, 0, st>>>(g, *P, C, dt, f->s11, f->s12, f->s13, f->s22, f->s23, f->s33, f->chi, f->cchi,
                                        f->sbar, adapt, adnew, flag);
    update_kernel<<<grd, blk, 0, st>>>(g, *P, C, dt, f->u, f->v, f->w, f->s11, f->s12, f->s13, f->s22, f->s23, f->s33,
                                       f->chi, f->ad_dpl, adapt, adnew, f->cs11, f->cs12, f->cs13, f->cs22, f->cs23,
                                       f->cs33, f->cchi);
    copy_interior_kernel<<<grd, blk, 0, st>>>(g, adnew, f->ad_dpl);
    if (cudaGetLastError() != cudaSuccess) return STZ_MG_ERR_CUDA;
    if (yielded) {
        double h[2] = {0, 0};
        if (cudaMemcpyAsync(h, flag, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return STZ_MG_ERR_CUDA;
        *yielded = h[0] != 0.0;
        if (h[1] != 0.0) return STZ_MG_ERR_NONFINITE;
    }
    return STZ_MG_OK;
}
