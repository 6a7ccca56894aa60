/* CPU restatement of the quasi-static advection step of shear_sim_3d
 * (src/shear_sim_3d.cpp:393-525).  TEST INFRASTRUCTURE ONLY: the GPU step
 * (stzpp_gb300/csrc/advect.cu) is checked against it; nothing in the product
 * calls it.  Pinned bit for bit to the unmodified reference step run through
 * oracle/adv_harness.cc (tests/test_oracle_advect.py, golden fixture
 * tests/golden/adv_step.npz).
 *
 * The grid is the reference's: points of 28 doubles (struct Field,
 * src/field.hh:10-23), nghost = 2 ghost layers on every side
 * (shear_sim_3d.cpp:39,49,81-82), x fastest.  Only interior points are
 * updated; the ghosts are inputs.  Every expression keeps the reference's
 * operation order, and the file is compiled with -ffp-contract=off, so the
 * results equal the reference's on the same machine. */
#include <math.h>
#include <stddef.h>

#include "stzadv_oracle.h"

/* Field members (field.hh:11-22). */
enum {
    FU, FV, FW, FS11, FS12, FS13, FS22, FS23, FS33, FCHI,
    FCU, FCV, FCW, FCS11, FCS12, FCS13, FCS22, FCS23, FCS33, FCCHI,
    FXI, FYI, FZI, FCXI, FCYI, FCZI, FSBAR, FADPL, FN
};

typedef struct {
    const adv_par_t *p;
    double dx_inv, dy_inv, dz_inv;
    long nxg, nxyg;
} ctx_t;

#define AT(f, off, m) ((f)[((off)) * FN + (m)])

/* Field::devsq / dev (field.hh:147-184); dev() also stores sbar. */
static double dev(double *q) {
    double p = -(q[FS11] + q[FS22] + q[FS33]) * (1 / 3.);
    double t11 = q[FS11] + p, t22 = q[FS22] + p, t33 = q[FS33] + p;
    double dsq = 0.5 * (t11 * t11 + t22 * t22 + t33 * t33) + q[FS12] * q[FS12] + q[FS13] * q[FS13] +
                 q[FS23] * q[FS23];
    double val = sqrt(dsq);
    q[FSBAR] = val;
    return val;
}

/* calc_Lambda, calc_curly_c, calc_Dpl, calc_chi_F (shear_sim_3d.cpp:1170-1188, 1240-1244). */
static double lambda_(const adv_par_t *p, double chi) { return exp(-p->ez / chi); }

static double curly_c(const adv_par_t *p, double sbar) {
    double f1 = exp((p->omega * p->eps0 * sbar - p->delta) / p->bath_temp);
    double f2 = exp(-(p->omega * p->eps0 * sbar + p->delta) / p->bath_temp);
    return .5 * (f1 + f2);
}

static double dpl(const adv_par_t *p, double sbar, double chi) {
    return (sbar >= p->sy) ? lambda_(p, chi) * curly_c(p, sbar) * (1 - p->sy / sbar) / p->tau0 : 0;
}

static double chi_f(const adv_par_t *p, double d, double sbar, double chi) {
    return 2 * d * sbar * (p->chi_inf - chi) / (p->sy * p->c0);
}

/* adaptive_plastic_term (shear_sim_3d.cpp:108-147): sub-steps of at most
 * eta in the scaled plastic strain; adds the plastic change of chi to cchi
 * and returns 2 mu dt Dpl / sbar. */
static double adaptive_plastic_term(const adv_par_t *p, double *q, double dt) {
    const double eta = .0005;
    double tr = dt, ts;
    int keep = 1;
    double sbar0 = dev(q), chi0 = q[FCHI];
    double sbar = sbar0, chi = chi0;
    while (keep) {
        double d = dpl(p, sbar, chi);
        double dp = 2 * p->mu * d / p->sy;
        double F = chi_f(p, d, sbar, chi);
        if (dp * tr > eta) {
            ts = eta / fabs(dp);
            tr = tr - ts;
        } else {
            ts = tr;
            keep = 0;
        }
        sbar = sbar - ts * dp * p->sy;
        chi = chi + ts * F;
    }
    q[FCCHI] += (chi - chi0);
    return 1 - sbar / sbar0;
}

/* eno2 (shear_sim_3d.cpp:1256-1266). */
static double eno2(double h, double vel, double f2p, double fp, double f, double fm, double f2m) {
    double c2 = fabs(fp - 2 * f + fm);
    double fw2 = fabs(f2p - 2 * fp + f);
    double bk2 = fabs(f - 2 * fm + f2m);
    return .5 / h * (vel < 0 ? (c2 > fw2 ? -f2p + 4 * fp - 3 * f : fp - fm) : (c2 > bk2 ? 3 * f - 4 * fm + f2m : fp - fm));
}

/* chi_diffusion (shear_sim_3d.cpp:1216-1236) at point q. */
static double chi_diffusion(const ctx_t *c, const double *q) {
    const long X = FN, Y = c->nxg * FN, Z = c->nxyg * FN;
    double dD_dx = .5 * c->dx_inv * (q[X + FADPL] - q[-X + FADPL]);
    double dD_dy = .5 * c->dy_inv * (q[Y + FADPL] - q[-Y + FADPL]);
    double dD_dz = .5 * c->dz_inv * (q[Z + FADPL] - q[-Z + FADPL]);
    double dchi_dx = .5 * c->dx_inv * (q[X + FCHI] - q[-X + FCHI]);
    double dchi_dy = .5 * c->dy_inv * (q[Y + FCHI] - q[-Y + FCHI]);
    double dchi_dz = .5 * c->dz_inv * (q[Z + FCHI] - q[-Z + FCHI]);
    double ddx2 = c->dx_inv * c->dx_inv * (q[X + FCHI] - 2 * q[FCHI] + q[-X + FCHI]);
    double ddy2 = c->dy_inv * c->dy_inv * (q[Y + FCHI] - 2 * q[FCHI] + q[-Y + FCHI]);
    double ddz2 = c->dz_inv * c->dz_inv * (q[Z + FCHI] - 2 * q[FCHI] + q[-Z + FCHI]);
    double ddx = dD_dx * dchi_dx + q[FADPL] * ddx2;
    double ddy = dD_dy * dchi_dy + q[FADPL] * ddy2;
    double ddz = dD_dz * dchi_dz + q[FADPL] * ddz2;
    return c->p->diff_l * c->p->diff_l * (ddx + ddy + ddz);
}

/* advection_grid_step (shear_sim_3d.cpp:409-525) at point q. */
static void grid_step(const ctx_t *c, double *q, double dt, int *yielded) {
    const adv_par_t *p = c->p;
    const long X = FN, Y = c->nxg * FN, Z = c->nxyg * FN;
    double dx_dt = p->dx / dt, dy_dt = p->dy / dt, dz_dt = p->dz / dt;
    /* calculate_first_order_velocities (shear_sim_3d.cpp:900-917) */
#define D8(m, a, b, cc, d, e, f, g, h) \
    (q[a + m] - q[b + m] + q[cc + m] - q[d + m] + q[e + m] - q[f + m] + q[g + m] - q[h + m])
    double du_dx = .25 * c->dx_inv * D8(FU, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z);
    double dv_dx = .25 * c->dx_inv * D8(FV, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z);
    double dw_dx = .25 * c->dx_inv * D8(FW, X, 0, X + Y, Y, X + Z, Z, X + Y + Z, Y + Z);
    double du_dy = .25 * c->dy_inv * D8(FU, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z);
    double dv_dy = .25 * c->dy_inv * D8(FV, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z);
    double dw_dy = .25 * c->dy_inv * D8(FW, Y, 0, X + Y, X, Y + Z, Z, X + Y + Z, X + Z);
    double du_dz = .25 * c->dz_inv * D8(FU, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y);
    double dv_dz = .25 * c->dz_inv * D8(FV, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y);
    double dw_dz = .25 * c->dz_inv * D8(FW, Z, 0, X + Z, X, Y + Z, Y, X + Y + Z, X + Y);
#undef D8
    double sbar = dev(q);
    double adapt = (sbar > p->sy) ? adaptive_plastic_term(p, q, dt) : 0;
    if (adapt > 0) *yielded = 1;
    q[FADPL] = adapt / 2. / p->mu * sbar;
    /* staggered velocities: the mean of the cell's 8 nodes */
#define A8(m) (q[m] + q[X + m] + q[Z + m] + q[X + Z + m] + q[Y + m] + q[X + Y + m] + q[Y + Z + m] + q[X + Y + Z + m])
    double u = 0.125 * A8(FU), v = 0.125 * A8(FV), w = 0.125 * A8(FW);
#undef A8
#define ENO_X(m) eno2(dx_dt, u, q[2 * X + m], q[X + m], q[m], q[-X + m], q[-2 * X + m])
#define ENO_Y(m) eno2(dy_dt, v, q[2 * Y + m], q[Y + m], q[m], q[-Y + m], q[-2 * Y + m])
#define ENO_Z(m) eno2(dz_dt, w, q[2 * Z + m], q[Z + m], q[m], q[-Z + m], q[-2 * Z + m])
    double g[6];
    static const int S[6] = {FS11, FS12, FS13, FS22, FS23, FS33};
    for (int n = 0; n < 6; n++) {
        double a = ENO_X(S[n]), b = ENO_Y(S[n]), d = ENO_Z(S[n]);
        g[n] = u * a + v * b + w * d;
    }
    double third = 1. / 3.;
    double s11 = q[FS11], s12 = q[FS12], s13 = q[FS13], s22 = q[FS22], s23 = q[FS23], s33 = q[FS33];
    double t11 = s11 * (du_dx - dv_dy - dw_dz) + 2 * s13 * du_dz + 2 * s12 * du_dy;
    double t12 = s23 * du_dz + s13 * dv_dz - s12 * dw_dz + s22 * du_dy + s11 * dv_dx;
    double t13 = s33 * du_dz + s11 * dw_dx + s23 * du_dy + s12 * dw_dy - s13 * dv_dy;
    double t22 = 2 * s23 * dv_dz + s22 * (dv_dy - du_dx - dw_dz) + 2 * s12 * dv_dx;
    double t23 = s33 * dv_dz + s22 * dw_dy + s13 * dv_dx - s23 * du_dx + s12 * dw_dx;
    double t33 = s33 * (dw_dz - dv_dy - du_dx) + 2 * s23 * dw_dy + 2 * s13 * dw_dx;
    q[FCS11] = adapt * third * (s33 + s22 - 2 * s11) - g[0] + dt * t11;
    q[FCS12] = -adapt * s12 - g[1] + dt * t12;
    q[FCS13] = -adapt * s13 - g[2] + dt * t13;
    q[FCS22] = adapt * third * (s11 - 2 * s22 + s33) - g[3] + dt * t22;
    q[FCS23] = -adapt * s23 - g[4] + dt * t23;
    q[FCS33] = adapt * third * (s11 + s22 - 2 * s33) - g[5] + dt * t33;
    double dchi_dx = ENO_X(FCHI), dchi_dy = ENO_Y(FCHI), dchi_dz = ENO_Z(FCHI);
#undef ENO_X
#undef ENO_Y
#undef ENO_Z
    q[FCCHI] -= u * dchi_dx + v * dchi_dy + w * dchi_dz;
    q[FCCHI] += chi_diffusion(c, q) / p->c0;
}

/* advection_step (shear_sim_3d.cpp:393-405): every interior point in
 * z, y, x order, in place (a point's chi diffusion sees the new ad_Dpl of
 * the interior points before it in that order and the old one of the rest).
 * Returns 1 if some point reached the yield stress. */
int so_adv_step(double *fields, const adv_par_t *p, double dt) {
    ctx_t c;
    const int g = 2;
    c.p = p;
    c.dx_inv = 1. / p->dx;
    c.dy_inv = 1. / p->dy;
    c.dz_inv = 1. / p->dz;
    c.nxg = p->nx + 2 * g;
    c.nxyg = c.nxg * (p->ny + 2 * g);
    int yielded = 0;
    for (int k = 0; k < p->nz; k++)
        for (int j = 0; j < p->ny; j++)
            for (int i = 0; i < p->nx; i++) {
                long pt = (i + g) + c.nxg * (j + g) + c.nxyg * (k + g);
                grid_step(&c, fields + pt * FN, dt, &yielded);
            }
    return yielded;
}
