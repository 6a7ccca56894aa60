/* CPU restatement of the quasi-static advection step (test infrastructure only). */
#ifndef STZADV_ORACLE_H
#define STZADV_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Interior cells nx x ny x nz of spacing dx, dy, dz and the STZ parameters
 * of shear_sim_3d (shear_sim_3d.hh:120-136). */
typedef struct {
    int nx, ny, nz;
    double dx, dy, dz;
    double mu, sy, tau0, eps0, c0, delta, omega, bath_temp, chi_inf, ez, diff_l;
} adv_par_t;

int so_adv_step(double *fields, const adv_par_t *p, double dt);

#ifdef __cplusplus
}
#endif

#endif
