/* C restatement of the reference multigrid for V=vec3, M=mat3 on one rank.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): used by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU baseline.  It
 * is never linked into the product library.
 *
 * It restates, function by function, mg_3d_template/{region,multigrid}.cc for
 * a single process: the ghost/strip MPI exchanges of the reference become
 * periodic index wrapping, with the same lagged-ghost semantics in the
 * Gauss-Seidel sweep (ghosts refreshed once per sweep, region.cc:1600).
 * Parity with the compiled reference (oracle/_ref) is checked by the CPU
 * tests: box bounds exactly, coefficients and iterates to round-off. */
#ifndef STZMG_ORACLE_H
#define STZMG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

const char *so_last_error(void);

/* stencil: 27x9 shared interior stencil, fix: 9 (Dirichlet rows) -- the
 * external_ptr path; or pts: npts x 27 x 9 per-point stencils (boundary
 * points use block 13) -- the internal()/fill_entries path.
 * max_coarse: coarsen while the coarsest level has more points (1024 in the
 * reference, multigrid.cc:40). */
int so_create(int m, int n, int o, int xp, int yp, int zp, const double *stencil,
              const double *fix, const double *pts, int max_coarse, void **out);
void so_destroy(void *h);
int so_num_levels(void *h);
int so_level_dims(void *h, int l, int *dims);
int so_level_S(void *h, int l, int *S);
int so_level_A(void *h, int l, double *A27);
int so_set_field(void *h, int l, int which, const double *v);
int so_get_field(void *h, int l, int which, double *v);
/* smoother: 0 = lexicographic (reference), 1 = 8-colour parity order */
int so_gauss_seidel(void *h, int l, int sweeps, int smoother);
int so_restriction(void *h, int l);
int so_interpolation(void *h, int l);
/* bottom: 0 = 24 Gauss-Seidel sweeps (reference solve_exact), 1 = dense LU */
int so_vcycle(void *h, int smoother, int bottom);
int so_residual(void *h, int l, double *out, double *sq);
int so_solve(void *h, double tol, int max_cycles, int smoother, int bottom, int *cycles,
             double *hist);
int so_set_cycle(void *h, int v_down, int v_up, int bottom_sweeps, int grow);
/* Host threads for every handle (default 1, the serial restatement): P > 1
 * runs each level as min(P, o/8) z-slab sub-domains, one thread each, with
 * the reference's per-sweep ghost refresh at the slab faces (its MPI
 * decomposition along z); transfers, residuals and RAT run their planes in
 * parallel.  so_threads() is the count in effect (1 without OpenMP). */
void so_set_threads(int n);
int so_threads(void);

#ifdef __cplusplus
}
#endif
#endif
