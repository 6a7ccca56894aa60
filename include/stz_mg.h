/* stz_mg -- GB300 multigrid for the quasi-static projection solve.
 *
 * C-ABI drop-in for the reference's templated multigrid (nmboffi/stzpp,
 * mg_3d_template) instantiated as multigrid<vec3, M> with M = mat3 or
 * sym_mat3.  The reference's interface is a compile-time duck-typed contract;
 * each entry point below names the member it replaces (paths relative to the
 * reference checkout).  Plain pointers and sizes only; no CUDA or torch types.
 *
 * Data layout at this boundary is the reference's: nodes in natural order
 * (x fastest, index i + m*(j + n*k)), vec3 fields as 3 consecutive doubles
 * per node (region::r0 / x0 without ghosts, region.hh:75-83), 3x3 blocks as 9
 * doubles row-major (mat3, mg_3d_template/mat3.hh), a node's 27 blocks in the
 * stencil order b = (dx+1) + 3(dy+1) + 9(dz+1) of shear_sim_3d.cpp:224.
 *
 * Every function returns STZ_MG_OK (0) or an error code; the message of the
 * last error on the calling thread is stz_mg_last_error().  The reference
 * aborts the MPI job instead (p_fatal_error, common.cc:52).  A handle is not
 * thread safe; all work of a handle runs on its CUDA stream.
 *
 * Device pointers (where = STZ_MG_DEVICE): the caller's writes to an input
 * must be complete before the call (synchronise the stream that produced
 * it), and every call that reads or writes caller memory synchronises the
 * handle's stream before it returns, so inputs may be freed or reused and
 * outputs read on any stream as soon as the call returns.
 */
#ifndef STZ_MG_H
#define STZ_MG_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    STZ_MG_OK = 0,
    STZ_MG_ERR_ARG = 1,         /* bad argument or call order */
    STZ_MG_ERR_CUDA = 2,        /* CUDA runtime failure */
    STZ_MG_ERR_UNSUPPORTED = 3, /* grid shape the GPU path does not support */
    STZ_MG_ERR_NOCONV = 4,      /* max_cycles reached above tolerance */
    STZ_MG_ERR_SINGULAR = 5,    /* singular diagonal block or bottom matrix */
    STZ_MG_ERR_NONFINITE = 6,   /* NaN/Inf in inputs or iterates */
    STZ_MG_ERR_OOM = 7          /* device allocation failed */
};

enum { STZ_MG_FP64 = 0, STZ_MG_MIXED = 1 };          /* precision */
enum { STZ_MG_BOTTOM_DIRECT = 0, STZ_MG_BOTTOM_GS = 1 };
enum { STZ_MG_HOST = 0, STZ_MG_DEVICE = 1 };        /* where a pointer lives */
enum { STZ_MG_FIELD_X = 0, STZ_MG_FIELD_R = 1, STZ_MG_FIELD_RES = 2 };   /* a level's x, r, residual work field */

typedef struct stz_mg_handle_s *stz_mg_handle;

/* Problem and solver description.  m, n, o and the periodicity replace the
 * geometry / sim fields the region ctor reads (region.hh:663-700, 792-830):
 * a periodic dimension with N cells has N nodes, a non-periodic one N+1. */
typedef struct {
    int m, n, o;
    int x_prd, y_prd, z_prd;
    int precision;      /* STZ_MG_FP64 or STZ_MG_MIXED (FP32 cycles inside FP64 defect correction; the
                         * correction's residual of a shared-stencil top level is formed in double-float
                         * arithmetic from the FP64 x and b, to about 1e-13 of sum |a x| per row;
                         * STZ_MG_DF=0 in the environment forms it in FP64.  Mixed precision needs
                         * b, x and A x inside FP32's normal range: above it the solve stops with
                         * STZ_MG_ERR_NONFINITE, below it values count as zero) */
    int v_down, v_up;   /* sweeps per level: v_down+i down, v_up+i-1 up (multigrid.hh:123, multigrid.cc:265,288) */
    int max_coarse;     /* coarsen while the coarsest level has more nodes (reference: 1024, multigrid.cc:40) */
    int bottom;         /* STZ_MG_BOTTOM_DIRECT (FP64 dense solve) or STZ_MG_BOTTOM_GS */
    int bottom_sweeps;  /* sweeps of the GS bottom solve (reference: 24, common.hh:57) */
    int sweep_growth;   /* 1: v_down+i / v_up+i-1 sweeps on level i as the reference; 0: v_down / v_up on every level */
    int device;         /* CUDA device ordinal */
    void *stream;       /* cudaStream_t to run on, or NULL for a handle-owned stream */
} stz_mg_desc;

/* Defaults: FP64, v_down = v_up = 2 with the reference's growth, max_coarse =
 * 1024 (the reference's hierarchy), direct bottom, 24 bottom sweeps, device 0,
 * own stream. */
void stz_mg_desc_default(stz_mg_desc *d);

const char *stz_mg_last_error(void);

/* multigrid(sim, comm_buffer) / multigrid(pr, gm, com) (multigrid.hh:126-189):
 * builds the level hierarchy (setup_hierarchy, multigrid.cc:19-132). */
int stz_mg_create(const stz_mg_desc *desc, stz_mg_handle *out);
int stz_mg_destroy(stz_mg_handle h);

/* Shared stencil of interior nodes and `fix` block of Dirichlet nodes: the
 * external_ptr path (shear_sim_3d.hh:388-402; stencil/fix set up by
 * set_up_stencil_and_matrices, shear_sim_3d.hh:45-55).  27*9 and 9 doubles. */
int stz_mg_set_stencil_const(stz_mg_handle h, const double *stencil, const double *fix);

/* Per-node stencils, npts*27*9 doubles (a Dirichlet node uses block 13 only):
 * the internal()/mem_size()/fill_entries() path (region.hh:196-206). */
int stz_mg_set_stencil_points(stz_mg_handle h, const double *A, int where);

/* Variable-coefficient operator -dt*div(mu(grad u + grad u^T) + lam div(u) I)
 * from per-node mu, lambda (npts doubles each), applied matrix-free on the
 * top level.  With constant mu, lambda it is the stencil of
 * shear_sim_3d::set_up_stencil_base (shear_sim_3d.cpp:215-331). */
int stz_mg_set_coeffs_lame(stz_mg_handle h, const double *mu, const double *lam, double dx, double dy,
                           double dz, double dt, int where);

/* multigrid::setup_matrices -> compute_rats (multigrid.hh:194-198,
 * multigrid.cc:330-344): Galerkin coarse operators on every level.  Call again
 * after a coefficient change. */
int stz_mg_setup(stz_mg_handle h);

/* multigrid::setup_fields (region.hh:209-241): right-hand side and initial
 * guess, 3*npts doubles. */
int stz_mg_set_rhs(stz_mg_handle h, const double *r, int where);
int stz_mg_set_x(stz_mg_handle h, const double *x, int where);
/* The solution, read by the drivers through reg[0]->x0 (shear_sim_3d.cpp:616-674). */
int stz_mg_get_x(stz_mg_handle h, double *x, int where);
int stz_mg_get_rhs(stz_mg_handle h, double *r, int where);

/* Right-hand side assembled on the device from a cell-centred symmetric
 * tensor field: the r_field of shear_sim_3d (shear_sim_3d.hh:283-385, plates
 * at rest) using calculate_first_order_stresses (shear_sim_3d.cpp:979-998).
 * eps holds 6 doubles per cell (s11 s12 s13 s22 s23 s33), cells in natural
 * order; a periodic dimension has as many cells as nodes, a non-periodic one
 * one fewer.  Dirichlet nodes get 0. */
int stz_mg_set_rhs_divergence(stz_mg_handle h, const double *eps, double dx, double dy, double dz, int where);

/* Projection-step stress update after the solve (shear_sim_3d::projection_step,
 * shear_sim_3d.cpp:681-710): for every cell, the velocity derivatives of
 * calculate_first_order_velocities (shear_sim_3d.cpp:901-916) from the
 * handle's current solution x, the increment ds = dt (lam tr(grad u) I +
 * mu (grad u + grad u^T)) added to the cell's stress sigma in place, and
 * *proj_mag = sum over cells of sym_mat3::modsq(ds) (mat3.hh:338-340; may be
 * NULL).  sigma holds 6 doubles per cell (s11 s12 s13 s22 s23 s33), cells as
 * for stz_mg_set_rhs_divergence; constant lam, mu.  The plates' velocities are
 * the solved ones (x = fix^-1 b on the Dirichlet nodes). */
int stz_mg_stress_update(stz_mg_handle h, double *sigma, double lam, double mu, double dt, double dx, double dy,
                         double dz, double *proj_mag, int where);

/* multigrid::v_cycle (multigrid.cc:253-297).  In mixed precision one call is
 * one defect-correction step: top-level residual, one FP32 V-cycle, FP64
 * update. */
int stz_mg_vcycle(stz_mg_handle h);

/* V-cycles until |b - A x|_2 <= rel_tol |b|_2 (the loop of
 * shear_sim_3d::projection_step, shear_sim_3d.cpp:567-582, with the true
 * residual norm).  cycles = V-cycles run, relres = final relative residual;
 * STZ_MG_ERR_NOCONV when max_cycles is reached first. */
int stz_mg_solve(stz_mg_handle h, double rel_tol, int max_cycles, int *cycles, double *relres);

/* Counters of the last stz_mg_solve: V-cycles, top-level residual
 * evaluations, and kernels this library launched (no counterpart in the
 * reference; its drivers time v_cycle only, shear_sim_3d.cpp:568-571). */
int stz_mg_solve_stats(stz_mg_handle h, int *vcycles, int *residuals, long long *kernel_launches);

/* |b - A x|_2 and |b|_2 in FP64 on the top level. */
int stz_mg_residual_norm(stz_mg_handle h, double *rnorm, double *bnorm);

/* region::l2_error_all (region.cc:3030-3057) as shipped: for V = vec3 the
 * reference sums |r|^4 (its mg3d_mod_sq squares the vec3 -> double cast). */
int stz_mg_l2_error_all(stz_mg_handle h, double *out);

/* Adjoint of the projection solve (no counterpart in the reference, whose
 * solver is not differentiated).  For a scalar loss L(u) with u = A^{-1} b:
 *   dL/db = w with A^T w = g, g = dL/du,
 *   dL/dmu_p, dL/dlam_p = -w^T (dA/dmu_p) u, -w^T (dA/dlam_p) u.
 *
 * stz_mg_adjoint_solve solves A^T w = g (npts*3 doubles in natural order,
 * from/to host or device memory per `where`) for a top-level operator set by
 * stz_mg_set_stencil_const (symmetric blocks, S[d] = S[-d]^T, as the
 * elasticity stencil of shear_sim_3d.cpp:215-331) or stz_mg_set_coeffs_lame.
 * The interior block of such an A is symmetric, so the interior part of w is
 * the handle's own V-cycle solve of A y = g with g zeroed on the Dirichlet
 * nodes (rel_tol, max_cycles, cycles, relres as in stz_mg_solve, relative to
 * that masked g); the Dirichlet part follows from F^T w_D = g_D - A_ID^T w_I.
 * It overwrites the handle's x and right-hand side (save u first).
 *
 * stz_mg_coeff_grad contracts w and u (npts*3 each) into dmu, dlam (npts
 * each) for the Lame operator of stz_mg_set_coeffs_lame, with the same
 * discretisation the solver applies (face-midpoint averages, node values on
 * the edge terms, the fix blocks of the Dirichlet nodes).  It does not solve
 * anything and leaves x and the right-hand side alone. */
int stz_mg_adjoint_solve(stz_mg_handle h, const double *g, double *w, int where, double rel_tol, int max_cycles,
                         int *cycles, double *relres);
int stz_mg_coeff_grad(stz_mg_handle h, const double *w, const double *u, double *dmu, double *dlam, int where);

/* Level-wise operations on the FP64 hierarchy, the region members the
 * reference's multigrid class calls (used for parity checks). */
int stz_mg_num_levels(stz_mg_handle h, int *nlevels);
int stz_mg_level_dims(stz_mg_handle h, int level, int *dims3);
/* Coefficients as npts*27*9 doubles (zero outside each node's box) and box
 * bounds S as npts*6 ints (region::S, region.hh:337-344); either may be NULL. */
int stz_mg_level_operator(stz_mg_handle h, int level, double *A, int *S);
int stz_mg_level_set_field(stz_mg_handle h, int level, int which, const double *v, int where);
int stz_mg_level_get_field(stz_mg_handle h, int level, int which, double *v, int where);
/* region::gauss_seidel (region.cc:1557), 8-colour order */
int stz_mg_level_gauss_seidel(stz_mg_handle h, int level, int sweeps);
/* multigrid::restriction(level) (multigrid.cc:436-449): coarse r from the residual of level-1, coarse x = 0 */
int stz_mg_level_restriction(stz_mg_handle h, int level);
/* multigrid::interpolation(level) (multigrid.cc:418-430): x(level-1) += P x(level) */
int stz_mg_level_interpolation(stz_mg_handle h, int level);
/* region::residual (region.cc:1008) of every node, 3*npts doubles (may be NULL), and sum |r|^2 */
int stz_mg_level_residual(stz_mg_handle h, int level, double *out, double *sumsq, int where);

/* Pieces of a decomposed sweep and transfer, for callers that split the grid
 * over several handles (stzpp_gb300/slabs.py: z-slabs exchanging ghost planes,
 * the reference's MPI decomposition of region.cc:2759-2910).
 * z-planes k0 .. k0+nk-1 of a level's field (STZ_MG_FIELD_X, _R or _RES) to or
 * from 3*m*n*nk doubles in natural order (x fastest) -- the planes a
 * neighbour sub-domain needs (region::communicate, region.cc:2759-2847). */
int stz_mg_level_get_planes(stz_mg_handle h, int level, int which, int k0, int nk, double *v, int where);
int stz_mg_level_set_planes(stz_mg_handle h, int level, int which, int k0, int nk, const double *v, int where);
/* Colour passes q0 .. q1-1 of the 8-colour Gauss-Seidel sweep of a level (FP64);
 * a sweep split where a sub-domain exchanges its ghost planes. */
int stz_mg_level_gs_colours(stz_mg_handle h, int level, int q0, int q1);
/* multigrid::restriction (multigrid.cc:436-449) from the level-1 residual
 * field as it stands (STZ_MG_FIELD_RES, e.g. with ghost planes filled in by a
 * neighbour) instead of recomputing it; coarse x = 0. */
int stz_mg_level_restrict_residual(stz_mg_handle h, int level);

/* Measurement hook (no counterpart in the reference): launches one kernel of
 * the solver `reps` times on the handle's stream between CUDA events and
 * returns the average time per launch and the algorithmic bytes (or FP64
 * flops for STZ_MG_K_RESIDUAL64) one launch moves.  Overwrites the level's
 * work fields.  Kernels run in the handle's solver precision. */
enum {
    STZ_MG_K_GS_COLOUR = 0,   /* one colour pass of the smoother (colour 0) */
    STZ_MG_K_RESIDUAL = 1,    /* residual of a level */
    STZ_MG_K_RESTRICT = 2,    /* restriction into `level` */
    STZ_MG_K_INTERP = 3,      /* interpolation from `level` */
    STZ_MG_K_RESIDUAL64 = 4,  /* FP64 top-level residual of the defect correction */
    STZ_MG_K_GS_SWEEP = 5     /* two full smoother sweeps of a level (one smoothing step of the cycle) */
};
int stz_mg_time_kernel(stz_mg_handle h, int kernel, int level, int reps, double *ms_per_launch,
                       double *work_per_launch);
/* Measurement hook (no counterpart in the reference): how the solver sweeps
 * a level in its precision -- STZ_MG_SWEEP_COLOUR (eight colour launches per
 * sweep), _TILE (two-buffer tiles), _BAND (full-width bands staged by TMA),
 * _PHASE (a block per plane) -- and the kernel launches of one sweep. */
enum { STZ_MG_SWEEP_COLOUR = 0, STZ_MG_SWEEP_TILE = 1, STZ_MG_SWEEP_BAND = 2, STZ_MG_SWEEP_PHASE = 3 };
int stz_mg_sweep_kind(stz_mg_handle h, int level, int *kind, int *launches_per_sweep);

/* Allocation-free residual check (no counterpart in the reference).
 *
 * Computes sum over nodes of |b - A x|^2, where A is one shared 27-block
 * stencil on interior nodes and one fix block on Dirichlet nodes (the
 * external_ptr form of shear_sim_3d.hh:401-402; same stencil and fix layout as
 * stz_mg_set_stencil_const), for fields x and b that the caller already holds
 * on `device` in the natural layout (3 doubles per node, node
 * i + m*(j + n*k)).  The result is stored, not accumulated, into the device
 * double *sumsq; the kernels are queued on `stream` (a cudaStream_t of that
 * device, NULL for the legacy default stream) and the call returns without
 * waiting for them.  No handle is needed.
 *
 * It is meant for callers that must not allocate at the point of the check:
 * cudaMalloc and cudaFree can synchronise the whole device, stalling the
 * caller's work in flight on other streams, and an allocation can fail when
 * the caller's own fields already fill the GPU's memory.  The call allocates
 * nothing (no cudaMalloc, no cudaFree, no pinned host memory): its partial
 * sums live in a fixed device array of STZ_MG_NOALLOC_PARTIALS doubles
 * (1 MiB) compiled into the library, which limits it to grids of at most
 * STZ_MG_NOALLOC_MAX_NODES nodes; larger grids get STZ_MG_ERR_ARG and
 * stz_mg_residual_norm does the job.  No memory has to start at zero.
 *
 * All calls on one device share that array: calls whose kernels may run at
 * the same time on one device (different streams, or host threads without
 * ordering) race and corrupt each other's results, so keep them on one stream
 * or order them with events.  The first call on a device looks up the array's
 * device address (once per device); make that first call before any stream
 * capture begins, and do not reset the device (cudaDeviceReset) between
 * calls: the address kept from the first call would no longer be valid.  A
 * stream of another device than `device` is refused with STZ_MG_ERR_ARG. */
#define STZ_MG_NOALLOC_PARTIALS 131072
#define STZ_MG_NOALLOC_MAX_NODES (1024LL * STZ_MG_NOALLOC_PARTIALS)
int stz_mg_const_residual_sumsq_noalloc(int m, int n, int o, int x_prd, int y_prd, int z_prd,
                                        const double *stencil, const double *fix, const double *x,
                                        const double *b, double *sumsq, int device, void *stream);

/* ------------------------------------------------------------------------
 * Quasi-static advection step (shear_sim_3d::advection_step,
 * src/shear_sim_3d.cpp:393-525, with advection_grid_step :409-525,
 * adaptive_plastic_term :108-147, chi_diffusion :1216-1236, eno2
 * :1256-1266): the part of step_forward_qs (:381-389) before merge_updates and
 * the projection solve, on the device.
 *
 * Every field is a device array over the reference's ghosted grid of
 * (nx + 4) x (ny + 4) x (nz + 4) points (nghost = 2, shear_sim_3d.cpp:39-49,
 * 81-82), x fastest, one array per Field member (src/field.hh:11-22); the
 * ghost layers are inputs, filled by the caller as set_up_ghost_regions and
 * set_boundary_conditions fill them.  For every interior point the step
 * writes sbar (Field::dev), the stress changes cs11..cs33, adds the chi
 * change to cchi (the reference's +=) and replaces ad_Dpl; a point's chi
 * diffusion sees the new ad_Dpl of its interior -x, -y, -z neighbours and the
 * old one of the others, as the reference's in-place sweep does.
 * work: 2 x (ghosted points) + 2 doubles of scratch.  Asynchronous on
 * `stream` (a cudaStream_t, NULL: the default stream) unless yielded is
 * non-NULL: then the call waits and sets *yielded to 1 if some point reached
 * the yield stress (the reference's "Starting to reach the yield stress"
 * message), and returns STZ_MG_ERR_NONFINITE if a point's adaptive plastic
 * sub-stepping did not finish within 2^22 sub-steps. */
typedef struct {
    int nx, ny, nz;     /* interior points */
    double dx, dy, dz;  /* grid spacing */
    /* STZ parameters (shear_sim_3d.hh:120-136) */
    double mu, sy, tau0, eps0, c0, delta, omega, bath_temp, chi_inf, ez, diff_l;
} stz_adv_params;

typedef struct {
    const double *u, *v, *w;                       /* node velocities */
    const double *s11, *s12, *s13, *s22, *s23, *s33; /* cell stresses */
    const double *chi;                             /* effective temperature */
    double *ad_dpl;                                /* in: previous step (every point); out: interior */
    double *sbar;                                  /* out */
    double *cs11, *cs12, *cs13, *cs22, *cs23, *cs33; /* out: stress changes */
    double *cchi;                                  /* in/out: chi change */
    double *work;                                  /* scratch */
} stz_adv_fields;

int stz_mg_advection_step(const stz_adv_params *p, const stz_adv_fields *f, double dt, void *stream, int *yielded);

/* ------------------------------------------------------------------------
 * Output in the reference's file formats, values made on the device.
 *
 * region::output_x / output_r / output_residual of the top level
 * (mg_3d_template/region.cc:3062-3120) through region::output_internal
 * (region.cc:3135-3202): the z-slice k of the solution x, the right-hand side
 * r or the residual b - A x, written to `filename` as floats: {m, ax + i dx
 * (i < m)}, then per row j {ay + j dy, m values}, dx = (bx-ax)/(m-1), dy =
 * (by-ay)/(n-1) (the reference's default box is (0, m-1, 0, n-1)).  As in the
 * reference, a vec3 value goes through vec3::operator double (src/vec3.hh:110,
 * the squared magnitude): x and r slices hold float(|v|^2), the residual
 * slice float(|r|^2 |r|^2). */
enum { STZ_MG_SLICE_X = 0, STZ_MG_SLICE_R = 1, STZ_MG_SLICE_RESIDUAL = 2 };
int stz_mg_output_slice(stz_mg_handle h, int which, int k, double ax, double bx, double ay, double by,
                        const char *filename);

/* shear_sim_3d::output_cube (src/shear_sim_3d.cpp:1961-2158) for one process:
 * Field member `mode` (Field::fval, src/field.hh:157-177: 0-2 u v w, 3-8
 * s11 s12 s13 s22 s23 s33, 9 pressure, 10 deviatoric stress, 11 chi,
 * 12 chi*21000, 13-15 the reference map) of every interior point, x slowest
 * and z fastest, as floats; the node-based members (0-2, 13-15) include the
 * top z node (nz + 1 values per column).  Fields are device arrays over the
 * ghosted grid of stz_mg_advection_step; members the mode does not read may
 * be NULL.  stz_mg_cube_values writes the values to the device array `out`
 * (asynchronous on `stream`); stz_mg_output_cube appends them to
 * <dir>/<prefix>_grid.<frame>, creating dir if needed, as the reference does.
 * Unlike the reference, mode 10 does not store sbar in the Field. */
typedef struct {
    const double *u, *v, *w;
    const double *s11, *s12, *s13, *s22, *s23, *s33;
    const double *chi;
    const double *xi_x, *xi_y, *xi_z;
} stz_cube_fields;

int stz_mg_cube_values(const stz_cube_fields *f, int nx, int ny, int nz, int mode, float *out, void *stream);
int stz_mg_output_cube(const stz_cube_fields *f, int nx, int ny, int nz, int mode, const char *dir,
                       const char *prefix, int frame);

#ifdef __cplusplus
}
#endif
#endif
