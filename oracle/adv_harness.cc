// CPU harness around the UNMODIFIED reference quasi-static advection step.
//
// Test infrastructure only: this file includes src/shear_sim_3d.cpp where it
// lies (that file itself includes mg_3d_template/region.cc and multigrid.cc)
// and is compiled with src/common.cpp, mg_3d_template/geometry.cc, common.cc,
// buffer.cc and the single-rank MPI shim into oracle/_ref/libstzadv.so.
// Python tests load it with ctypes to pin the C restatement of the step
// (oracle/stzadv_oracle.c) and to generate golden fixtures.  Nothing in the
// product links it.
//
// A shear_sim_3d<mat3> is built on a 1x1x1 process grid; its Field array
// (28 doubles per point, 2 ghost layers, shear_sim_3d.cpp:81-82) is filled
// from the caller, shear_sim_3d::advection_step (shear_sim_3d.cpp:393-405)
// runs once, and the array is copied back; shear_sim_3d::output_cube
// (:1961-2158) writes a Field member to a file; r_field
// (shear_sim_3d.hh:283-385) gives the solve's right-hand side of every node,
// and projection_step (shear_sim_3d.cpp:528-724) runs the whole quasi-static
// projection: multigrid solve and stress update.
#include <cstring>
#include <string>

#include "mpi.h"
#include "shear_sim_3d.cpp"

static_assert(sizeof(Field) == 28 * sizeof(double), "Field is 28 doubles");

namespace {

struct AdvProbe : public shear_sim_3d<mat3> {
    using shear_sim_3d<mat3>::shear_sim_3d;
    Field *points() { return grid; }
    size_t npoints() const { return (size_t)nxg * nyg * nzg; }
    void step(double dt) { advection_step(dt); }
    // Nodes the multigrid solves for (region.hh:805): N per periodic
    // dimension, N + 1 otherwise.
    int nodes(int N, bool prd) const { return prd ? N : N + 1; }
    // r_field (shear_sim_3d.hh:283-385) of every node, global = local indices
    // on one rank, after the ghost regions are filled.
    void rhs_all(double *out) {
        set_up_ghost_regions();
        const int nm = nodes(gN_x, x_period), nn = nodes(gN_y, y_period), no = nodes(gN_z, z_period);
        size_t p = 0;
        for (int k = 0; k < no; k++)
            for (int j = 0; j < nn; j++)
                for (int i = 0; i < nm; i++, p++) {
                    const vec3 v = r_field(i, j, k, 0, 0, 0);
                    out[3 * p] = v.x;
                    out[3 * p + 1] = v.y;
                    out[3 * p + 2] = v.z;
                }
    }
    // The quasi-static projection step (shear_sim_3d.cpp:528-724): stencil
    // for dt (solve_qs, :343-346), the multigrid solve for the velocities and
    // the stress update; returns the step's proj_mag, summed over the solved
    // velocities in the order of :683-704 with the simulation's own
    // calculate_first_order_velocities and sym_mat3::modsq.
    double project(double dt) {
        set_up_stencil_base(dt);
        set_up_stencil_and_matrices(dt);
        projection_step(dt);
        double du_dx, dv_dx, dw_dx, du_dy, dv_dy, dw_dy, du_dz, dv_dz, dw_dz, lproj = 0;
        me = grido;
        for (int kk = 0; kk < N_z; ++kk, me += 2 * nghost * nxg)
            for (int jj = 0; jj < N_y; ++jj, me += 2 * nghost)
                for (int ii = 0; ii < N_x; ++ii, me++) {
                    calculate_first_order_velocities(du_dx, dv_dx, dw_dx, du_dy, dv_dy, dw_dy, du_dz, dv_dz, dw_dz);
                    const double ds11 = dt * (lamb * (dw_dz + dv_dy) + (lamb + 2 * mu) * du_dx);
                    const double ds12 = dt * mu * (du_dy + dv_dx);
                    const double ds13 = dt * mu * (du_dz + dw_dx);
                    const double ds22 = dt * (lamb * (dw_dz + du_dx) + (lamb + 2 * mu) * dv_dy);
                    const double ds23 = dt * mu * (dv_dz + dw_dy);
                    const double ds33 = dt * (lamb * (dv_dy + du_dx) + (lamb + 2 * mu) * dw_dz);
                    sym_mat3 d(ds11, ds12, ds13, ds22, ds23, ds33);
                    lproj += d.modsq();
                }
        return lproj;
    }
};

// The simulation keeps pointers to its communicator and process-grid
// dimensions (parallel_info.hh:93), so they live as long as it does.
struct Handle {
    MPI_Comm comm;
    int dims[3], periods[3];
    AdvProbe *sim;
};

}  // namespace

extern "C" {

// p: mu, lamb, sy, tau0, c0, eps0, delta, omega, bath_temp, chi_inf, ez, diff_l.
// Cells of size (lx/nx, ly/ny, lz/nz); x and y periodic, z periodic if zper;
// output_cube writes into the folder outdir.
void *adv_new(int nx, int ny, int nz, double lx, double ly, double lz, const double *p, int zper,
              const char *outdir) {
    Handle *h = new Handle;
    int *dims = h->dims, *periods = h->periods;
    dims[0] = dims[1] = dims[2] = 1;
    periods[0] = periods[1] = 1;
    periods[2] = zper;
    MPI_Cart_create(MPI_COMM_WORLD, 3, dims, periods, 0, &h->comm);
    h->sim = new AdvProbe(nx, ny, nz, 0.0, 0.0, 0.0, lx, ly, lz,
                          /*t0*/ 0.0, /*tf*/ 1.0, /*tmult*/ 1.0, /*N_tp*/ 1, std::string(outdir),
                          /*mu*/ p[0], /*lamb*/ p[1], /*rho*/ 1.0, /*kap*/ 0.0, /*sy*/ p[2], /*tau0*/ p[3],
                          /*c0*/ p[4], /*eps0*/ p[5], /*delta*/ p[6], /*omega*/ p[7], /*bath_temp*/ p[8],
                          /*chi_inf*/ p[9], /*ez*/ p[10], /*TZ*/ 1.0, /*diff_l*/ p[11], /*U*/ 0.0,
                          /*gauss_fac*/ 1.0, /*conv_l*/ 1.0, /*chi_avg*/ 0.0, /*sigma*/ 1.0, /*zeta*/ 0.0,
                          &h->comm, dims, /*sim_case*/ 0, /*om*/ 0.0, /*rsq*/ 0.0, periods);
    return h;
}

long adv_npoints(void *hh) { return (long)static_cast<Handle *>(hh)->sim->npoints(); }

void adv_set(void *hh, const double *fields) {
    AdvProbe *s = static_cast<Handle *>(hh)->sim;
    std::memcpy(static_cast<void *>(s->points()), fields, s->npoints() * sizeof(Field));
}

void adv_get(void *hh, double *fields) {
    AdvProbe *s = static_cast<Handle *>(hh)->sim;
    std::memcpy(fields, static_cast<const void *>(s->points()), s->npoints() * sizeof(Field));
}

void adv_step(void *hh, double dt) { static_cast<Handle *>(hh)->sim->step(dt); }

// r_field of every node (3 doubles per node, natural order) from the Field
// array's stresses; fills the array's ghost regions first.
void adv_rhs(void *hh, double *out) { static_cast<Handle *>(hh)->sim->rhs_all(out); }

// One quasi-static projection step of length dt on the Field array (solved
// velocities and updated stresses stay in it); returns proj_mag.
double adv_project(void *hh, double dt) { return static_cast<Handle *>(hh)->sim->project(dt); }

// shear_sim_3d::output_cube (shear_sim_3d.cpp:1961-2158) of Field member `mode`.
void adv_output_cube(void *hh, const char *prefix, int mode, int frame) {
    static_cast<Handle *>(hh)->sim->output_cube(prefix, mode, frame);
}

void adv_free(void *hh) {
    Handle *h = static_cast<Handle *>(hh);
    delete h->sim;
    delete h;
}

}  // extern "C"
