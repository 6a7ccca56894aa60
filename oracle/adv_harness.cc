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
// (:1961-2158) writes a Field member to a file.
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
