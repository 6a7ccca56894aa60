// Drives the GPU multigrid through include/stz_mg_multigrid.hh the way the
// reference's shear_sim_3d drives multigrid<vec3, M>: a simulation-like class
// with the duck-typed problem contract (shared stencil on interior nodes, a
// fix block on the Dirichlet plates), setup_matrices / setup_fields /
// v_cycle, and the solution read through reg[0]->x0.  The value types are
// minimal stand-ins with the member names of the reference's vec3, mat3 and
// sym_mat3.  Prints "cycles relres checksum" for each matrix type; with a
// second argument, also writes the right-hand side and the mat3 solution
// there as raw doubles (node-major, x fastest) for comparison with the oracle.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "stz_mg_multigrid.hh"

struct vec3 {
    double x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(double a, double b, double c) : x(a), y(b), z(c) {}
};
struct mat3 {
    double a11, a12, a13, a21, a22, a23, a31, a32, a33;
};
struct sym_mat3 {
    double a11, a12, a13, a22, a23, a33;
};

template <class M>
M make_block(const double *b);
template <>
mat3 make_block<mat3>(const double *b) {
    return mat3{b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8]};
}
template <>
sym_mat3 make_block<sym_mat3>(const double *b) {
    return sym_mat3{b[0], b[1], b[2], b[4], b[5], b[8]};
}

// elasticity stencil of set_up_stencil_base with kappa = 0, stencil = -dt*base
void elastic(double mu, double lam, double h, double dt, double *st, double *fix) {
    std::memset(st, 0, 243 * sizeof(double));
    auto B = [&](int dx, int dy, int dz) { return st + 9 * (13 + dx + 3 * dy + 9 * dz); };
    const double h2 = h * h, lm = (lam + mu) / (4 * h2);
    for (int ax = 0; ax < 3; ax++)
        for (int s = -1; s <= 1; s += 2) {
            int d[3] = {0, 0, 0};
            d[ax] = s;
            double *b = B(d[0], d[1], d[2]);
            for (int c = 0; c < 3; c++) b[4 * c] = -dt * ((c == ax ? lam + 2 * mu : mu) / h2);
        }
    double *c = B(0, 0, 0);
    for (int r = 0; r < 3; r++) c[4 * r] = dt * 2 * ((lam + 2 * mu) / h2 + 2 * mu / h2);
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto &p : pr)
        for (int sr = -1; sr <= 1; sr += 2)
            for (int sc = -1; sc <= 1; sc += 2) {
                int d[3] = {0, 0, 0};
                d[p[0]] = sr;
                d[p[1]] = sc;
                double *b = B(d[0], d[1], d[2]);
                b[3 * p[0] + p[1]] = b[3 * p[1] + p[0]] = -dt * sr * sc * lm;
            }
    std::memset(fix, 0, 9 * sizeof(double));
    fix[0] = fix[4] = fix[8] = -dt * 2 * ((lam + 2 * mu) / h2 + 2 * mu / h2);
}

template <class M>
struct sim {
    int gN_x, gN_y, gN_z;
    bool x_period = true, y_period = true, z_period = false;
    M stencil[27], fix[1];
    std::vector<vec3> rhs;
    sim(int N) : gN_x(N), gN_y(N), gN_z(N) {
        double st[243], fx[9];
        elastic(1.0, 2.0, 1.0 / N, 1.0, st, fx);
        for (int b = 0; b < 27; b++) stencil[b] = make_block<M>(st + 9 * b);
        fix[0] = make_block<M>(fx);
        std::mt19937_64 rng(7);
        std::normal_distribution<double> g(0.0, 1.0);
        rhs.resize((size_t)N * N * (N + 1));
        for (size_t p = 0; p < rhs.size(); p++) {
            int k = p / ((size_t)N * N);
            rhs[p] = (k == 0 || k == N) ? vec3() : vec3(g(rng), g(rng), g(rng));
        }
    }
    bool interior(int, int, int k) { return k != 0 && k != gN_z; }
    int range_xd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    int range_xu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    int range_yd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    int range_yu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    int range_zd(int i, int j, int k) { return interior(i, j, k) ? -1 : 0; }
    int range_zu(int i, int j, int k) { return interior(i, j, k) ? 2 : 1; }
    bool internal(int, int, int) { return false; }
    int mem_size(int, int, int) { return 0; }
    M *external_ptr(int i, int j, int k) { return interior(i, j, k) ? stencil : fix; }
    void fill_entries(int, int, int, M *&) {}
    vec3 x_field(int, int, int, int, int, int) { return vec3(); }
    vec3 r_field(int i, int j, int k, int, int, int) { return rhs[i + gN_x * ((size_t)j + gN_y * k)]; }
};

template <class M>
int run(int N, const char *dump) {
    sim<M> s(N);
    stz_mg::multigrid_gpu<vec3, M> mgrid(s);
    mgrid.setup_matrices(s);
    mgrid.setup_fields(s);
    // the projection_step loop: v_cycle until the residual is small
    double rel = 1;
    int cycles = mgrid.solve(1e-10, 100, &rel);
    mgrid.v_cycle();   // "a few more for good measure" (shear_sim_3d.cpp:599)
    const stz_mg::top_region<vec3> *top = mgrid.reg[0];
    double cs = 0;
    for (int k = 0; k <= N; k++)
        for (int j = 0; j < N; j++)
            for (int i = 0; i < N; i++) {
                const vec3 &v = top->x0[i + top->mg * (j + top->ng * k)];
                cs += v.x * 1.0 + v.y * 2.0 + v.z * 3.0;
            }
    std::printf("%d %.3e %.12e\n", cycles, rel, cs);
    if (dump) {
        FILE *f = std::fopen(dump, "wb");
        if (!f) return 3;
        for (const vec3 &v : s.rhs) std::fwrite(&v, sizeof(double), 3, f);
        for (size_t p = 0; p < s.rhs.size(); p++) std::fwrite(&top->x0[p], sizeof(double), 3, f);
        std::fclose(f);
    }
    return rel <= 1e-10 ? 0 : 1;
}

// The projection_step loop of shear_sim_3d.cpp:565-599 verbatim in its
// calls: v_cycle() and reg[0]->l2_error_all() (twice once the cycle count
// reaches std_iters/16) until the sum of |r|^4 drops below
// (1e3 eps stencil[13].a11)^2, then two more v_cycle()s; the solution is
// read through reg[0]->x0 afterwards.  Prints "cycles relres checksum".
template <class M>
int run_driver_loop(int N) {
    sim<M> s(N);
    stz_mg::multigrid_gpu<vec3, M> mgrid(s);
    mgrid.setup_matrices(s);
    mgrid.setup_fields(s);
    const double a11 = s.stencil[13].a11;
    double tol = std::numeric_limits<double>::epsilon() * a11 * 1e3;
    tol *= tol;
    const int std_iters = 16;
    int num_iters = 1, cycles = 0;
    double err = 1e16;
    while (err > tol && cycles < 100) {
        mgrid.v_cycle();
        cycles++;
        err = mgrid.reg[0]->l2_error_all();
        if (num_iters >= std_iters / 16) err = mgrid.reg[0]->l2_error_all();
        num_iters++;
    }
    mgrid.v_cycle();
    mgrid.v_cycle();
    cycles += 2;
    auto *top = mgrid.reg[0];
    double cs = 0;
    for (int k = 0; k <= N; k++)
        for (int j = 0; j < N; j++)
            for (int i = 0; i < N; i++) {
                const vec3 *v = top->x0 + i + top->mg * (j + top->ng * k);
                cs += v->x * 1.0 + v->y * 2.0 + v->z * 3.0;
            }
    double rn = 0, bn = 0;
    stz_mg::check(stz_mg_residual_norm(mgrid.handle(), &rn, &bn));
    std::printf("%d %.3e %.12e\n", cycles, rn / bn, cs);
    return err <= tol ? 0 : 1;
}

int main(int argc, char **argv) {
    int N = argc > 1 ? std::atoi(argv[1]) : 16;
    try {
        const char *dump = argc > 2 ? argv[2] : nullptr;
        return run<mat3>(N, dump) | run<sym_mat3>(N, nullptr) | run_driver_loop<mat3>(N);
    } catch (const stz_mg::error &e) {
        std::fprintf(stderr, "stz_mg error %d: %s\n", e.code, e.what());
        return 2;
    }
}
