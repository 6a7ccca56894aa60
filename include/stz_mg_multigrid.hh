// stz_mg_multigrid.hh -- header-only C++ adapter over the stz_mg C-ABI with
// the interface the reference's simulation drivers use.
//
// In nmboffi/stzpp, shear_sim_3d / trans_sim_3d hold a
//     multigrid<vec3, M> mgrid;          (src/shear_sim_3d.hh, M = sym_mat3 / mat3)
// built with  mgrid(*this, buf)          (src/shear_sim_3d.cpp:61)
// and call    mgrid.setup_matrices(*this) (src/shear_sim_3d.hh:54, trans_sim_3d.cpp:1488)
//             mgrid.setup_fields(*this)   (src/shear_sim_3d.cpp:550)
//             mgrid.v_cycle()             (src/shear_sim_3d.cpp:569, 599)
//             mgrid.reg[0]->l2_error_all() (src/shear_sim_3d.cpp:573, 578)
// and read    reg[0]->x0, mg, ng, mng     (src/shear_sim_3d.cpp:541-544, 616-674).
// multigrid_gpu<V, M> offers exactly these members, computing on the GPU.
// It reads the simulation through the same duck-typed contract as the
// reference's region constructor (region.hh:792-933): gN_x.., x_period..,
// interior(), internal(), mem_size(), external_ptr(), fill_entries(),
// x_field(), r_field().  One rank: the simulation's own grid must be the
// whole domain (the GPU path does not shard).
//
// V must have members x, y, z (vec3); M may be mat3 (a11..a33) or sym_mat3
// (a11, a12, a13, a22, a23, a33), told apart by size.
#ifndef STZ_MG_MULTIGRID_HH
#define STZ_MG_MULTIGRID_HH

#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "stz_mg.h"

namespace stz_mg {

struct error : std::runtime_error {
    int code;
    error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != STZ_MG_OK) throw error(rc, stz_mg_last_error());
}

// 3x3 block as 9 doubles, row-major
template <class M>
inline void block9(const M &a, double *o, std::true_type /* full mat3 */) {
    o[0] = a.a11; o[1] = a.a12; o[2] = a.a13;
    o[3] = a.a21; o[4] = a.a22; o[5] = a.a23;
    o[6] = a.a31; o[7] = a.a32; o[8] = a.a33;
}
template <class M>
inline void block9(const M &a, double *o, std::false_type /* sym_mat3 */) {
    o[0] = a.a11; o[1] = a.a12; o[2] = a.a13;
    o[3] = a.a12; o[4] = a.a22; o[5] = a.a23;
    o[6] = a.a13; o[7] = a.a23; o[8] = a.a33;
}
template <class M>
inline void block9(const M &a, double *o) {
    block9(a, o, std::integral_constant<bool, sizeof(M) == 9 * sizeof(double)>());
}

// Host mirror of the top region's solution, laid out like region::x0 with
// mg = m, ng = n (no ghost layers).  The mirror is filled lazily: a V-cycle
// only marks it stale, and the first read of x0 afterwards copies the
// solution from the device once.  So the drivers' loop of v_cycle() and
// l2_error_all() (shear_sim_3d.cpp:567-599) moves one scalar per call, not
// the whole field, and the solution crosses to the host once, when the
// driver reads it (shear_sim_3d.cpp:616-674).
template <class V>
struct top_region {
    // x0 behaves like region::x0 (a V*): x0 + offset, x0[offset], *x0, and
    // conversion to V*; each access refreshes a stale mirror first.
    struct lazy_x0 {
        top_region *r = nullptr;
        V *get() const { return r->fresh(); }
        operator V *() const { return get(); }
        V *operator+(std::ptrdiff_t o) const { return get() + o; }
        V &operator[](std::ptrdiff_t o) const { return get()[o]; }
        V &operator*() const { return *get(); }
    };
    lazy_x0 x0;
    int mg = 0, ng = 0, mng = 0;
    stz_mg_handle h = nullptr;
    // region::l2_error_all as shipped (sum of |r|^4, region.cc:3030-3057),
    // reduced on the device
    double l2_error_all() const {
        double v = 0;
        check(stz_mg_l2_error_all(h, &v));
        return v;
    }
    // marks the mirror stale (the device solution changed)
    void invalidate() { stale_ = true; }
    V *fresh() {
        if (stale_) {
            std::vector<double> x(3 * host_.size());
            check(stz_mg_get_x(h, x.data(), STZ_MG_HOST));
            for (size_t p = 0; p < host_.size(); p++) {
                host_[p].x = x[3 * p];
                host_[p].y = x[3 * p + 1];
                host_[p].z = x[3 * p + 2];
            }
            stale_ = false;
        }
        return host_.data();
    }
    void resize(size_t n) {
        host_.assign(n, V());
        stale_ = true;
    }

   private:
    std::vector<V> host_;
    bool stale_ = true;
};

template <class V, class M>
class multigrid_gpu {
   public:
    int nlevels = 0;
    top_region<V> *reg[1];

    // `desc` may preset solver options (precision, v_down, v_up, hierarchy,
    // bottom solve, device); the grid fields are taken from the simulation.
    template <class sim_class>
    explicit multigrid_gpu(sim_class &sim, const stz_mg_desc *desc = nullptr) {
        px_ = sim.x_period; py_ = sim.y_period; pz_ = sim.z_period;
        m_ = sim.gN_x + (sim.x_period ? 0 : 1);   // region.hh:805
        n_ = sim.gN_y + (sim.y_period ? 0 : 1);
        o_ = sim.gN_z + (sim.z_period ? 0 : 1);
        stz_mg_desc d;
        if (desc) d = *desc;
        else stz_mg_desc_default(&d);
        d.m = m_; d.n = n_; d.o = o_;
        d.x_prd = sim.x_period; d.y_prd = sim.y_period; d.z_prd = sim.z_period;
        check(stz_mg_create(&d, &h_));
        check(stz_mg_num_levels(h_, &nlevels));
        top_.h = h_;
        top_.mg = m_;
        top_.ng = n_;
        top_.mng = m_ * n_;
        top_.resize(npts());
        top_.x0.r = &top_;
        reg[0] = &top_;
    }
    ~multigrid_gpu() { stz_mg_destroy(h_); }
    multigrid_gpu(const multigrid_gpu &) = delete;
    multigrid_gpu &operator=(const multigrid_gpu &) = delete;

    // multigrid::setup_matrices: the operator from the simulation, then RAT.
    // A simulation whose interior nodes all point at one shared stencil and
    // whose boundary nodes all point at one fix block (shear_sim_3d.hh:401-402)
    // is uploaded once as a constant stencil; anything else node by node.
    template <class sim_class>
    void setup_matrices(sim_class &sim) {
        const M *st = nullptr, *fx = nullptr;
        bool shared = true;
        for (int k = 0; k < o_; k++)
            for (int j = 0; j < n_; j++)
                for (int i = 0; i < m_; i++) {
                    const bool full = box(sim, i, j, k) == 27;
                    if (!shared) continue;
                    if (sim.internal(i, j, k)) { shared = false; continue; }
                    const M *p = sim.external_ptr(i, j, k);
                    const M *&slot = full ? st : fx;
                    if (!slot) slot = p;
                    else if (slot != p) shared = false;
                }
        if (shared && st) {
            double s[243], f[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            for (int b = 0; b < 27; b++) block9(st[b], s + 9 * b);
            if (fx) block9(*fx, f);
            check(stz_mg_set_stencil_const(h_, s, f));
        } else {
            std::vector<double> A(243 * npts(), 0.0);
            std::vector<M> tmp(27);
            for (int k = 0; k < o_; k++)
                for (int j = 0; j < n_; j++)
                    for (int i = 0; i < m_; i++) {
                        double *dst = &A[243 * idx(i, j, k)];
                        const bool full = box(sim, i, j, k) == 27;
                        const M *src;
                        if (sim.internal(i, j, k)) {
                            M *en = tmp.data();
                            sim.fill_entries(i, j, k, en);
                            src = tmp.data();
                        } else {
                            src = sim.external_ptr(i, j, k);
                        }
                        for (int b = 0; b < (full ? 27 : 1); b++) block9(src[b], dst + 9 * (full ? b : 13));
                    }
            check(stz_mg_set_stencil_points(h_, A.data(), STZ_MG_HOST));
        }
        check(stz_mg_setup(h_));
    }

    // multigrid::setup_fields: x_field / r_field of every node (global indices, origin 0).
    template <class sim_class>
    void setup_fields(sim_class &sim) {
        std::vector<double> x(3 * npts()), r(3 * npts());
        for (int k = 0; k < o_; k++)
            for (int j = 0; j < n_; j++)
                for (int i = 0; i < m_; i++) {
                    const size_t p = idx(i, j, k);
                    V xv = sim.x_field(i, j, k, 0, 0, 0);
                    V rv = sim.r_field(i, j, k, 0, 0, 0);
                    x[3 * p] = xv.x; x[3 * p + 1] = xv.y; x[3 * p + 2] = xv.z;
                    r[3 * p] = rv.x; r[3 * p + 1] = rv.y; r[3 * p + 2] = rv.z;
                }
        check(stz_mg_set_x(h_, x.data(), STZ_MG_HOST));
        check(stz_mg_set_rhs(h_, r.data(), STZ_MG_HOST));
        top_.invalidate();
    }

    // multigrid::v_cycle; the host mirror reg[0]->x0 refreshes on its next read.
    void v_cycle() {
        check(stz_mg_vcycle(h_));
        top_.invalidate();
    }

    // V-cycles to |b - A x| <= tol |b| (the projection_step loop with the true residual).
    int solve(double tol, int max_cycles, double *relres = nullptr) {
        int c = 0;
        double rr = 0;
        check(stz_mg_solve(h_, tol, max_cycles, &c, &rr));
        if (relres) *relres = rr;
        top_.invalidate();
        return c;
    }

    // Copies the solution to the host mirror now (it otherwise happens on the
    // first read of reg[0]->x0).
    void sync_x() { top_.fresh(); }

    stz_mg_handle handle() const { return h_; }

   private:
    // Box of node (i,j,k) from the problem's range_* (region.hh:716-735): the
    // GPU path takes full 3x3x3 boxes on interior nodes and single-node boxes
    // on the Dirichlet faces, as shear_sim_3d.hh:262-273 defines them.
    template <class sim_class>
    int box(sim_class &sim, int i, int j, int k) const {
        const int xd = sim.range_xd(i, j, k), xu = sim.range_xu(i, j, k), yd = sim.range_yd(i, j, k),
                  yu = sim.range_yu(i, j, k), zd = sim.range_zd(i, j, k), zu = sim.range_zu(i, j, k);
        const bool full = xd == -1 && xu == 2 && yd == -1 && yu == 2 && zd == -1 && zu == 2;
        const bool single = xd == 0 && xu == 1 && yd == 0 && yu == 1 && zd == 0 && zu == 1;
        const bool interior = (px_ || (i != 0 && i != m_ - 1)) && (py_ || (j != 0 && j != n_ - 1)) &&
                              (pz_ || (k != 0 && k != o_ - 1));
        if (!(full && interior) && !(single && !interior))
            throw error(STZ_MG_ERR_UNSUPPORTED, "stencil box is not 3x3x3 on interior nodes and 1x1x1 on Dirichlet nodes");
        return full ? 27 : 1;
    }
    size_t npts() const { return (size_t)m_ * n_ * o_; }
    size_t idx(int i, int j, int k) const { return i + (size_t)m_ * (j + (size_t)n_ * k); }
    int m_ = 0, n_ = 0, o_ = 0;
    bool px_ = false, py_ = false, pz_ = false;
    stz_mg_handle h_ = nullptr;
    top_region<V> top_;
};

}  // namespace stz_mg

#endif
