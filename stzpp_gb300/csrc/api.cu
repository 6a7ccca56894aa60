// Host runtime and C-ABI of the GB300 multigrid (include/stz_mg.h).
//
// One handle = one problem on one GPU: the level hierarchy
// (multigrid::setup_hierarchy, mg_3d_template/multigrid.cc:19-132), the FP64
// operators of every level (top level as given, coarse levels by RAT), the
// FP32 copy of the hierarchy used by the mixed-precision solver, the FP64
// dense inverse of the coarsest level, and the V-cycle (multigrid.cc:253-297)
// captured once into a CUDA graph per precision and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include "../../include/stz_mg.h"
#include "launch.h"
#include "ops.cuh"

using namespace stzmg;

namespace {

thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

struct CudaError {
    int code;
};

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(e_ == cudaErrorMemoryAllocation ? STZ_MG_ERR_OOM : STZ_MG_ERR_CUDA,        \
                      "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);      \
            throw CudaError{e_ == cudaErrorMemoryAllocation ? STZ_MG_ERR_OOM : STZ_MG_ERR_CUDA}; \
        }                                                                                        \
    } while (0)

struct ApiError {
    int code;
};

[[noreturn]] void fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    throw ApiError{code};
}

template <typename T>
struct Level {
    T *x = nullptr, *r = nullptr, *res = nullptr;   // 3*npad each
    T *coef = nullptr, *dinv = nullptr;             // coarse operators (243 and 9 per row)
    size_t coef_rows = 0;                           // rows coef / dinv were allocated for
};

constexpr int kMaxLev = kMaxLevels;

}  // namespace

struct stz_mg_handle_s {
    stz_mg_desc d;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    int nlev = 0;
    Geom geo[kMaxLev];
    Level<double> L64[kMaxLev];
    Level<float> L32[kMaxLev];
    LevelOp<double> op64[kMaxLev];
    LevelOp<float> op32[kMaxLev];
    int *S[kMaxLev] = {};
    int top_kind = -1;          // OpKind of the top level once set
    double *mu64 = nullptr, *lam64 = nullptr;
    float *mu32 = nullptr, *lam32 = nullptr;
    double *top_coef64 = nullptr, *top_dinv64 = nullptr;  // per-point top level
    float *top_coef32 = nullptr, *top_dinv32 = nullptr;
    // bottom
    double *ainv_t = nullptr;
    int *nat_slot = nullptr;
    int nbot_rows = 0;
    // set-up scratch kept between set-ups (a coefficient change re-runs set-up)
    double *bot_aug = nullptr, *bot_col = nullptr, *bot_dense = nullptr;
    int *bot_piv = nullptr, *bot_S = nullptr;
    bool bottom_fourier = false;   // the bottom inverse came from the Fourier blocks
    size_t bot_aug_len = 0, bot_dense_len = 0, bot_S_len = 0;
    // scratch
    double *partial = nullptr;
    int partial_len = 0;
    double *dscal = nullptr;    // device scalars
    double *hscal = nullptr;    // pinned host scalars
    int *dflag = nullptr;
    double *stage = nullptr;    // device staging for host<->device natural-order copies
    size_t stage_len = 0;
    double *adj_g = nullptr, *adj_t = nullptr;   // adjoint: natural-order g and work vector
    double *grad_c = nullptr;                    // coefficient gradient: 14 doubles per node
    double bnorm = -1.0;
    bool setup_done = false;
    cudaGraphExec_t gx64 = nullptr, gx32 = nullptr;
    long long graph_kernels64 = 0, graph_kernels32 = 0;   // kernel nodes per captured V-cycle
    // persistent cluster tail: levels tail_lo..nlev-2 (tail_lo < 0: none)
    int tail_lo = -1, tail_cluster = 0, tail_cap_planes = 0;
    int stat_cycles = 0, stat_residuals = 0;
    long long stat_launches = 0;
    // C-ABI calls on this handle so far; l2_error_all records the call that
    // computed its value, and the residual it left in the FP32 top-level
    // right-hand side (mixed precision) stays valid only while no other
    // call has run since
    long long api_calls = 0, l2_call = -1;
    double l2_value = 0.0;
    std::vector<void *> allocs;

    template <typename T>
    T *alloc(size_t n) {
        void *p = nullptr;
        const size_t bytes = n * sizeof(T);
        CK(cudaMalloc(&p, bytes ? bytes : 1));
        allocs.push_back(p);
        return (T *)p;
    }
    // p holds at least n elements afterwards (reallocated only to grow)
    template <typename T>
    void ensure(T *&p, size_t &cap, size_t n) {
        if (p && cap >= n) return;
        release(p);
        p = alloc<T>(n);
        cap = n;
    }
    void release(void *p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) {
            cudaFree(p);
            allocs.erase(it);
        }
    }
};

namespace {

template <typename F>
int guarded(stz_mg_handle h, F &&f) {
    try {
        if (h) {
            h->api_calls++;
            CK(cudaSetDevice(h->d.device));
        }
        f();
        return STZ_MG_OK;
    } catch (const ApiError &e) {
        return e.code;
    } catch (const CudaError &e) {
        return e.code;
    } catch (const std::bad_alloc &) {
        return set_error(STZ_MG_ERR_OOM, "host allocation failed");
    }
}

size_t npts(const Geom &g) { return (size_t)g.m * g.n * g.o; }

void check_launch() { CK(cudaGetLastError()); }

void sync(stz_mg_handle h) {
    CK(cudaStreamSynchronize(h->st));
    check_launch();
}

// The band sweep's CTAs give up (and record it) when their staged copies do
// not arrive in time; a solve or sweep that saw that fails.
void check_band(stz_mg_handle h) {
    const int e = band_take_error(h->st);
    if (e < 0) fail(STZ_MG_ERR_CUDA, "cannot read the band sweep's record");
    if (e == 2) fail(STZ_MG_ERR_CUDA, "band sweep: shared memory not 128-byte aligned");
    if (e > 0) fail(STZ_MG_ERR_CUDA, "band sweep: staged copies did not arrive within 0.2 s");
}

double *staging(stz_mg_handle h, size_t n) {
    if (h->stage_len < n) {
        h->release(h->stage);
        h->stage = h->alloc<double>(n);
        h->stage_len = n;
    }
    return h->stage;
}

// Copies a natural-order host or device array of n doubles to device memory.
const double *to_device(stz_mg_handle h, const double *src, size_t n, int where) {
    if (!src) fail(STZ_MG_ERR_ARG, "null input pointer");
    if (where == STZ_MG_DEVICE) return src;
    if (where != STZ_MG_HOST) fail(STZ_MG_ERR_ARG, "where must be STZ_MG_HOST or STZ_MG_DEVICE");
    double *d = staging(h, n);
    CK(cudaMemcpyAsync(d, src, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
    return d;
}

void need_setup(stz_mg_handle h) {
    if (!h->setup_done) fail(STZ_MG_ERR_ARG, "stz_mg_setup has not been called");
}

void check_level(stz_mg_handle h, int l) {
    if (l < 0 || l >= h->nlev) fail(STZ_MG_ERR_ARG, "level %d out of range [0,%d)", l, h->nlev);
}

// ------------------------------------------------------------ hierarchy
// The 8-colour smoother needs every periodic dimension even (or 1): an odd
// periodic dimension would couple two nodes of the same colour.
bool odd_periodic(int m, int n, int o, int xp, int yp, int zp) {
    return (xp && m > 1 && (m & 1)) || (yp && n > 1 && (n & 1)) || (zp && o > 1 && (o & 1));
}

// multigrid::multigrid's hierarchy (multigrid.cc:40): coarsen until a level
// has at most max_coarse nodes.  Where the next level would have an odd
// periodic dimension (a periodic size whose halving chain reaches an odd
// size above max_coarse, e.g. 72 -> 36 -> 18 -> 9), the hierarchy stops at
// the last even level instead, which then is the bottom level.
void build_geometry(stz_mg_handle h) {
    const stz_mg_desc &d = h->d;
    h->geo[0] = make_geom(d.m, d.n, d.o, d.x_prd, d.y_prd, d.z_prd);
    h->nlev = 1;
    while (npts(h->geo[h->nlev - 1]) > (size_t)d.max_coarse) {
        const Geom &P = h->geo[h->nlev - 1];
        int mc = (P.m + (P.xp ? 1 : 2)) >> 1, nc = (P.n + (P.yp ? 1 : 2)) >> 1, oc = (P.o + (P.zp ? 1 : 2)) >> 1;
        if (mc == P.m && nc == P.n && oc == P.o) break;
        if (odd_periodic(mc, nc, oc, P.xp, P.yp, P.zp)) break;
        if (h->nlev == kMaxLev) fail(STZ_MG_ERR_UNSUPPORTED, "more than %d levels", kMaxLev);
        h->geo[h->nlev++] = make_geom(mc, nc, oc, P.xp, P.yp, P.zp);
    }
    for (int l = 0; l < h->nlev; l++) {
        const Geom &g = h->geo[l];
        if (odd_periodic(g.m, g.n, g.o, g.xp, g.yp, g.zp))
            fail(STZ_MG_ERR_UNSUPPORTED,
                 "level %d has an odd periodic dimension (%dx%dx%d); the 8-colour smoother needs even periodic sizes",
                 l, g.m, g.n, g.o);
        if ((size_t)g.npad * 243 > (size_t)1 << 40) fail(STZ_MG_ERR_UNSUPPORTED, "grid too large");
    }
}

void alloc_fields(stz_mg_handle h) {
    for (int l = 0; l < h->nlev; l++) {
        const size_t n3 = 3 * (size_t)h->geo[l].npad;
        Level<double> &A = h->L64[l];
        A.x = h->alloc<double>(n3);
        A.r = h->alloc<double>(n3);
        A.res = h->alloc<double>(n3);
        CK(cudaMemsetAsync(A.x, 0, n3 * sizeof(double), h->st));
        CK(cudaMemsetAsync(A.r, 0, n3 * sizeof(double), h->st));
        CK(cudaMemsetAsync(A.res, 0, n3 * sizeof(double), h->st));
        h->S[l] = h->alloc<int>(6 * (size_t)h->geo[l].npad);
        if (h->d.precision == STZ_MG_MIXED) {
            Level<float> &B = h->L32[l];
            B.x = h->alloc<float>(n3);
            B.r = h->alloc<float>(n3);
            B.res = h->alloc<float>(n3);
            CK(cudaMemsetAsync(B.x, 0, n3 * sizeof(float), h->st));
            CK(cudaMemsetAsync(B.r, 0, n3 * sizeof(float), h->st));
            CK(cudaMemsetAsync(B.res, 0, n3 * sizeof(float), h->st));
        }
    }
    h->partial_len = residual_blocks(h->geo[0]);
    h->partial = h->alloc<double>(h->partial_len);
    h->dscal = h->alloc<double>(8);
    h->dflag = h->alloc<int>(4);
    CK(cudaMallocHost(&h->hscal, 8 * sizeof(double)));
}

void release_graphs(stz_mg_handle h) {
    if (h->gx64) cudaGraphExecDestroy(h->gx64);
    if (h->gx32) cudaGraphExecDestroy(h->gx32);
    h->gx64 = h->gx32 = nullptr;
}

void invalidate(stz_mg_handle h) {
    h->setup_done = false;
    release_graphs(h);
}

// ------------------------------------------------------------ operators
void set_const_op(stz_mg_handle h, const double *stencil, const double *fix) {
    ConstOp<double> c{};
    std::memcpy(c.a, stencil, sizeof(c.a));
    std::memcpy(c.fix, fix, sizeof(c.fix));
    bool ok = inverse3(c.a[13], c.inv_int) & inverse3(c.fix, c.inv_fix);
    if (!ok) fail(STZ_MG_ERR_SINGULAR, "singular centre or fix block");
    for (int v = 0; v < 243; v++)
        if (!std::isfinite(stencil[v])) fail(STZ_MG_ERR_NONFINITE, "non-finite stencil entry %d", v);
    int elastic = 1;
    for (int b = 0; b < 27; b++)
        for (int e = 0; e < 9; e++)
            if (!elastic_entry(b, e) && c.a[b][e] != 0.0) elastic = 0;
    c.elastic = elastic;
    c.centre_diag = c.a[13][1] == 0.0 && c.a[13][2] == 0.0 && c.a[13][3] == 0.0 && c.a[13][5] == 0.0 &&
                    c.a[13][6] == 0.0 && c.a[13][7] == 0.0;
    ConstOp<float> f{};
    for (int b = 0; b < 27; b++)
        for (int e = 0; e < 9; e++) f.a[b][e] = (float)c.a[b][e];
    for (int e = 0; e < 9; e++) {
        f.fix[e] = (float)c.fix[e];
        f.inv_int[e] = (float)c.inv_int[e];
        f.inv_fix[e] = (float)c.inv_fix[e];
    }
    f.elastic = elastic;
    f.centre_diag = c.centre_diag;
    h->op64[0] = LevelOp<double>{};
    h->op64[0].kind = OP_CONST;
    h->op64[0].cop = c;
    h->op32[0] = LevelOp<float>{};
    h->op32[0].kind = OP_CONST;
    h->op32[0].cop = f;
    h->top_kind = OP_CONST;
}

}  // namespace

namespace stzmg {
__global__ void finite_check_kernel(const double *__restrict__ v, size_t n, int *bad) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; t < n; t += (size_t)gridDim.x * blockDim.x)
        if (!(v[t] - v[t] == 0.0)) { atomicExch(bad, 1); return; }
}

// flag[0] = 1 if any of v[0..n) is not zero
__global__ void nonzero_kernel(const double *__restrict__ v, size_t n, int *flag) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; t < n; t += (size_t)gridDim.x * blockDim.x)
        if (v[t] != 0.0) { atomicExch(flag, 1); return; }
}

// Sum of squares of v[0..n): one partial per block (fixed grid, fixed order),
// then one block sums the partials -- deterministic.
__global__ void sumsq_partial_kernel(const double *__restrict__ v, size_t n, double *__restrict__ partial) {
    __shared__ double red[8];
    double s = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        s += v[t] * v[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

// z-planes k0 .. k0+nk-1 of a colour-blocked FP64 vec3 field <-> natural
// order (x fastest, 3 doubles per node, the planes' nodes only).
__global__ void planes_cb_to_nat_kernel(Geom g, int k0, int nk, const double *__restrict__ cb,
                                        double *__restrict__ nat) {
    const long long n = (long long)g.m * g.n * nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.m), j = (int)((t / g.m) % g.n), k = k0 + (int)(t / ((long long)g.m * g.n));
        const int s = slot(g, i, j, k);
        nat[3 * t] = cb[s];
        nat[3 * t + 1] = cb[s + g.npad];
        nat[3 * t + 2] = cb[s + 2 * (size_t)g.npad];
    }
}

__global__ void planes_nat_to_cb_kernel(Geom g, int k0, int nk, const double *__restrict__ nat,
                                        double *__restrict__ cb) {
    const long long n = (long long)g.m * g.n * nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.m), j = (int)((t / g.m) % g.n), k = k0 + (int)(t / ((long long)g.m * g.n));
        const int s = slot(g, i, j, k);
        cb[s] = nat[3 * t];
        cb[s + g.npad] = nat[3 * t + 1];
        cb[s + 2 * (size_t)g.npad] = nat[3 * t + 2];
    }
}

// region::l2_error_all for vec3 (region.cc:3030-3057): sum over nodes of
// mg3d_mod_sq(|r|^2) = |r|^4, from the colour-blocked FP64 residual (3 planes
// of npad; the slots of no node hold zero).  One partial per block, fixed
// grid and order: deterministic.
template <typename R>
__global__ void quartic_partial_kernel(const R *__restrict__ res, int npad, double *__restrict__ partial) {
    __shared__ double red[8];
    double s = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npad; t += gridDim.x * blockDim.x) {
        const double a = res[t], b = res[t + npad], c = res[t + 2 * (size_t)npad];
        const double q = a * a + b * b + c * c;
        s += q * q;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

__global__ void sum_blocks_kernel(const double *__restrict__ partial, int nb, double *__restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) s += partial[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = red[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) out[0] = s;
    }
}
}  // namespace stzmg

namespace {

void require_finite(stz_mg_handle h, const double *d, size_t n, const char *what) {
    CK(cudaMemsetAsync(h->dflag, 0, sizeof(int), h->st));
    size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 16);
    finite_check_kernel<<<(unsigned)std::max<size_t>(blocks, 1), 256, 0, h->st>>>(d, n, h->dflag);
    check_launch();
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    sync(h);
    if (bad) fail(STZ_MG_ERR_NONFINITE, "%s contains NaN or Inf", what);
}

// ------------------------------------------------------------ setup
// Inverse of a bottom operator M (nr x nr, natural node order, 3 rows per
// node) that commutes with the translations of a grid periodic in x and y:
// M couples column (i, j) to column (i + dx, j + dy) through a block A(d) of
// (3o x 3o) that does not depend on (i, j), so the discrete Fourier transform
// in x and y splits M into m n independent complex systems
//   D(t) = sum_d A(d) e^{i t.d},  t = 2 pi (kx / m, ky / n),
// and M^-1 couples (i, j) to (i + dx, j + dy) through
//   B(d) = 1/(m n) sum_t D(t)^-1 e^{-i t.d}.
// m n inversions of order 3o instead of one of order 3 m n o.  False when M
// is not exactly invariant (then the general inverse runs); fails if some
// D(t) is singular.
bool fourier_bottom_inverse(const Geom &g, const std::vector<double> &M, int nr, std::vector<double> &inv) {
    using cd = std::complex<double>;
    const int m = g.m, n = g.n, o = g.o, bs = 3 * o, cols = m * n;
    if (!g.xp || !g.yp || nr != 3 * cols * o) return false;
    auto row = [&](int i, int j, int k, int a) { return (size_t)3 * (i + (size_t)m * (j + (size_t)n * k)) + a; };
    // A(d)[(k,a),(k',c)] from the rows of column (0, 0); every other row must match
    std::vector<double> A((size_t)cols * bs * bs);
    for (int dj = 0; dj < n; dj++)
        for (int di = 0; di < m; di++)
            for (int k = 0; k < o; k++)
                for (int a = 0; a < 3; a++)
                    for (int k2 = 0; k2 < o; k2++)
                        for (int c = 0; c < 3; c++)
                            A[((size_t)(di + m * dj) * bs + 3 * k + a) * bs + 3 * k2 + c] =
                                M[row(0, 0, k, a) * nr + row(di, dj, k2, c)];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++)
            for (int k = 0; k < o; k++)
                for (int a = 0; a < 3; a++) {
                    const double *r = &M[row(i, j, k, a) * nr];
                    for (int dj = 0; dj < n; dj++)
                        for (int di = 0; di < m; di++)
                            for (int k2 = 0; k2 < o; k2++)
                                for (int c = 0; c < 3; c++)
                                    if (r[row((i + di) % m, (j + dj) % n, k2, c)] !=
                                        A[((size_t)(di + m * dj) * bs + 3 * k + a) * bs + 3 * k2 + c])
                                        return false;
                }
    std::vector<cd> ex(m), ey(n);   // e^{2 pi i q / m}, e^{2 pi i q / n}
    const double tau = 6.283185307179586476925286766559;
    for (int q = 0; q < m; q++) ex[q] = std::polar(1.0, tau * q / m);
    for (int q = 0; q < n; q++) ey[q] = std::polar(1.0, tau * q / n);
    std::vector<cd> G((size_t)cols * bs * bs), D((size_t)bs * 2 * bs);
    for (int ky = 0; ky < n; ky++)
        for (int kx = 0; kx < m; kx++) {
            // [D(t) | I], then Gauss-Jordan with partial pivoting
            std::fill(D.begin(), D.end(), cd(0.0));
            for (int dj = 0; dj < n; dj++)
                for (int di = 0; di < m; di++) {
                    const double *Ad = &A[(size_t)(di + m * dj) * bs * bs];
                    bool any = false;
                    for (int e = 0; e < bs * bs && !any; e++) any = Ad[e] != 0.0;
                    if (!any) continue;
                    const cd w = ex[(kx * di) % m] * ey[(ky * dj) % n];
                    for (int r = 0; r < bs; r++)
                        for (int c = 0; c < bs; c++) D[(size_t)r * 2 * bs + c] += Ad[r * bs + c] * w;
                }
            for (int r = 0; r < bs; r++) D[(size_t)r * 2 * bs + bs + r] = 1.0;
            for (int col = 0; col < bs; col++) {
                int piv = col;
                for (int r = col + 1; r < bs; r++)
                    if (std::abs(D[(size_t)r * 2 * bs + col]) > std::abs(D[(size_t)piv * 2 * bs + col])) piv = r;
                const double pv = std::abs(D[(size_t)piv * 2 * bs + col]);
                if (!(pv > 0.0) || !std::isfinite(pv)) fail(STZ_MG_ERR_SINGULAR, "bottom-level matrix is singular");
                if (piv != col)
                    for (int c = 0; c < 2 * bs; c++) std::swap(D[(size_t)piv * 2 * bs + c], D[(size_t)col * 2 * bs + c]);
                const cd ip = 1.0 / D[(size_t)col * 2 * bs + col];
                for (int c = 0; c < 2 * bs; c++) D[(size_t)col * 2 * bs + c] *= ip;
                for (int r = 0; r < bs; r++) {
                    if (r == col) continue;
                    const cd f = D[(size_t)r * 2 * bs + col];
                    if (f == cd(0.0)) continue;
                    for (int c = 0; c < 2 * bs; c++) D[(size_t)r * 2 * bs + c] -= f * D[(size_t)col * 2 * bs + c];
                }
            }
            cd *Gt = &G[(size_t)(kx + m * ky) * bs * bs];
            for (int r = 0; r < bs; r++)
                for (int c = 0; c < bs; c++) Gt[r * bs + c] = D[(size_t)r * 2 * bs + bs + c];
        }
    // B(d), then every block of the inverse
    std::vector<double> B((size_t)cols * bs * bs);
    std::vector<cd> acc((size_t)bs * bs);
    for (int dj = 0; dj < n; dj++)
        for (int di = 0; di < m; di++) {
            std::fill(acc.begin(), acc.end(), cd(0.0));
            for (int ky = 0; ky < n; ky++)
                for (int kx = 0; kx < m; kx++) {
                    const cd w = std::conj(ex[(kx * di) % m] * ey[(ky * dj) % n]);
                    const cd *Gt = &G[(size_t)(kx + m * ky) * bs * bs];
                    for (int e = 0; e < bs * bs; e++) acc[e] += Gt[e] * w;
                }
            double *Bd = &B[(size_t)(di + m * dj) * bs * bs];
            for (int e = 0; e < bs * bs; e++) Bd[e] = acc[e].real() / cols;
        }
    inv.assign((size_t)nr * nr, 0.0);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++)
            for (int k = 0; k < o; k++)
                for (int a = 0; a < 3; a++) {
                    double *r = &inv[row(i, j, k, a) * nr];
                    for (int dj = 0; dj < n; dj++)
                        for (int di = 0; di < m; di++) {
                            const double *Bd = &B[((size_t)(di + m * dj) * bs + 3 * k + a) * bs];
                            for (int k2 = 0; k2 < o; k2++)
                                for (int c = 0; c < 3; c++) r[row((i + di) % m, (j + dj) % n, k2, c)] = Bd[3 * k2 + c];
                        }
                }
    return true;
}

void build_bottom(stz_mg_handle h) {
    const int lb = h->nlev - 1;
    const Geom &g = h->geo[lb];
    const size_t N = npts(g);
    if (N > 4096) fail(STZ_MG_ERR_UNSUPPORTED, "direct bottom solve limited to 4096 nodes (have %zu)", N);
    const int nr = (int)(3 * N);
    // dense operator of the bottom level, natural order
    std::vector<double> Anat(243 * N);
    {
        const double *src = nullptr;
        if (h->op64[lb].kind != OP_DENSE) {
            h->ensure(h->bot_dense, h->bot_dense_len, 243 * (size_t)g.npad);
            launch_expand_dense(h->op64[lb], g, h->bot_dense, h->st);
            src = h->bot_dense;
        } else {
            src = h->op64[lb].dop.coef;
        }
        double *nat = staging(h, 243 * N);
        launch_coef_cb_to_nat(g, src, nat, h->st);
        check_launch();
        CK(cudaMemcpyAsync(Anat.data(), nat, 243 * N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    }
    std::vector<int> Snat(6 * N);
    {
        h->ensure(h->bot_S, h->bot_S_len, 6 * N);
        launch_bounds_cb_to_nat(g, h->S[lb], h->bot_S, h->st);
        check_launch();
        CK(cudaMemcpyAsync(Snat.data(), h->bot_S, 6 * N * sizeof(int), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    }
    std::vector<double> M((size_t)nr * nr, 0.0);
    auto wrap = [](int a, int len) { a %= len; return a < 0 ? a + len : a; };
    for (int k = 0; k < g.o; k++)
        for (int j = 0; j < g.n; j++)
            for (int i = 0; i < g.m; i++) {
                size_t p = i + (size_t)g.m * (j + (size_t)g.n * k);
                const int *S = &Snat[6 * p];
                for (int dk = S[4]; dk < S[5]; dk++)
                    for (int dj = S[2]; dj < S[3]; dj++)
                        for (int di = S[0]; di < S[1]; di++) {
                            if (di < -1 || di > 1 || dj < -1 || dj > 1 || dk < -1 || dk > 1)
                                fail(STZ_MG_ERR_UNSUPPORTED, "bottom stencil reaches beyond one node");
                            int ii = i + di, jj = j + dj, kk = k + dk;
                            if (g.xp) ii = wrap(ii, g.m);
                            if (g.yp) jj = wrap(jj, g.n);
                            if (g.zp) kk = wrap(kk, g.o);
                            if (ii < 0 || ii >= g.m || jj < 0 || jj >= g.n || kk < 0 || kk >= g.o) continue;
                            size_t q = ii + (size_t)g.m * (jj + (size_t)g.n * kk);
                            const double *blk = &Anat[243 * p + 9 * ((di + 1) + 3 * (dj + 1) + 9 * (dk + 1))];
                            for (int a = 0; a < 3; a++)
                                for (int c = 0; c < 3; c++) M[(3 * p + a) * nr + 3 * q + c] += blk[3 * a + c];
                        }
            }
    // buffers are sized by the bottom level, which does not change between set-ups
    if (!h->ainv_t || h->nbot_rows != nr) {
        h->release(h->bot_aug);
        h->release(h->bot_col);
        h->release(h->bot_piv);
        h->release(h->ainv_t);
        h->release(h->nat_slot);
        h->bot_aug = nullptr;
        h->ainv_t = h->alloc<double>((size_t)nr * nr);
        h->nat_slot = h->alloc<int>(N);
        std::vector<int> ns(N);
        for (int k = 0; k < g.o; k++)
            for (int j = 0; j < g.n; j++)
                for (int i = 0; i < g.m; i++) ns[i + (size_t)g.m * (j + (size_t)g.n * k)] = slot(g, i, j, k);
        CK(cudaMemcpyAsync(h->nat_slot, ns.data(), N * sizeof(int), cudaMemcpyHostToDevice, h->st));
        sync(h);
        h->nbot_rows = nr;
    }
    // a plane-invariant bottom periodic in x and y: Fourier blocks on the host
    // (STZ_MG_BOTTOM_FOURIER=0 turns that off)
    const char *fe = std::getenv("STZ_MG_BOTTOM_FOURIER");
    const bool fourier_ok = !(fe && std::atoi(fe) == 0) && h->op64[lb].kind == OP_PLANE;
    {
        std::vector<double> inv;
        if (fourier_ok && fourier_bottom_inverse(g, M, nr, inv)) {
            CK(cudaMemcpyAsync(h->ainv_t, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
            sync(h);
            h->bottom_fourier = true;
            return;
        }
    }
    h->bottom_fourier = false;
    // Gauss-Jordan inverse with partial pivoting, FP64, on the device.
    std::vector<double> aug((size_t)nr * 2 * nr, 0.0);
    for (int r = 0; r < nr; r++) {
        std::memcpy(&aug[(size_t)r * 2 * nr], &M[(size_t)r * nr], nr * sizeof(double));
        aug[(size_t)r * 2 * nr + nr + r] = 1.0;
    }
    if (!h->bot_aug) {
        h->bot_aug = h->alloc<double>(aug.size());
        h->bot_col = h->alloc<double>(nr);
        h->bot_piv = h->alloc<int>(1);
    }
    CK(cudaMemcpyAsync(h->bot_aug, aug.data(), aug.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(h->dflag, 0, sizeof(int), h->st));
    launch_gauss_jordan(h->bot_aug, nr, h->ainv_t, h->bot_piv, h->bot_col, h->dflag, h->st);
    check_launch();
    int singular = 0;
    CK(cudaMemcpyAsync(&singular, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    sync(h);
    if (singular) fail(STZ_MG_ERR_SINGULAR, "bottom-level matrix is singular");
}

// Levels small enough for the persistent cluster kernels: the first coarse
// level with at most kTailMaxNodes nodes down to the level above the bottom.
constexpr size_t kTailMaxNodes = 300000;

void choose_tail(stz_mg_handle h) {
    h->tail_lo = -1;
    h->tail_cluster = 0;
    // off unless asked for: one 8-16 SM cluster is latency bound on these
    // levels (see the design notes); kept for measurement
    if (!std::getenv("STZ_MG_TAIL")) return;
    const int L = h->nlev;
    int lo = -1;
    for (int l = 1; l <= L - 2; l++)
        if (npts(h->geo[l]) <= kTailMaxNodes) { lo = l; break; }
    if (lo < 0) return;
    const bool mixed = h->d.precision == STZ_MG_MIXED;
    const size_t tsz = mixed ? sizeof(float) : sizeof(double);
    int cap = 0;
    for (int l = lo; l <= L - 2; l++)
        if (h->op64[l].kind == OP_PLANE) cap = std::max(cap, h->geo[l].o);
    const int budget = 200 * 1024;
    if ((size_t)cap * 252 * tsz > (size_t)budget) cap = (int)(budget / (252 * tsz));
    const int smem = (int)(cap * 252 * tsz);
    const int cl = mixed ? tail_cluster_size<float>(smem) : tail_cluster_size<double>(smem);
    cudaGetLastError();
    if (cl == 0) return;
    h->tail_lo = lo;
    h->tail_cluster = cl;
    h->tail_cap_planes = cap;
}

// Wall time of set-up phases on stderr when STZ_MG_TRACE is set (the stream
// is synchronised at each mark, so only for measurement).
struct PhaseTrace {
    stz_mg_handle h;
    bool on;
    std::chrono::steady_clock::time_point t0;
    explicit PhaseTrace(stz_mg_handle hh) : h(hh), on(std::getenv("STZ_MG_TRACE") != nullptr) {
        if (on) t0 = std::chrono::steady_clock::now();
    }
    void mark(const char *what) {
        if (!on) return;
        sync(h);
        auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "stz_mg setup: %-22s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t - t0).count());
        t0 = t;
    }
};

void setup(stz_mg_handle h) {
    if (h->top_kind < 0) fail(STZ_MG_ERR_ARG, "no operator: call stz_mg_set_stencil_const, _points or _coeffs_lame first");
    invalidate(h);
    PhaseTrace trace(h);
    const bool mixed = h->d.precision == STZ_MG_MIXED;
    // top level: dense per-point operator needs its centre inverses
    if (h->top_kind == OP_DENSE) {
        const Geom &g = h->geo[0];
        CK(cudaMemsetAsync(h->dflag, 0, sizeof(int), h->st));
        launch_dense_dinv<double>(g, h->top_coef64, h->top_dinv64, h->dflag, h->st);
        check_launch();
        h->op64[0].dop.dinv = h->top_dinv64;
        if (mixed) {
            launch_convert(h->top_coef64, h->top_coef32, 243 * (size_t)g.npad, h->st);
            launch_convert(h->top_dinv64, h->top_dinv32, 9 * (size_t)g.npad, h->st);
            check_launch();
            h->op32[0].dop.coef = h->top_coef32;
            h->op32[0].dop.dinv = h->top_dinv32;
        }
    }
    launch_top_bounds(h->geo[0], h->S[0], h->st);
    check_launch();
    CK(cudaMemsetAsync(h->dflag, 0, 2 * sizeof(int), h->st));
    // A shared stencil on a grid periodic in x and y gives Galerkin operators
    // that are the same on every node of an x-y plane: store and build one
    // row per plane (exact, not an approximation).
    const bool plane = h->top_kind == OP_CONST && h->geo[0].xp && h->geo[0].yp;
    for (int l = 1; l < h->nlev; l++) {
        const Geom &gf = h->geo[l - 1], &gc = h->geo[l];
        const size_t rows = plane ? (size_t)gc.o : (size_t)gc.npad;
        Level<double> &C = h->L64[l];
        if (C.coef_rows != rows) {
            h->release(C.coef);
            h->release(C.dinv);
            C.coef = h->alloc<double>(243 * rows);
            C.dinv = h->alloc<double>(9 * rows);
            C.coef_rows = rows;
        }
        launch_rat_bounds(gf, h->S[l - 1], gc, h->S[l], h->dflag + 1, h->st);
        launch_rat(h->op64[l - 1], gf, gc, C.coef, plane, h->st);
        if (plane) launch_plane_dinv<double>(gc.o, C.coef, C.dinv, h->dflag, h->st);
        else launch_dense_dinv<double>(gc, C.coef, C.dinv, h->dflag, h->st);
        check_launch();
        h->op64[l] = LevelOp<double>{};
        int sparse = 0, sparse32 = 0;
        if (plane) {
            // The Galerkin operators of the constant elasticity stencil vanish on
            // the entries outside coarse_entry() up to cancellation round-off.
            // FP64 kernels skip them only when they are exactly zero; FP32
            // kernels when they are below 1e-9 of the plane's largest entry
            // (far below FP32 resolution).
            std::vector<double> pc(243 * rows);
            CK(cudaMemcpyAsync(pc.data(), C.coef, pc.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
            sync(h);
            double worst_rel = 0.0;
            bool exact = true;
            for (size_t k = 0; k < rows; k++) {
                double amax = 0.0, dropped = 0.0;
                for (int b = 0; b < 27; b++)
                    for (int e = 0; e < 9; e++) {
                        double v = std::fabs(pc[(9 * b + e) * rows + k]);
                        amax = std::max(amax, v);
                        if (!coarse_entry(b, e)) dropped = std::max(dropped, v);
                    }
                if (dropped != 0.0) exact = false;
                if (amax > 0) worst_rel = std::max(worst_rel, dropped / amax);
            }
            sparse = exact;
            sparse32 = worst_rel <= 1e-9;
        }
        if (plane) {
            h->op64[l].kind = OP_PLANE;
            h->op64[l].pop = PlaneOp<double>{C.coef, C.dinv, gc.o, sparse};
        } else {
            h->op64[l].kind = OP_DENSE;
            h->op64[l].dop = DenseOp<double>{C.coef, C.dinv};
        }
        if (mixed) {
            Level<float> &F = h->L32[l];
            if (F.coef_rows != rows) {
                h->release(F.coef);
                h->release(F.dinv);
                F.coef = h->alloc<float>(243 * rows);
                F.dinv = h->alloc<float>(9 * rows);
                F.coef_rows = rows;
            }
            launch_convert(C.coef, F.coef, 243 * rows, h->st);
            launch_convert(C.dinv, F.dinv, 9 * rows, h->st);
            check_launch();
            h->op32[l] = LevelOp<float>{};
            if (plane) {
                h->op32[l].kind = OP_PLANE;
                h->op32[l].pop = PlaneOp<float>{F.coef, F.dinv, gc.o, sparse32};
            } else {
                h->op32[l].kind = OP_DENSE;
                h->op32[l].dop = DenseOp<float>{F.coef, F.dinv};
            }
        }
    }
    int flags[2] = {0, 0};
    CK(cudaMemcpyAsync(flags, h->dflag, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    sync(h);
    if (flags[1]) fail(STZ_MG_ERR_UNSUPPORTED, "RAT box bounds out of range");
    if (flags[0]) fail(STZ_MG_ERR_SINGULAR, "singular or non-finite diagonal block on a coarse level");
    trace.mark("coarse operators (RAT)");
    if (h->d.bottom == STZ_MG_BOTTOM_DIRECT) build_bottom(h);
    trace.mark("bottom inverse");
    choose_tail(h);
    h->setup_done = true;
}

// ------------------------------------------------------------ cycles
template <typename T>
struct Hier {
    Level<T> *L;
    LevelOp<T> *op;
};

template <typename T>
void bottom_solve(stz_mg_handle h, Hier<T> H) {
    const int lb = h->nlev - 1;
    const Geom &g = h->geo[lb];
    if (h->d.bottom == STZ_MG_BOTTOM_DIRECT) {
        launch_bottom_direct<T>(h->nbot_rows, h->ainv_t, h->nat_slot, g.npad, H.L[lb].r, H.L[lb].x, h->st);
    } else {
        launch_gs_sweeps<T>(H.op[lb], g, H.L[lb].r, H.L[lb].x, H.L[lb].res, h->d.bottom_sweeps, h->st);
    }
}

// multigrid::v_cycle (multigrid.cc:253-297): level i gets v_down+i sweeps
// going down, then restriction (residual + (1/8)P^T, coarse x cleared); the
// bottom is solved; going up, interpolation then v_up+i-1 sweeps.
template <typename T>
TailDesc<T> tail_desc(stz_mg_handle h, Hier<T> H) {
    TailDesc<T> d{};
    d.lo = h->tail_lo;
    d.hi = h->nlev - 2;
    d.v_down = h->d.v_down;
    d.v_up = h->d.v_up;
    d.growth = h->d.sweep_growth;
    d.cap_planes = h->tail_cap_planes;
    for (int l = 0; l < h->nlev; l++) {
        TailLev<T> &t = d.L[l];
        t.g = h->geo[l];
        t.kind = H.op[l].kind;
        if (t.kind == OP_PLANE) {
            t.coef = H.op[l].pop.coef; t.dinv = H.op[l].pop.dinv; t.O = H.op[l].pop.O; t.sparse = H.op[l].pop.sparse;
        } else {
            t.coef = H.op[l].dop.coef; t.dinv = H.op[l].dop.dinv; t.O = 0; t.sparse = 0;
        }
        t.x = H.L[l].x; t.r = H.L[l].r; t.res = H.L[l].res;
    }
    return d;
}

// multigrid::v_cycle (multigrid.cc:253-297) with the levels below the tail
// threshold run by the two persistent cluster kernels.
template <typename T>
void enqueue_vcycle(stz_mg_handle h, Hier<T> H) {
    const int L = h->nlev;
    const int lo = h->tail_lo >= 0 ? h->tail_lo : L - 1;
    for (int i = 0; i < lo; i++) {
        const Geom &g = h->geo[i];
        launch_gs_sweeps<T>(H.op[i], g, H.L[i].r, H.L[i].x, H.L[i].res, h->d.v_down + (h->d.sweep_growth ? i : 0),
                            h->st);
        if (!launch_residual_restrict<T>(H.op[i], g, h->geo[i + 1], H.L[i].r, H.L[i].x, H.L[i + 1].r, h->st)) {
            launch_residual<T, T>(H.op[i], g, H.L[i].r, H.L[i].x, H.L[i].res, nullptr, nullptr, h->st);
            launch_restriction<T>(g, h->geo[i + 1], H.L[i].res, H.L[i + 1].r, h->st);
        }
        CK(cudaMemsetAsync(H.L[i + 1].x, 0, 3 * (size_t)h->geo[i + 1].npad * sizeof(T), h->st));
    }
    TailDesc<T> td{};
    if (h->tail_lo >= 0) {
        td = tail_desc<T>(h, H);
        CK(launch_tail_down<T>(td, h->tail_cluster, h->st));
    }
    bottom_solve<T>(h, H);
    if (h->tail_lo >= 0) CK(launch_tail_up<T>(td, h->tail_cluster, h->st));
    for (int i = lo; i > 0; i--) {
        launch_interpolation<T>(h->geo[i - 1], h->geo[i], H.L[i].x, H.L[i - 1].x, h->st);
        launch_gs_sweeps<T>(H.op[i - 1], h->geo[i - 1], H.L[i - 1].r, H.L[i - 1].x, H.L[i - 1].res,
                            h->d.v_up + (h->d.sweep_growth ? i - 1 : 0), h->st);
    }
}

template <typename T>
cudaGraphExec_t capture_vcycle(stz_mg_handle h, Hier<T> H, long long *kernel_nodes) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue_vcycle<T>(h, H);
    } catch (...) {
        cudaStreamEndCapture(h->st, &graph);
        throw;
    }
    CK(cudaStreamEndCapture(h->st, &graph));
    size_t nn = 0;
    CK(cudaGraphGetNodes(graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
    long long nk = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) nk++;
    }
    *kernel_nodes = nk;
    cudaGraphExec_t ex;
    CK(cudaGraphInstantiate(&ex, graph, 0));
    CK(cudaGraphDestroy(graph));
    return ex;
}

Hier<double> hier64(stz_mg_handle h) { return Hier<double>{h->L64, h->op64}; }
Hier<float> hier32(stz_mg_handle h) { return Hier<float>{h->L32, h->op32}; }

void run_vcycle64(stz_mg_handle h, int count) {
    if (!h->gx64) h->gx64 = capture_vcycle<double>(h, hier64(h), &h->graph_kernels64);
    for (int c = 0; c < count; c++) CK(cudaGraphLaunch(h->gx64, h->st));
    h->stat_cycles += count;
    h->stat_launches += count * h->graph_kernels64;
}

void run_vcycle32(stz_mg_handle h, int count) {
    if (!h->gx32) h->gx32 = capture_vcycle<float>(h, hier32(h), &h->graph_kernels32);
    for (int c = 0; c < count; c++) CK(cudaGraphLaunch(h->gx32, h->st));
    h->stat_cycles += count;
    h->stat_launches += count * h->graph_kernels32;
}

// |b - A x|^2 of the top FP64 level; when r32 is non-null the residual is
// also written there in FP32 (the right-hand side of the correction solve).
double rhs_norm(stz_mg_handle h);

// The residual of the mixed solver's correction steps (r32 non-null): in
// double-float arithmetic on a shared-stencil top level (residual_df.cu),
// with x split into float pairs in the FP64 level's res field (scratch: the
// calls that report a residual recompute it there) -- else in FP64.  With
// corr non-null the correction x += corr is applied first (in the split's
// pass where the double-float residual runs).  Returns |b - A x|^2 in FP64.
double top_residual_sq(stz_mg_handle h, float *r32, const float *corr = nullptr) {
    const Geom &g = h->geo[0];
    double unscale = 1.0;
    if (r32 && residual_df_applies(h->op64[0])) {
        const double bn = rhs_norm(h);
        const double scale = df_norm_scale(bn * bn, 3 * npts(g));
        launch_residual_df(h->op64[0], g, h->L64[0].r, h->L64[0].x, corr, reinterpret_cast<float2 *>(h->L64[0].res),
                           r32, scale, h->partial, h->dscal, h->st);
        unscale = 1.0 / (scale * scale);
        h->stat_launches += 1;   // the split of x
    } else if (corr) {
        launch_add_correction(h->L64[0].x, corr, 3 * (size_t)g.npad, h->st);
        h->stat_launches += 1;
        return top_residual_sq(h, r32);
    } else if (r32) {
        launch_residual<double, float>(h->op64[0], g, h->L64[0].r, h->L64[0].x, r32, h->partial, h->dscal, h->st);
    } else {
        launch_residual<double, double>(h->op64[0], g, h->L64[0].r, h->L64[0].x, (double *)nullptr, h->partial,
                                        h->dscal, h->st);
    }
    check_launch();
    h->stat_residuals++;
    h->stat_launches += 2;   // residual + partial-sum reduction
    CK(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    sync(h);
    double v = h->hscal[0] * unscale;
    if (!std::isfinite(v)) fail(STZ_MG_ERR_NONFINITE, "residual is not finite");
    return v;
}

// |b|_2 of the top level, cached until the right-hand side changes: a plain
// sum of squares over the field (the slots of no node hold zero).
double rhs_norm(stz_mg_handle h) {
    if (h->bnorm < 0) {
        const Geom &g = h->geo[0];
        const int nb = std::min(h->partial_len, 4 * 152);
        sumsq_partial_kernel<<<nb, 256, 0, h->st>>>(h->L64[0].r, 3 * (size_t)g.npad, h->partial);
        sum_blocks_kernel<<<1, 1024, 0, h->st>>>(h->partial, nb, h->dscal);
        check_launch();
        CK(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
        h->bnorm = std::sqrt(h->hscal[0]);
        if (!std::isfinite(h->bnorm)) fail(STZ_MG_ERR_NONFINITE, "right-hand side is not finite");
    }
    return h->bnorm;
}

// Whether the top-level x is zero (the usual start of a solve): then b - A x
// is b and the first FP64 residual pass is not needed.
bool top_x_is_zero(stz_mg_handle h) {
    const size_t n = 3 * (size_t)h->geo[0].npad;
    CK(cudaMemsetAsync(h->dflag, 0, sizeof(int), h->st));
    const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16));
    nonzero_kernel<<<blocks, 256, 0, h->st>>>(h->L64[0].x, n, h->dflag);
    check_launch();
    h->stat_launches += 1;
    int flag = 1;
    CK(cudaMemcpyAsync(&flag, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    sync(h);
    return flag == 0;
}

// One mixed-precision defect-correction step with k FP32 V-cycles:
// r32 = b - A x (FP64 residual rounded to FP32), e = 0, k cycles on A e = r32,
// x += e in FP64 -- here, or (apply false) by the caller's next
// top_residual_sq(h, r32, e).
void mixed_step(stz_mg_handle h, int k, bool apply = true) {
    const Geom &g = h->geo[0];
    const size_t n3 = 3 * (size_t)g.npad;
    CK(cudaMemsetAsync(h->L32[0].x, 0, n3 * sizeof(float), h->st));
    run_vcycle32(h, k);
    if (!apply) return;
    launch_add_correction(h->L64[0].x, h->L32[0].x, n3, h->st);
    check_launch();
    h->stat_launches += 1;
}

void solve(stz_mg_handle h, double tol, int max_cycles, int *cycles_out, double *relres_out) {
    need_setup(h);
    h->stat_cycles = h->stat_residuals = 0;
    h->stat_launches = 0;
    const double bn = rhs_norm(h);
    const double target = tol * (bn > 0 ? bn : 1.0);
    const bool x_zero = top_x_is_zero(h);
    int cycles = 0;
    double rsq;
    if (h->d.precision == STZ_MG_FP64) {
        rsq = x_zero ? bn * bn : top_residual_sq(h, nullptr);
        while (std::sqrt(rsq) > target && cycles < max_cycles) {
            run_vcycle64(h, 1);
            cycles++;
            rsq = top_residual_sq(h, nullptr);
        }
    } else {
        // defect correction: each step solves A e = b - A x with FP32 V-cycles;
        // the number of cycles per step follows the observed contraction so
        // that each step gains about five digits (the FP32 floor) or reaches
        // the tolerance.
        if (x_zero) {   // the correction's right-hand side is b itself
            launch_convert(h->L64[0].r, h->L32[0].r, 3 * (size_t)h->geo[0].npad, h->st);
            check_launch();
            h->stat_launches += 1;
            rsq = bn * bn;
        } else {
            rsq = top_residual_sq(h, h->L32[0].r);
        }
        double rn = std::sqrt(rsq), rho = 0.2;
        int k = 6;
        const bool trace = std::getenv("STZ_MG_TRACE") != nullptr;
        while (rn > target && cycles < max_cycles) {
            k = std::max(1, std::min(k, max_cycles - cycles));
            mixed_step(h, k, false);   // x += e in the residual's first pass
            cycles += k;
            rsq = top_residual_sq(h, h->L32[0].r, h->L32[0].x);
            double rn_new = std::sqrt(rsq);
            if (trace) fprintf(stderr, "stz_mg mixed: %d cycles, |r|/|b| %.3e -> %.3e\n", k, rn / bn, rn_new / bn);
            double gain = rn_new / rn;
            if (gain > 0 && gain < 1) rho = std::min(0.9, std::max(1e-3, std::pow(gain, 1.0 / k)));
            else rho = 0.9;
            rn = rn_new;
            // aim a decade below the tolerance when it is within reach, so the
            // last step does not fall just short (each step costs an FP64 residual)
            double want = std::max(0.1 * target / rn, 1e-6);
            k = (int)std::ceil(std::log(want) / std::log(rho) - 1e-9);
            k = std::max(1, std::min(k, 12));
        }
    }
    check_band(h);
    if (cycles_out) *cycles_out = cycles;
    double rel = std::sqrt(rsq) / (bn > 0 ? bn : 1.0);
    if (relres_out) *relres_out = rel;
    if (std::sqrt(rsq) > target)
        fail(STZ_MG_ERR_NOCONV, "not converged: relative residual %.3e after %d cycles", rel, cycles);
}

}  // namespace

// ====================================================================== C-ABI
extern "C" {

void stz_mg_desc_default(stz_mg_desc *d) {
    if (!d) return;
    std::memset(d, 0, sizeof *d);
    d->precision = STZ_MG_FP64;
    d->v_down = 2;
    d->v_up = 2;
    d->max_coarse = 1024;
    d->bottom = STZ_MG_BOTTOM_DIRECT;
    d->bottom_sweeps = 24;
    d->sweep_growth = 1;
    d->device = 0;
    d->stream = nullptr;
}

const char *stz_mg_last_error(void) { return g_last_error.c_str(); }

int stz_mg_create(const stz_mg_desc *desc, stz_mg_handle *out) {
    if (!desc || !out) return set_error(STZ_MG_ERR_ARG, "null argument");
    *out = nullptr;
    const stz_mg_desc &d = *desc;
    if (d.m < 1 || d.n < 1 || d.o < 1) return set_error(STZ_MG_ERR_ARG, "grid sizes must be positive");
    if (d.precision != STZ_MG_FP64 && d.precision != STZ_MG_MIXED) return set_error(STZ_MG_ERR_ARG, "bad precision");
    if (d.bottom != STZ_MG_BOTTOM_DIRECT && d.bottom != STZ_MG_BOTTOM_GS) return set_error(STZ_MG_ERR_ARG, "bad bottom");
    if (d.v_down < 0 || d.v_up < 0 || d.bottom_sweeps < 0 || d.max_coarse < 1)
        return set_error(STZ_MG_ERR_ARG, "negative sweep count or max_coarse < 1");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_error(STZ_MG_ERR_CUDA, "no CUDA device available");
    if (d.device < 0 || d.device >= ndev) return set_error(STZ_MG_ERR_ARG, "bad device ordinal %d", d.device);
    stz_mg_handle h = new (std::nothrow) stz_mg_handle_s();
    if (!h) return set_error(STZ_MG_ERR_OOM, "host allocation failed");
    h->d = d;
    int rc = guarded(h, [&] {
        if (d.stream) {
            h->st = (cudaStream_t)d.stream;
        } else {
            CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
            h->own_stream = true;
        }
        build_geometry(h);
        alloc_fields(h);
        sync(h);
    });
    if (rc != STZ_MG_OK) {
        stz_mg_destroy(h);
        return rc;
    }
    *out = h;
    return STZ_MG_OK;
}

int stz_mg_destroy(stz_mg_handle h) {
    if (!h) return STZ_MG_OK;
    cudaSetDevice(h->d.device);
    if (h->st) cudaStreamSynchronize(h->st);
    release_graphs(h);
    for (void *p : h->allocs) cudaFree(p);
    if (h->hscal) cudaFreeHost(h->hscal);
    if (h->own_stream && h->st) cudaStreamDestroy(h->st);
    delete h;
    return STZ_MG_OK;
}

int stz_mg_set_stencil_const(stz_mg_handle h, const double *stencil, const double *fix) {
    if (!h || !stencil || !fix) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        invalidate(h);
        set_const_op(h, stencil, fix);
    });
}

int stz_mg_set_stencil_points(stz_mg_handle h, const double *A, int where) {
    if (!h || !A) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        invalidate(h);
        const Geom &g = h->geo[0];
        const size_t n = 243 * npts(g);
        const double *src = to_device(h, A, n, where);
        require_finite(h, src, n, "stencil");
        if (!h->top_coef64) {
            h->top_coef64 = h->alloc<double>(243 * (size_t)g.npad);
            h->top_dinv64 = h->alloc<double>(9 * (size_t)g.npad);
            if (h->d.precision == STZ_MG_MIXED) {
                h->top_coef32 = h->alloc<float>(243 * (size_t)g.npad);
                h->top_dinv32 = h->alloc<float>(9 * (size_t)g.npad);
            }
        }
        CK(cudaMemsetAsync(h->top_coef64, 0, 243 * (size_t)g.npad * sizeof(double), h->st));
        launch_coef_nat_to_cb(g, src, h->top_coef64, h->st);
        check_launch();
        // Dirichlet nodes keep only their centre block (fill_entries stores one entry)
        h->op64[0] = LevelOp<double>{};
        h->op64[0].kind = OP_DENSE;
        h->op64[0].dop.coef = h->top_coef64;
        h->op64[0].dop.dinv = h->top_dinv64;
        h->op32[0] = LevelOp<float>{};
        h->op32[0].kind = OP_DENSE;
        h->top_kind = OP_DENSE;
        sync(h);
    });
}

int stz_mg_set_coeffs_lame(stz_mg_handle h, const double *mu, const double *lam, double dx, double dy, double dz,
                           double dt, int where) {
    if (!h || !mu || !lam) return set_error(STZ_MG_ERR_ARG, "null argument");
    if (!(dx > 0 && dy > 0 && dz > 0 && std::isfinite(dt))) return set_error(STZ_MG_ERR_ARG, "bad spacing or dt");
    return guarded(h, [&] {
        invalidate(h);
        const Geom &g = h->geo[0];
        const size_t n = npts(g);
        if (!h->mu64) {
            h->mu64 = h->alloc<double>(g.npad);
            h->lam64 = h->alloc<double>(g.npad);
            CK(cudaMemsetAsync(h->mu64, 0, g.npad * sizeof(double), h->st));
            CK(cudaMemsetAsync(h->lam64, 0, g.npad * sizeof(double), h->st));
            if (h->d.precision == STZ_MG_MIXED) {
                h->mu32 = h->alloc<float>(g.npad);
                h->lam32 = h->alloc<float>(g.npad);
            }
        }
        const double *s1 = to_device(h, mu, n, where);
        require_finite(h, s1, n, "mu");
        launch_scalar_nat_to_cb<double>(g, s1, h->mu64, h->st);
        sync(h);
        const double *s2 = to_device(h, lam, n, where);
        require_finite(h, s2, n, "lambda");
        launch_scalar_nat_to_cb<double>(g, s2, h->lam64, h->st);
        check_launch();
        h->op64[0] = LevelOp<double>{};
        h->op64[0].kind = OP_LAME;
        h->op64[0].lop = make_lame_op<double>(h->mu64, h->lam64, dx, dy, dz, dt);
        if (h->d.precision == STZ_MG_MIXED) {
            launch_convert(h->mu64, h->mu32, g.npad, h->st);
            launch_convert(h->lam64, h->lam32, g.npad, h->st);
            check_launch();
            h->op32[0] = LevelOp<float>{};
            h->op32[0].kind = OP_LAME;
            h->op32[0].lop = make_lame_op<float>(h->mu32, h->lam32, dx, dy, dz, dt);
        }
        h->top_kind = OP_LAME;
        sync(h);
    });
}

int stz_mg_setup(stz_mg_handle h) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] { setup(h); });
}

int stz_mg_set_rhs(stz_mg_handle h, const double *r, int where) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const double *src = to_device(h, r, 3 * npts(g), where);
        launch_nat_to_cb<double>(g, src, h->L64[0].r, h->st);
        check_launch();
        h->bnorm = -1.0;
        sync(h);   // the caller may reuse or free r once this returns
    });
}

int stz_mg_set_x(stz_mg_handle h, const double *x, int where) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const double *src = to_device(h, x, 3 * npts(g), where);
        launch_nat_to_cb<double>(g, src, h->L64[0].x, h->st);
        check_launch();
        sync(h);   // the caller may reuse or free x once this returns
    });
}

int stz_mg_get_x(stz_mg_handle h, double *x, int where) {
    if (!h || !x) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const size_t n = 3 * npts(g);
        if (where == STZ_MG_DEVICE) {
            launch_cb_to_nat<double>(g, h->L64[0].x, x, h->st);
            check_launch();
            sync(h);   // x is complete when this returns, whatever stream reads it next
        } else {
            double *d = staging(h, n);
            launch_cb_to_nat<double>(g, h->L64[0].x, d, h->st);
            check_launch();
            CK(cudaMemcpyAsync(x, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
            sync(h);
        }
    });
}

int stz_mg_get_rhs(stz_mg_handle h, double *r, int where) {
    if (!h || !r) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const size_t n = 3 * npts(g);
        double *d = where == STZ_MG_DEVICE ? r : staging(h, n);
        launch_cb_to_nat<double>(g, h->L64[0].r, d, h->st);
        check_launch();
        if (where != STZ_MG_DEVICE) CK(cudaMemcpyAsync(r, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    });
}

int stz_mg_set_rhs_divergence(stz_mg_handle h, const double *eps, double dx, double dy, double dz, int where) {
    if (!h || !eps) return set_error(STZ_MG_ERR_ARG, "null argument");
    if (!(dx > 0 && dy > 0 && dz > 0)) return set_error(STZ_MG_ERR_ARG, "bad spacing");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const size_t ncells = (size_t)(g.xp ? g.m : g.m - 1) * (g.yp ? g.n : g.n - 1) * (g.zp ? g.o : g.o - 1);
        const double *src = to_device(h, eps, 6 * ncells, where);
        launch_rhs_divergence(g, src, dx, dy, dz, h->L64[0].r, h->st);
        check_launch();
        h->bnorm = -1.0;
        sync(h);
    });
}

int stz_mg_stress_update(stz_mg_handle h, double *sigma, double lam, double mu, double dt, double dx, double dy,
                         double dz, double *proj_mag, int where) {
    if (!h || !sigma) return set_error(STZ_MG_ERR_ARG, "null argument");
    if (!(dx > 0 && dy > 0 && dz > 0)) return set_error(STZ_MG_ERR_ARG, "bad spacing");
    if (where != STZ_MG_HOST && where != STZ_MG_DEVICE)
        return set_error(STZ_MG_ERR_ARG, "where must be STZ_MG_HOST or STZ_MG_DEVICE");
    return guarded(h, [&] {
        const Geom &g = h->geo[0];
        const size_t ncells = (size_t)(g.xp ? g.m : g.m - 1) * (g.yp ? g.n : g.n - 1) * (g.zp ? g.o : g.o - 1);
        double *dsig = sigma;
        if (where == STZ_MG_HOST) {
            dsig = staging(h, 6 * ncells);
            CK(cudaMemcpyAsync(dsig, sigma, 6 * ncells * sizeof(double), cudaMemcpyHostToDevice, h->st));
        }
        const int nb = std::min(h->partial_len, 4 * 152);
        launch_stress_update(g, h->L64[0].x, dsig, lam, mu, dt, dx, dy, dz, h->partial, nb, h->st);
        sum_blocks_kernel<<<1, 1024, 0, h->st>>>(h->partial, nb, h->dscal);
        check_launch();
        if (where == STZ_MG_HOST)
            CK(cudaMemcpyAsync(sigma, dsig, 6 * ncells * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CK(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
        if (proj_mag) *proj_mag = h->hscal[0];
    });
}

int stz_mg_vcycle(stz_mg_handle h) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        if (h->d.precision == STZ_MG_FP64) {
            run_vcycle64(h, 1);
        } else {
            // a stz_mg_l2_error_all call just before left b - A x of the
            // current x in the FP32 right-hand side
            if (h->l2_call != h->api_calls - 1) top_residual_sq(h, h->L32[0].r);
            mixed_step(h, 1);
        }
        sync(h);
        check_band(h);
    });
}

int stz_mg_solve(stz_mg_handle h, double rel_tol, int max_cycles, int *cycles, double *relres) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    if (!(rel_tol > 0) || max_cycles < 0) return set_error(STZ_MG_ERR_ARG, "bad tolerance or cycle cap");
    return guarded(h, [&] { solve(h, rel_tol, max_cycles, cycles, relres); });
}

int stz_mg_solve_stats(stz_mg_handle h, int *vcycles, int *residuals, long long *kernel_launches) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    if (vcycles) *vcycles = h->stat_cycles;
    if (residuals) *residuals = h->stat_residuals;
    if (kernel_launches) *kernel_launches = h->stat_launches;
    return STZ_MG_OK;
}

int stz_mg_residual_norm(stz_mg_handle h, double *rnorm, double *bnorm) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        double rs = top_residual_sq(h, nullptr);
        if (rnorm) *rnorm = std::sqrt(rs);
        if (bnorm) *bnorm = rhs_norm(h);
    });
}

int stz_mg_adjoint_solve(stz_mg_handle h, const double *g, double *w, int where, double rel_tol, int max_cycles,
                         int *cycles, double *relres) {
    if (!h || !g || !w) return set_error(STZ_MG_ERR_ARG, "null argument");
    if (!(rel_tol > 0) || max_cycles < 0) return set_error(STZ_MG_ERR_ARG, "bad tolerance or cycle cap");
    if (where != STZ_MG_HOST && where != STZ_MG_DEVICE)
        return set_error(STZ_MG_ERR_ARG, "where must be STZ_MG_HOST or STZ_MG_DEVICE");
    return guarded(h, [&] {
        need_setup(h);
        const LevelOp<double> &top = h->op64[0];
        if (top.kind != OP_CONST && top.kind != OP_LAME)
            fail(STZ_MG_ERR_UNSUPPORTED, "the adjoint solve needs a shared-stencil or Lame top-level operator");
        if (top.kind == OP_CONST) {
            // A_II^T = A_II needs S[d] = S[-d]^T
            for (int b = 0; b < 27; b++)
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        if (top.cop.a[b][3 * r + c] != top.cop.a[26 - b][3 * c + r])
                            fail(STZ_MG_ERR_UNSUPPORTED, "the shared stencil is not symmetric (block %d)", b);
        }
        const Geom &g0 = h->geo[0];
        const size_t n3 = 3 * npts(g0);
        if (!h->adj_g) {
            h->adj_g = h->alloc<double>(n3);
            h->adj_t = h->alloc<double>(n3);
        }
        CK(cudaMemcpyAsync(h->adj_g, g, n3 * sizeof(double),
                           where == STZ_MG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, h->st));
        require_finite(h, h->adj_g, n3, "adjoint right-hand side");
        // interior part: A y = g' with g'_D = 0 gives y_D = 0 and A_II y_I = g_I
        launch_mask_dirichlet(g0, h->adj_g, h->adj_t, h->st);
        launch_nat_to_cb<double>(g0, h->adj_t, h->L64[0].r, h->st);
        check_launch();
        CK(cudaMemsetAsync(h->L64[0].x, 0, 3 * (size_t)g0.npad * sizeof(double), h->st));
        h->bnorm = -1.0;
        solve(h, rel_tol, max_cycles, cycles, relres);
        // Dirichlet part, node by node
        double *wd = where == STZ_MG_DEVICE ? w : h->adj_t;
        launch_cb_to_nat<double>(g0, h->L64[0].x, wd, h->st);
        launch_adjoint_dirichlet(top, g0, h->adj_g, wd, h->st);
        check_launch();
        if (where == STZ_MG_HOST) CK(cudaMemcpyAsync(w, wd, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    });
}

int stz_mg_coeff_grad(stz_mg_handle h, const double *w, const double *u, double *dmu, double *dlam, int where) {
    if (!h || !w || !u || !dmu || !dlam) return set_error(STZ_MG_ERR_ARG, "null argument");
    if (where != STZ_MG_HOST && where != STZ_MG_DEVICE)
        return set_error(STZ_MG_ERR_ARG, "where must be STZ_MG_HOST or STZ_MG_DEVICE");
    return guarded(h, [&] {
        if (h->top_kind != OP_LAME)
            fail(STZ_MG_ERR_UNSUPPORTED, "coefficient gradients need the Lame operator (stz_mg_set_coeffs_lame)");
        const Geom &g0 = h->geo[0];
        const size_t n = npts(g0);
        if (!h->grad_c) h->grad_c = h->alloc<double>(14 * n);
        if (!h->adj_g) {
            h->adj_g = h->alloc<double>(3 * n);
            h->adj_t = h->alloc<double>(3 * n);
        }
        const double *wd = w, *ud = u;
        double *om = dmu, *ol = dlam;
        if (where == STZ_MG_HOST) {
            CK(cudaMemcpyAsync(h->adj_g, w, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->st));
            CK(cudaMemcpyAsync(h->adj_t, u, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->st));
            wd = h->adj_g;
            ud = h->adj_t;
            double *st = staging(h, 2 * n);
            om = st;
            ol = st + n;
        }
        launch_lame_grad(h->op64[0].lop, g0, wd, ud, h->grad_c, om, ol, h->st);
        check_launch();
        if (where == STZ_MG_HOST) {
            CK(cudaMemcpyAsync(dmu, om, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
            CK(cudaMemcpyAsync(dlam, ol, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        }
        sync(h);
    });
}

int stz_mg_l2_error_all(stz_mg_handle h, double *out) {
    if (!h || !out) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        need_setup(h);
        if (h->l2_call == h->api_calls - 1) {   // nothing has run since the last evaluation
            h->l2_call = h->api_calls;
            *out = h->l2_value;
            return;
        }
        const Geom &g = h->geo[0];
        const int nb = std::min(h->partial_len, 4 * 152);
        if (h->d.precision == STZ_MG_FP64) {
            // FP64 residual into the top level's res field, then a device sum of |r|^4
            launch_residual<double, double>(h->op64[0], g, h->L64[0].r, h->L64[0].x, h->L64[0].res, nullptr,
                                            nullptr, h->st);
            quartic_partial_kernel<double><<<nb, 256, 0, h->st>>>(h->L64[0].res, g.npad, h->partial);
        } else {
            // the residual the next defect-correction step starts from (FP32
            // top-level right-hand side, formed exactly as stz_mg_vcycle forms
            // it), summed as |r|^4 in FP64; stz_mg_vcycle then reuses it
            top_residual_sq(h, h->L32[0].r);
            quartic_partial_kernel<float><<<nb, 256, 0, h->st>>>(h->L32[0].r, g.npad, h->partial);
        }
        sum_blocks_kernel<<<1, 1024, 0, h->st>>>(h->partial, nb, h->dscal);
        check_launch();
        CK(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
        if (!std::isfinite(h->hscal[0])) fail(STZ_MG_ERR_NONFINITE, "residual is not finite");
        *out = h->l2_value = h->hscal[0];
        h->l2_call = h->api_calls;
    });
}

int stz_mg_num_levels(stz_mg_handle h, int *nlevels) {
    if (!h || !nlevels) return set_error(STZ_MG_ERR_ARG, "null argument");
    *nlevels = h->nlev;
    return STZ_MG_OK;
}

int stz_mg_level_dims(stz_mg_handle h, int level, int *dims3) {
    if (!h || !dims3) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        check_level(h, level);
        dims3[0] = h->geo[level].m; dims3[1] = h->geo[level].n; dims3[2] = h->geo[level].o;
    });
}

int stz_mg_level_operator(stz_mg_handle h, int level, double *A, int *S) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        const Geom &g = h->geo[level];
        const size_t N = npts(g);
        if (A) {
            double *dcoef = nullptr;
            const double *src;
            if (h->op64[level].kind != OP_DENSE) {
                dcoef = h->alloc<double>(243 * (size_t)g.npad);
                launch_expand_dense(h->op64[level], g, dcoef, h->st);
                src = dcoef;
            } else {
                src = h->op64[level].dop.coef;
            }
            double *nat = staging(h, 243 * N);
            launch_coef_cb_to_nat(g, src, nat, h->st);
            check_launch();
            CK(cudaMemcpyAsync(A, nat, 243 * N * sizeof(double), cudaMemcpyDefault, h->st));
            sync(h);
            h->release(dcoef);
        }
        if (S) {
            int *tmp = h->alloc<int>(6 * N);
            launch_bounds_cb_to_nat(g, h->S[level], tmp, h->st);
            check_launch();
            CK(cudaMemcpyAsync(S, tmp, 6 * N * sizeof(int), cudaMemcpyDefault, h->st));
            sync(h);
            h->release(tmp);
        }
    });
}

// The FP64 field `which` of a level.
double *level_field(stz_mg_handle h, int level, int which) {
    if (which == STZ_MG_FIELD_X) return h->L64[level].x;
    if (which == STZ_MG_FIELD_R) return h->L64[level].r;
    if (which == STZ_MG_FIELD_RES) return h->L64[level].res;
    fail(STZ_MG_ERR_ARG, "which must be STZ_MG_FIELD_X, _R or _RES");
}

int stz_mg_level_set_field(stz_mg_handle h, int level, int which, const double *v, int where) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        check_level(h, level);
        const Geom &g = h->geo[level];
        double *dst = level_field(h, level, which);
        const double *src = to_device(h, v, 3 * npts(g), where);
        launch_nat_to_cb<double>(g, src, dst, h->st);
        check_launch();
        if (level == 0 && which == STZ_MG_FIELD_R) h->bnorm = -1.0;
        sync(h);
    });
}

int stz_mg_level_get_field(stz_mg_handle h, int level, int which, double *v, int where) {
    if (!h || !v) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        check_level(h, level);
        const Geom &g = h->geo[level];
        const size_t n = 3 * npts(g);
        const double *src = level_field(h, level, which);
        double *d = where == STZ_MG_DEVICE ? v : staging(h, n);
        launch_cb_to_nat<double>(g, src, d, h->st);
        check_launch();
        if (where != STZ_MG_DEVICE) CK(cudaMemcpyAsync(v, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    });
}

int stz_mg_level_get_planes(stz_mg_handle h, int level, int which, int k0, int nk, double *v, int where) {
    if (!h || !v) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        check_level(h, level);
        const Geom &g = h->geo[level];
        if (k0 < 0 || nk < 0 || k0 + nk > g.o) fail(STZ_MG_ERR_ARG, "planes %d..%d outside [0,%d)", k0, k0 + nk, g.o);
        const double *src = level_field(h, level, which);
        const size_t n = 3 * (size_t)g.m * g.n * nk;
        if (n == 0) return;
        if (where != STZ_MG_HOST && where != STZ_MG_DEVICE) fail(STZ_MG_ERR_ARG, "bad where");
        double *d = where == STZ_MG_DEVICE ? v : staging(h, n);
        const unsigned blocks = (unsigned)std::min<size_t>((n / 3 + 255) / 256, 152 * 8);
        planes_cb_to_nat_kernel<<<blocks, 256, 0, h->st>>>(g, k0, nk, src, d);
        check_launch();
        if (where == STZ_MG_HOST) CK(cudaMemcpyAsync(v, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        sync(h);
    });
}

int stz_mg_level_set_planes(stz_mg_handle h, int level, int which, int k0, int nk, const double *v, int where) {
    if (!h || !v) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        check_level(h, level);
        const Geom &g = h->geo[level];
        if (k0 < 0 || nk < 0 || k0 + nk > g.o) fail(STZ_MG_ERR_ARG, "planes %d..%d outside [0,%d)", k0, k0 + nk, g.o);
        double *dst = level_field(h, level, which);
        const size_t n = 3 * (size_t)g.m * g.n * nk;
        if (n == 0) return;
        const double *src = to_device(h, v, n, where);
        const unsigned blocks = (unsigned)std::min<size_t>((n / 3 + 255) / 256, 152 * 8);
        planes_nat_to_cb_kernel<<<blocks, 256, 0, h->st>>>(g, k0, nk, src, dst);
        check_launch();
        if (level == 0 && which == STZ_MG_FIELD_R) h->bnorm = -1.0;
        sync(h);
    });
}

int stz_mg_level_gs_colours(stz_mg_handle h, int level, int q0, int q1) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        if (q0 < 0 || q1 > 8 || q0 > q1) fail(STZ_MG_ERR_ARG, "colours %d..%d outside [0,8)", q0, q1);
        for (int q = q0; q < q1; q++)
            launch_gs_colour<double>(h->op64[level], h->geo[level], q, h->L64[level].r, h->L64[level].x, h->st);
        check_launch();
        sync(h);
    });
}

int stz_mg_level_restrict_residual(stz_mg_handle h, int level) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        if (level < 1) fail(STZ_MG_ERR_ARG, "restriction target must be a coarse level");
        const int f = level - 1;
        launch_restriction<double>(h->geo[f], h->geo[level], h->L64[f].res, h->L64[level].r, h->st);
        CK(cudaMemsetAsync(h->L64[level].x, 0, 3 * (size_t)h->geo[level].npad * sizeof(double), h->st));
        check_launch();
        sync(h);
    });
}

int stz_mg_level_gauss_seidel(stz_mg_handle h, int level, int sweeps) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        launch_gs_sweeps<double>(h->op64[level], h->geo[level], h->L64[level].r, h->L64[level].x, h->L64[level].res,
                                 sweeps, h->st);
        sync(h);
        check_band(h);
    });
}

int stz_mg_level_restriction(stz_mg_handle h, int level) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        if (level < 1) fail(STZ_MG_ERR_ARG, "restriction target must be a coarse level");
        const int f = level - 1;
        launch_residual<double, double>(h->op64[f], h->geo[f], h->L64[f].r, h->L64[f].x, h->L64[f].res, nullptr,
                                        nullptr, h->st);
        launch_restriction<double>(h->geo[f], h->geo[level], h->L64[f].res, h->L64[level].r, h->st);
        CK(cudaMemsetAsync(h->L64[level].x, 0, 3 * (size_t)h->geo[level].npad * sizeof(double), h->st));
        sync(h);
    });
}

int stz_mg_level_interpolation(stz_mg_handle h, int level) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        if (level < 1) fail(STZ_MG_ERR_ARG, "interpolation source must be a coarse level");
        launch_interpolation<double>(h->geo[level - 1], h->geo[level], h->L64[level].x, h->L64[level - 1].x, h->st);
        sync(h);
    });
}

int stz_mg_level_residual(stz_mg_handle h, int level, double *out, double *sumsq, int where) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        const Geom &g = h->geo[level];
        launch_residual<double, double>(h->op64[level], g, h->L64[level].r, h->L64[level].x, h->L64[level].res,
                                        h->partial, h->dscal, h->st);
        check_launch();
        CK(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        if (out) {
            const size_t n = 3 * npts(g);
            double *d = where == STZ_MG_DEVICE ? out : staging(h, n);
            launch_cb_to_nat<double>(g, h->L64[level].res, d, h->st);
            check_launch();
            if (where != STZ_MG_DEVICE) CK(cudaMemcpyAsync(out, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        }
        sync(h);
        if (sumsq) *sumsq = h->hscal[0];
    });
}


int stz_mg_output_slice(stz_mg_handle h, int which, int k, double ax, double bx, double ay, double by,
                        const char *filename) {
    if (!h) return set_error(STZ_MG_ERR_ARG, "null handle");
    return guarded(h, [&] {
        if (which < STZ_MG_SLICE_X || which > STZ_MG_SLICE_RESIDUAL || !filename)
            fail(STZ_MG_ERR_ARG, "stz_mg_output_slice: which must be STZ_MG_SLICE_X, _R or _RESIDUAL");
        const Geom &g = h->geo[0];
        if (k < 0 || k >= g.o) fail(STZ_MG_ERR_ARG, "stz_mg_output_slice: slice out of range");
        if (g.m < 2 || g.n < 2) fail(STZ_MG_ERR_ARG, "stz_mg_output_slice: needs m, n >= 2");
        const double *f = h->L64[0].x;
        if (which == STZ_MG_SLICE_R) f = h->L64[0].r;
        if (which == STZ_MG_SLICE_RESIDUAL) {
            need_setup(h);
            launch_residual<double, double>(h->op64[0], g, h->L64[0].r, h->L64[0].x, h->L64[0].res, nullptr,
                                            nullptr, h->st);
            check_launch();
            f = h->L64[0].res;
        }
        const size_t n = (size_t)g.m * g.n;
        float *d = reinterpret_cast<float *>(staging(h, (n + 1) / 2));
        launch_slice(g, f, k, which == STZ_MG_SLICE_RESIDUAL, d, h->st);
        check_launch();
        std::vector<float> vals(n);
        CK(cudaMemcpyAsync(vals.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
        sync(h);
        if (!write_slice_file(vals.data(), g.m, g.n, ax, bx, ay, by, filename))
            fail(STZ_MG_ERR_ARG, "stz_mg_output_slice: cannot write %s", filename);
    });
}

int stz_mg_sweep_kind(stz_mg_handle h, int level, int *kind, int *launches_per_sweep) {
    if (!h || !kind) return set_error(STZ_MG_ERR_ARG, "null argument");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        const Geom &g = h->geo[level];
        const bool mixed = h->d.precision == STZ_MG_MIXED;
        *kind = mixed ? gs_sweep_kind<float>(h->op32[level], g, h->L32[level].x, true)
                      : gs_sweep_kind<double>(h->op64[level], g, h->L64[level].x, true);
        if (launches_per_sweep) *launches_per_sweep = *kind == 0 ? 8 : 2;
    });
}

int stz_mg_time_kernel(stz_mg_handle h, int kernel, int level, int reps, double *ms_per_launch,
                       double *work_per_launch) {
    if (!h || reps < 1) return set_error(STZ_MG_ERR_ARG, "bad argument");
    return guarded(h, [&] {
        need_setup(h);
        check_level(h, level);
        const bool mixed = h->d.precision == STZ_MG_MIXED;
        const Geom &g = h->geo[level];
        const double npts_l = (double)npts(g);
        const double s = mixed ? 4.0 : 8.0;
        auto coef_bytes = [&](int l) -> double {   // coefficient bytes per node of level l
            const LevelOp<double> &op = h->op64[l];
            if (op.kind == OP_DENSE) return (243 + 9) * s;
            if (op.kind == OP_LAME) return 2 * s;
            if (op.kind == OP_PLANE) return (243 + 9) * s * h->geo[l].o / (double)npts(h->geo[l]);
            return 0.0;
        };
        std::function<void()> launch;
        double work = 0;
        switch (kernel) {
            case STZ_MG_K_GS_COLOUR:
                // a full 8-colour sweep reads x and r and writes x once per node
                work = (9 * s + coef_bytes(level)) * npts_l / 8;
                if (mixed) launch = [&] { launch_gs_colour<float>(h->op32[level], g, 0, h->L32[level].r, h->L32[level].x, h->st); };
                else launch = [&] { launch_gs_colour<double>(h->op64[level], g, 0, h->L64[level].r, h->L64[level].x, h->st); };
                break;
            case STZ_MG_K_GS_SWEEP:
                // two sweeps, as the V-cycle smooths (v_down = v_up = 2)
                work = 2 * (9 * s + coef_bytes(level)) * npts_l;
                if (mixed) launch = [&] { launch_gs_sweeps<float>(h->op32[level], g, h->L32[level].r, h->L32[level].x, h->L32[level].res, 2, h->st); };
                else launch = [&] { launch_gs_sweeps<double>(h->op64[level], g, h->L64[level].r, h->L64[level].x, h->L64[level].res, 2, h->st); };
                break;
            case STZ_MG_K_RESIDUAL:
                work = (9 * s + coef_bytes(level)) * npts_l;
                if (mixed) launch = [&] { launch_residual<float, float>(h->op32[level], g, h->L32[level].r, h->L32[level].x, h->L32[level].res, nullptr, nullptr, h->st); };
                else launch = [&] { launch_residual<double, double>(h->op64[level], g, h->L64[level].r, h->L64[level].x, h->L64[level].res, nullptr, nullptr, h->st); };
                break;
            case STZ_MG_K_RESTRICT: {
                if (level < 1) fail(STZ_MG_ERR_ARG, "restriction target must be a coarse level");
                const Geom &gf = h->geo[level - 1];
                work = 3 * s * ((double)npts(gf) + npts_l);
                if (mixed) launch = [&] { launch_restriction<float>(gf, g, h->L32[level - 1].res, h->L32[level].r, h->st); };
                else launch = [&] { launch_restriction<double>(gf, g, h->L64[level - 1].res, h->L64[level].r, h->st); };
                break;
            }
            case STZ_MG_K_INTERP: {
                if (level < 1) fail(STZ_MG_ERR_ARG, "interpolation source must be a coarse level");
                const Geom &gf = h->geo[level - 1];
                work = 6 * s * (double)npts(gf) + 3 * s * npts_l;
                if (mixed) launch = [&] { launch_interpolation<float>(gf, g, h->L32[level].x, h->L32[level - 1].x, h->st); };
                else launch = [&] { launch_interpolation<double>(gf, g, h->L64[level].x, h->L64[level - 1].x, h->st); };
                break;
            }
            case STZ_MG_K_RESIDUAL64: {
                if (level != 0) fail(STZ_MG_ERR_ARG, "the FP64 residual is a top-level kernel");
                // FP64 flops of r = b - A x with the elasticity stencil: 6 faces x 3 + 12 edges x 2
                // + centre 9 multiply-adds per node (a dense stencil: 243)
                const LevelOp<double> &op = h->op64[0];
                double fma = op.kind == OP_CONST && op.cop.elastic ? 51 : op.kind == OP_LAME ? 51 : 243;
                work = 2 * fma * npts_l;
                if (mixed && residual_df_applies(op)) {
                    // the mixed solver's pass: split of x + double-float residual + sum
                    const double scale = df_norm_scale(rhs_norm(h) * rhs_norm(h), 3 * npts(g));
                    launch = [&, scale] {
                        launch_residual_df(h->op64[0], g, h->L64[0].r, h->L64[0].x, nullptr,
                                           reinterpret_cast<float2 *>(h->L64[0].res), h->L32[0].r, scale, h->partial,
                                           h->dscal, h->st);
                    };
                } else if (mixed) launch = [&] { launch_residual<double, float>(h->op64[0], g, h->L64[0].r, h->L64[0].x, h->L32[0].r, h->partial, h->dscal, h->st); };
                else launch = [&] { launch_residual<double, double>(h->op64[0], g, h->L64[0].r, h->L64[0].x, (double *)nullptr, h->partial, h->dscal, h->st); };
                break;
            }
            default: fail(STZ_MG_ERR_ARG, "unknown kernel id %d", kernel);
        }
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        for (int w = 0; w < 3; w++) launch();
        CK(cudaEventRecord(e0, h->st));
        for (int r = 0; r < reps; r++) launch();
        CK(cudaEventRecord(e1, h->st));
        sync(h);
        check_band(h);
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (ms_per_launch) *ms_per_launch = ms / reps;
        if (work_per_launch) *work_per_launch = work;
    });
}

}  // extern "C"

namespace stzmg {
// Sets the text stz_mg_last_error() returns, for entry points defined in other
// translation units.
int record_error(int code, const char *msg) {
    g_last_error = msg;
    return code;
}
}  // namespace stzmg
