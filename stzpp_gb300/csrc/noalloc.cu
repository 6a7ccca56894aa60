// Residual sum of squares of a shared-stencil grid on caller-owned device
// fields, computed without allocating anything (include/stz_mg.h,
// stz_mg_const_residual_sumsq_noalloc).
//
// The reduction needs one partial sum per thread block.  Those partials live
// in a file-scope __device__ array of fixed size (STZ_MG_NOALLOC_PARTIALS
// doubles, 1 MiB) instead of memory obtained from cudaMalloc, so a call makes
// no allocation of any kind: no cudaMalloc / cudaFree, no pinned host memory,
// no library routine that allocates.  Each block covers kNodesPerBlock nodes,
// which bounds the grids the entry point accepts; larger grids are refused
// with STZ_MG_ERR_ARG before anything is launched.
//
// Nothing has to start at zero: every partial slot the final sum reads has
// been written by the first kernel of the same call, and the result is stored
// (not accumulated) into the caller's double.
//
// All calls on one device share the one scratch array.  Two calls whose
// kernels can run at the same time on one device (different streams, or
// different host threads without ordering between them) race on it and
// corrupt each other's sums: callers serialise them (one stream, or an event).
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/stz_mg.h"

namespace stzmg {
int record_error(int code, const char *msg);   // api.cu: sets stz_mg_last_error()
}

namespace {

constexpr int kThreads = 256;
constexpr int kNodesPerThread = 4;
constexpr int kNodesPerBlock = kThreads * kNodesPerThread;
static_assert((long long)kNodesPerBlock * STZ_MG_NOALLOC_PARTIALS == STZ_MG_NOALLOC_MAX_NODES,
              "header limits disagree with the kernel's blocking");

// The scratch: one partial sum per block of the residual kernel.
static __device__ __align__(256) double g_noalloc_partials[STZ_MG_NOALLOC_PARTIALS];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
double *g_addr[kMaxDevices] = {};

// Device address of the scratch, looked up once per device with that device
// current (the lookup may load the module on the device, so the first call on
// a device is made before the caller starts any stream capture).  The address
// stays valid while the device's primary context lives: a cudaDeviceReset
// between calls would leave it stale, and callers do not reset the device
// between calls.
cudaError_t scratch_address(int device, double **out) {
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_addr[device] = static_cast<double *>(p);
    }
    *out = g_addr[device];
    return cudaSuccess;
}

struct SharedStencil {
    double s[243];   // 27 blocks 3x3 row-major, block 13 + dx + 3 dy + 9 dz
    double f[9];     // Dirichlet fix block
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// One thread: kNodesPerThread nodes kThreads apart (coalesced over x); the
// block's sum of |b - A x|^2 goes to partial[blockIdx.x].
__global__ void __launch_bounds__(kThreads)
    const_residual_sumsq_kernel(const __grid_constant__ SharedStencil A, int m, int n, int o, int xp, int yp,
                                int zp, const double *__restrict__ x, const double *__restrict__ b,
                                double *__restrict__ partial) {
    const long long npts = (long long)m * n * o;
    const long long base = (long long)blockIdx.x * kNodesPerBlock + threadIdx.x;
    double sq = 0.0;
#pragma unroll 1
    for (int s = 0; s < kNodesPerThread; s++) {
        const long long p = base + (long long)s * kThreads;
        if (p >= npts) break;
        const int i = (int)(p % m);
        const long long t = p / m;
        const int j = (int)(t % n);
        const int k = (int)(t / n);
        double a0 = b[3 * p], a1 = b[3 * p + 1], a2 = b[3 * p + 2];
        const bool interior = (xp || (i > 0 && i < m - 1)) && (yp || (j > 0 && j < n - 1)) &&
                              (zp || (k > 0 && k < o - 1));
        if (interior) {
#pragma unroll 1
            for (int dz = -1; dz <= 1; dz++) {
                const long long kk = wrap(k + dz, o);
#pragma unroll
                for (int dy = -1; dy <= 1; dy++) {
                    const long long row = ((long long)wrap(j + dy, n) + n * kk) * m;
#pragma unroll
                    for (int dx = -1; dx <= 1; dx++) {
                        const double *blk = A.s + 9 * (13 + dx + 3 * dy + 9 * dz);
                        const double *v = x + 3 * (row + wrap(i + dx, m));
                        const double v0 = v[0], v1 = v[1], v2 = v[2];
                        a0 -= blk[0] * v0 + blk[1] * v1 + blk[2] * v2;
                        a1 -= blk[3] * v0 + blk[4] * v1 + blk[5] * v2;
                        a2 -= blk[6] * v0 + blk[7] * v1 + blk[8] * v2;
                    }
                }
            }
        } else {
            const double v0 = x[3 * p], v1 = x[3 * p + 1], v2 = x[3 * p + 2];
            a0 -= A.f[0] * v0 + A.f[1] * v1 + A.f[2] * v2;
            a1 -= A.f[3] * v0 + A.f[4] * v1 + A.f[5] * v2;
            a2 -= A.f[6] * v0 + A.f[7] * v1 + A.f[8] * v2;
        }
        sq += a0 * a0 + a1 * a1 + a2 * a2;
    }
    __shared__ double warp_sums[kThreads / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x < 32) {
        sq = threadIdx.x < kThreads / 32 ? warp_sums[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
        if (threadIdx.x == 0) partial[blockIdx.x] = sq;
    }
}

// Sum of the nblocks partials in a fixed order (deterministic), stored to *out.
__global__ void __launch_bounds__(1024) sum_noalloc_partials_kernel(const double *__restrict__ partial, int nblocks,
                                                                    double *__restrict__ out) {
    __shared__ double warp_sums[32];
    double v = 0.0;
    for (int q = threadIdx.x; q < nblocks; q += blockDim.x) v += partial[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = warp_sums[threadIdx.x];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (threadIdx.x == 0) out[0] = v;
    }
}

int cuda_fail(cudaError_t e, const char *what) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return stzmg::record_error(STZ_MG_ERR_CUDA, buf);
}

}  // namespace

extern "C" int stz_mg_const_residual_sumsq_noalloc(int m, int n, int o, int x_prd, int y_prd, int z_prd,
                                                   const double *stencil, const double *fix, const double *x,
                                                   const double *b, double *sumsq, int device, void *stream) {
    if (m < 1 || n < 1 || o < 1) return stzmg::record_error(STZ_MG_ERR_ARG, "grid sizes must be positive");
    const long long npts = (long long)m * n * o;
    if (npts > STZ_MG_NOALLOC_MAX_NODES) {
        char buf[320];
        snprintf(buf, sizeof buf,
                 "grid of %lld nodes is too large for stz_mg_const_residual_sumsq_noalloc: its static scratch "
                 "holds %d partial sums of %d nodes each (at most %lld nodes); use stz_mg_residual_norm",
                 npts, STZ_MG_NOALLOC_PARTIALS, kNodesPerBlock, (long long)STZ_MG_NOALLOC_MAX_NODES);
        return stzmg::record_error(STZ_MG_ERR_ARG, buf);
    }
    if (!stencil || !fix || !x || !b || !sumsq) return stzmg::record_error(STZ_MG_ERR_ARG, "null argument");
    if (device < 0 || device >= kMaxDevices) return stzmg::record_error(STZ_MG_ERR_ARG, "bad device ordinal");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device >= ndev) return stzmg::record_error(STZ_MG_ERR_ARG, "bad device ordinal");
    int prev = -1;
    e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    int rc = STZ_MG_OK;
    double *partial = nullptr;
    if (stream) {   // the stream must belong to `device`
        int sdev = -1;
        e = cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamGetDevice");
        else if (sdev != device) rc = stzmg::record_error(STZ_MG_ERR_ARG, "stream belongs to another device");
        if (rc != STZ_MG_OK) {
            if (prev != device && prev >= 0) cudaSetDevice(prev);
            return rc;
        }
    }
    e = scratch_address(device, &partial);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "cudaGetSymbolAddress");
    } else {
        SharedStencil A;
        for (int q = 0; q < 243; q++) A.s[q] = stencil[q];
        for (int q = 0; q < 9; q++) A.f[q] = fix[q];
        const int nblocks = (int)((npts + kNodesPerBlock - 1) / kNodesPerBlock);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        cudaGetLastError();   // an earlier caller's launch error is not this call's
        const_residual_sumsq_kernel<<<nblocks, kThreads, 0, st>>>(A, m, n, o, x_prd != 0, y_prd != 0, z_prd != 0, x,
                                                                   b, partial);
        sum_noalloc_partials_kernel<<<1, 1024, 0, st>>>(partial, nblocks, sumsq);
        e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "kernel launch");
    }
    if (prev != device && prev >= 0) cudaSetDevice(prev);
    return rc;
}
