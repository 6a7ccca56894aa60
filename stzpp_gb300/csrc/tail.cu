// Persistent kernels for the small levels of the V-cycle.
//
// On the coarse levels a colour pass has a few hundred to a few tens of
// thousands of nodes, so one launch per colour pass (8 per sweep, 2+i sweeps
// each way on level i, multigrid.cc:265,288) is dominated by launch latency.
// Here the whole tail of the cycle below a size threshold runs inside one
// thread-block cluster: the down half (sweeps, residual, restriction, coarse
// x cleared) in one launch, the up half (interpolation, sweeps) in another,
// with the FP64 bottom solve between them as an ordinary full-GPU launch.
// Phases are separated by hardware cluster barriers (all blocks of a cluster
// are co-scheduled, so a barrier cannot wait on a block that never runs), and
// fields written inside the launch are read through L2 (ld.global.cg).
// Plane-invariant coefficients of the current level are staged in shared
// memory when they fit.
#include <cooperative_groups.h>

#include "launch.h"
#include "transfer.cuh"

namespace cg = cooperative_groups;

namespace stzmg {

template <typename T>
__device__ inline int stage_level(const TailLev<T> &L, T *sc, int cap_planes) {
    if (L.kind != OP_PLANE || L.O > cap_planes) return 0;
    for (int idx = threadIdx.x; idx < L.O * 252; idx += blockDim.x) {
        const int k = idx / 252, e = idx - k * 252;
        sc[idx] = e < 243 ? L.coef[e * L.O + k] : L.dinv[(e - 243) * L.O + k];
    }
    __syncthreads();
    return 1;
}

// x at node slot p of colour sweep: x = inv(A_c)(r - sum_{off-centre} A x)
template <typename T>
__device__ inline void tail_gs_node(const TailLev<T> &L, int q, int t, const T *sc, int staged) {
    int i, j, k;
    if (!colour_node(L.g, q, t, i, j, k)) return;
    const Geom &g = L.g;
    const int p = q * g.S + t;
    T acc[3], inv[9];
    load3<T, true>(L.r, g.npad, p, acc);
    NbrOffsets nb = nbr_offsets(g, i, j, k);
    if (L.kind == OP_PLANE) {
        const T *cf = staged ? sc + 252 * k : L.coef + k;
        const int stride = staged ? 1 : L.O;
        if (L.sparse) plane_row_coef<T, true, false, true>(cf, stride, g, nb, L.x, acc);
        else plane_row_coef<T, false, false, true>(cf, stride, g, nb, L.x, acc);
#pragma unroll
        for (int e = 0; e < 9; e++) inv[e] = staged ? sc[252 * k + 243 + e] : L.dinv[e * L.O + k];
    } else {
        DenseOp<T> op{L.coef, L.dinv};
        dense_row<T, false, true>(op, g, nb, p, L.x, acc);
#pragma unroll
        for (int e = 0; e < 9; e++) inv[e] = __ldg(L.dinv + (size_t)e * g.npad + p);
    }
    L.x[p] = dot3(inv[0], acc[0], inv[1], acc[1], inv[2], acc[2]);
    L.x[p + g.npad] = dot3(inv[3], acc[0], inv[4], acc[1], inv[5], acc[2]);
    L.x[p + 2 * g.npad] = dot3(inv[6], acc[0], inv[7], acc[1], inv[8], acc[2]);
}

template <typename T>
__device__ inline void tail_residual_node(const TailLev<T> &L, int p, const T *sc, int staged) {
    const Geom &g = L.g;
    int i, j, k;
    T acc[3] = {T(0), T(0), T(0)};
    if (slot_node(g, p, i, j, k)) {
        load3<T, true>(L.r, g.npad, p, acc);
        NbrOffsets nb = nbr_offsets(g, i, j, k);
        if (L.kind == OP_PLANE) {
            const T *cf = staged ? sc + 252 * k : L.coef + k;
            const int stride = staged ? 1 : L.O;
            if (L.sparse) plane_row_coef<T, true, true, true>(cf, stride, g, nb, L.x, acc);
            else plane_row_coef<T, false, true, true>(cf, stride, g, nb, L.x, acc);
        } else {
            DenseOp<T> op{L.coef, L.dinv};
            dense_row<T, true, true>(op, g, nb, p, L.x, acc);
        }
    }
    L.res[p] = acc[0];
    L.res[p + g.npad] = acc[1];
    L.res[p + 2 * g.npad] = acc[2];
}

template <typename T>
__device__ inline void tail_sweeps(const TailLev<T> &L, int sweeps, const T *sc, int staged, int tid, int nthr,
                                   cg::cluster_group &cl) {
    for (int s = 0; s < sweeps; s++)
        for (int q = 0; q < 8; q++) {
            for (int t = tid; t < L.g.S; t += nthr) tail_gs_node(L, q, t, sc, staged);
            cl.sync();
        }
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads) tail_down_kernel(const __grid_constant__ TailDesc<T> d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sc = reinterpret_cast<T *>(smem_raw);
    cg::cluster_group cl = cg::this_cluster();
    const int nthr = (int)(cl.num_blocks() * blockDim.x);
    const int tid = (int)(cl.block_rank() * blockDim.x + threadIdx.x);
    for (int i = d.lo; i <= d.hi; i++) {
        const TailLev<T> &L = d.L[i];
        const int staged = stage_level(L, sc, d.cap_planes);
        tail_sweeps(L, d.v_down + (d.growth ? i : 0), sc, staged, tid, nthr, cl);
        for (int p = tid; p < L.g.npad; p += nthr) tail_residual_node(L, p, sc, staged);
        cl.sync();
        const TailLev<T> &C = d.L[i + 1];
        for (int p = tid; p < C.g.npad; p += nthr) {
            int I, J, K;
            T acc[3] = {T(0), T(0), T(0)};
            if (slot_node(C.g, p, I, J, K)) restrict_node<T, true>(L.g, C.g, L.res, p, I, J, K, acc);
            C.r[p] = acc[0];
            C.r[p + C.g.npad] = acc[1];
            C.r[p + 2 * C.g.npad] = acc[2];
            C.x[p] = C.x[p + C.g.npad] = C.x[p + 2 * C.g.npad] = T(0);
        }
        cl.sync();
    }
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads) tail_up_kernel(const __grid_constant__ TailDesc<T> d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sc = reinterpret_cast<T *>(smem_raw);
    cg::cluster_group cl = cg::this_cluster();
    const int nthr = (int)(cl.num_blocks() * blockDim.x);
    const int tid = (int)(cl.block_rank() * blockDim.x + threadIdx.x);
    for (int i = d.hi + 1; i > d.lo; i--) {
        const TailLev<T> &F = d.L[i - 1], &C = d.L[i];
        for (int p = tid; p < F.g.npad; p += nthr) {
            int a, b, c;
            if (!slot_node(F.g, p, a, b, c)) continue;
            T s[3], v[3];
            interp_node<T, true>(F.g, C.g, C.x, a, b, c, s);
            load3<T, true>(F.x, F.g.npad, p, v);
            F.x[p] = v[0] + s[0];
            F.x[p + F.g.npad] = v[1] + s[1];
            F.x[p + 2 * F.g.npad] = v[2] + s[2];
        }
        cl.sync();
        const int staged = stage_level(F, sc, d.cap_planes);
        tail_sweeps(F, d.v_up + (d.growth ? i - 1 : 0), sc, staged, tid, nthr, cl);
    }
}

template <typename T>
static int tail_smem_bytes(const TailDesc<T> &d) {
    return d.cap_planes * 252 * (int)sizeof(T);
}

template <typename T>
static cudaError_t launch_cluster(void (*kern)(TailDesc<T>), const TailDesc<T> &d, int cluster, cudaStream_t st) {
    const int smem = tail_smem_bytes(d);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (cluster > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster, 1, 1);
    cfg.blockDim = dim3(kTailThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, d);
}

template <typename T>
cudaError_t launch_tail_down(const TailDesc<T> &d, int cluster, cudaStream_t st) {
    return launch_cluster<T>(tail_down_kernel<T>, d, cluster, st);
}
template <typename T>
cudaError_t launch_tail_up(const TailDesc<T> &d, int cluster, cudaStream_t st) {
    return launch_cluster<T>(tail_up_kernel<T>, d, cluster, st);
}

template <typename T>
int tail_cluster_size(int smem_bytes) {
    // largest cluster (16, non-portable, else 8) that can be scheduled with
    // this block size and shared memory
    for (int c : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(c, 1, 1);
        cfg.blockDim = dim3(kTailThreads, 1, 1);
        cfg.dynamicSmemBytes = smem_bytes;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = c;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        auto kern = tail_down_kernel<T>;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) != cudaSuccess) continue;
        if (c > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) continue;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n >= 1) return c;
        cudaGetLastError();
    }
    return 0;
}

template cudaError_t launch_tail_down<float>(const TailDesc<float> &, int, cudaStream_t);
template cudaError_t launch_tail_down<double>(const TailDesc<double> &, int, cudaStream_t);
template cudaError_t launch_tail_up<float>(const TailDesc<float> &, int, cudaStream_t);
template cudaError_t launch_tail_up<double>(const TailDesc<double> &, int, cudaStream_t);
template int tail_cluster_size<float>(int);
template int tail_cluster_size<double>(int);

}  // namespace stzmg
