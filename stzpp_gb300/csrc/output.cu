// File output in the reference's formats, with the values made on the device.
//
//  * z-slices of the solver's fields (region::output_x, output_r,
//    output_residual, mg_3d_template/region.cc:3062-3120), written in the
//    format of region::output_internal (region.cc:3135-3202): a float row
//    {m, x_0 .. x_{m-1}}, then per row j {y_j, m values}.  For vec3 fields the
//    reference converts each value through vec3::operator double (the squared
//    magnitude, src/vec3.hh:110-112): output_x and output_r write
//    float(|v|^2), output_residual float(|r|^2 * |r|^2).
//  * cubes of the simulation's Field members (shear_sim_3d::output_cube,
//    src/shear_sim_3d.cpp:1961-2158): for every x, the (y, z) plane with z
//    fastest, appended as floats to <dir>/<prefix>_grid.<frame>; the
//    node-based members (u, v, w, xi) include the top z node.
//
// Only the device-to-host copy of the finished float array crosses the bus
// (4 bytes per value instead of the Field's 224).
#include <sys/stat.h>
#include <sys/types.h>

#include <cstdio>
#include <string>
#include <vector>

#include "launch.h"
#include "stz_mg.h"

namespace stzmg {

namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }

// vec3::operator double: x*x + y*y + z*z
__device__ __forceinline__ double sq3(double x, double y, double z) { return ad(ad(ml(x, x), ml(y, y)), ml(z, z)); }

__global__ void slice_kernel(Geom g, const double *__restrict__ f, int k, int quartic, float *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= g.m) return;
    const int s = slot(g, i, j, k);
    const size_t np = (size_t)g.npad;
    const double a = sq3(f[s], f[s + np], f[s + 2 * np]);
    out[i + (size_t)g.m * j] = __double2float_rn(quartic ? ml(a, a) : a);
}

constexpr int kG = 2;   // ghost layers of the simulation grid

__global__ void cube_kernel(stz_cube_fields f, int nx, int ny, int nz, int mode, int zsize, float *__restrict__ out) {
    const long n = (long)nx * ny * zsize;
    const long sy = nx + 2 * kG, sz = sy * (ny + 2 * kG);
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int zz = (int)(t % zsize), yy = (int)((t / zsize) % ny), xx = (int)(t / ((long)zsize * ny));
        const long p = (xx + kG) + sy * (yy + kG) + sz * (zz + kG);
        double v = 0;
        switch (mode) {   // Field::fval (src/field.hh:157-177)
            case 0: v = f.u[p]; break;
            case 1: v = f.v[p]; break;
            case 2: v = f.w[p]; break;
            case 3: v = f.s11[p]; break;
            case 4: v = f.s12[p]; break;
            case 5: v = f.s13[p]; break;
            case 6: v = f.s22[p]; break;
            case 7: v = f.s23[p]; break;
            case 8: v = f.s33[p]; break;
            case 9:
            case 10: {
                // pressure: -(s11+s22+s33)*(1/3.); dev: sqrt(0.5*(t11^2+t22^2+t33^2) + s12^2 + s13^2 + s23^2)
                const double s11 = f.s11[p], s22 = f.s22[p], s33 = f.s33[p];
                const double pr = ml(-ad(ad(s11, s22), s33), 1 / 3.);
                if (mode == 9) {
                    v = pr;
                } else {
                    const double t11 = ad(s11, pr), t22 = ad(s22, pr), t33 = ad(s33, pr);
                    const double s12 = f.s12[p], s13 = f.s13[p], s23 = f.s23[p];
                    double q = ml(0.5, sq3(t11, t22, t33));
                    q = ad(ad(ad(q, ml(s12, s12)), ml(s13, s13)), ml(s23, s23));
                    v = __dsqrt_rn(q);
                }
                break;
            }
            case 11: v = f.chi[p]; break;
            case 12: v = ml(f.chi[p], 21000.); break;
            case 13: v = f.xi_x[p]; break;
            case 14: v = f.xi_y[p]; break;
            default: v = f.xi_z[p]; break;
        }
        out[t] = __double2float_rn(v);
    }
}

bool node_based(int mode) { return mode <= 2 || mode >= 13; }

}  // namespace

void launch_slice(const Geom &g, const double *f, int k, bool quartic, float *out, cudaStream_t st) {
    slice_kernel<<<dim3((g.m + 127) / 128, g.n), 128, 0, st>>>(g, f, k, quartic ? 1 : 0, out);
}

// The body of region::output_internal for one process (mp = np = 1).
bool write_slice_file(const float *vals, int m, int n, double ax, double bx, double ay, double by,
                      const char *filename) {
    FILE *fp = std::fopen(filename, "wb");
    if (!fp) return false;
    const double dx = (bx - ax) / (m - 1), dy = (by - ay) / (n - 1);
    std::vector<float> head(m + 1);
    head[0] = (float)m;
    for (int i = 0; i < m; i++) head[i + 1] = (float)(ax + dx * i);
    bool ok = std::fwrite(head.data(), sizeof(float), m + 1, fp) == (size_t)m + 1;
    for (int j = 0; ok && j < n; j++) {
        const float y = (float)(ay + dy * j);
        ok = std::fwrite(&y, sizeof(float), 1, fp) == 1 &&
             std::fwrite(vals + (size_t)m * j, sizeof(float), m, fp) == (size_t)m;
    }
    return std::fclose(fp) == 0 && ok;
}

}  // namespace stzmg

using namespace stzmg;

extern "C" int stz_mg_cube_values(const stz_cube_fields *f, int nx, int ny, int nz, int mode, float *out,
                                  void *stream) {
    if (!f || !out || nx < 1 || ny < 1 || nz < 1 || mode < 0 || mode > 15) return STZ_MG_ERR_ARG;
    const double *need = mode <= 2    ? (mode == 0 ? f->u : mode == 1 ? f->v : f->w)
                         : mode <= 10 ? f->s11
                         : mode <= 12 ? f->chi
                                      : (mode == 13 ? f->xi_x : mode == 14 ? f->xi_y : f->xi_z);
    if (!need) return STZ_MG_ERR_ARG;
    if (mode >= 3 && mode <= 10 && (!f->s12 || !f->s13 || !f->s22 || !f->s23 || !f->s33)) return STZ_MG_ERR_ARG;
    const int zsize = node_based(mode) ? nz + 1 : nz;
    const long n = (long)nx * ny * zsize;
    const int blocks = (int)std::min<long>((n + 255) / 256, 152L * 16);
    cube_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(*f, nx, ny, nz, mode, zsize, out);
    return cudaGetLastError() == cudaSuccess ? STZ_MG_OK : STZ_MG_ERR_CUDA;
}

extern "C" int stz_mg_output_cube(const stz_cube_fields *f, int nx, int ny, int nz, int mode, const char *dir,
                                  const char *prefix, int frame) {
    if (!dir || !prefix) return STZ_MG_ERR_ARG;
    const int zsize = (mode <= 2 || mode >= 13) ? nz + 1 : nz;
    const size_t n = (size_t)nx * ny * zsize;
    float *d = nullptr;
    if (cudaMalloc(&d, n * sizeof(float)) != cudaSuccess) return STZ_MG_ERR_OOM;
    std::vector<float> h(n);
    int rc = stz_mg_cube_values(f, nx, ny, nz, mode, d, nullptr);
    if (rc == STZ_MG_OK &&
        (cudaMemcpy(h.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = STZ_MG_ERR_CUDA;
    cudaFree(d);
    if (rc != STZ_MG_OK) return rc;
    mkdir(dir, 0700);   // as the reference: create the folder if it does not exist
    const std::string path = std::string(dir) + "/" + prefix + "_grid." + std::to_string(frame);
    FILE *fp = std::fopen(path.c_str(), "a");
    if (!fp) return STZ_MG_ERR_ARG;
    const bool ok = std::fwrite(h.data(), sizeof(float), n, fp) == n;
    return (std::fclose(fp) == 0 && ok) ? STZ_MG_OK : STZ_MG_ERR_ARG;
}
