// Model smoothing of the migration (Migration::smoothModel, cpp/Migration.cu:
// 171-236) on the GPU: a separable Gaussian of ceil(6 sigma + 1) taps (made
// odd) with indices clamped at the edges, applied to the slowness 1/v of a
// velocity model or to the value of an anisotropy parameter; cells within
// 1e-3 of the model's minimum (the water layer) keep their value.  Same taps
// and the same summation order as the host restatement; the device fuses
// each multiply-add.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/pam.h"

namespace {

constexpr int kMaxTaps = 4097;   // sigma up to about 680 cells

__global__ void smooth_rows_kernel(const float* __restrict__ f, const float* __restrict__ taps, int ks,
                                   float* __restrict__ tmp, int nz, int nx, int parameter)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x >= nx || z >= nz) return;
    const int half = ks / 2;
    const float* row = f + (long long)z * nx;
    float acc = 0.0f;
    for (int i = -half; i <= half; i++) {
        const int xx = min(max(x + i, 0), nx - 1);
        const float v = parameter ? row[xx] : 1.0f / row[xx];
        acc = __fadd_rn(acc, __fmul_rn(taps[i + half], v));   // no contraction: the reference's rounding
    }
    tmp[(long long)z * nx + x] = acc;
}

__global__ void smooth_cols_kernel(const float* __restrict__ f, const float* __restrict__ water,
                                   const float* __restrict__ tmp, const float* __restrict__ taps, int ks,
                                   float* __restrict__ out, int nz, int nx, float wmin, int parameter)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x >= nx || z >= nz) return;
    const int half = ks / 2;
    float acc = 0.0f;
    for (int i = -half; i <= half; i++) {
        const int zz = min(max(z + i, 0), nz - 1);
        acc = __fadd_rn(acc, __fmul_rn(taps[i + half], tmp[(long long)zz * nx + x]));
    }
    const long long c = (long long)z * nx + x;
    const float s0 = parameter ? f[c] : 1.0f / f[c];
    const float v = fabsf(__fsub_rn(water[c], wmin)) < 1e-3f ? s0 : acc;   // Migration::createMask
    out[c] = parameter ? v : 1.0f / v;
}

// Laplacian post-filter of an image (src/Viewdata.py:23-41):
// g = (f[z+1] + f[z-1] - 2 f[z]) / dz^2 + (f[x+1] + f[x-1] - 2 f[x]) / dx^2
// inside, in double as the reference's numpy loop; one thread per cell.
__global__ void laplacian_kernel(const float* __restrict__ f, double* __restrict__ g, int nz, int nx, double dz2,
                                 double dx2)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x < 1 || x >= nx - 1 || z < 1 || z >= nz - 1) return;
    const long long c = (long long)z * nx + x;
    const double fc = f[c];
    const double lz = (double)f[c + nx] + (double)f[c - nx] - 2.0 * fc;
    const double lx = (double)f[c + 1] + (double)f[c - 1] - 2.0 * fc;
    g[c] = lz / dz2 + lx / dx2;
}

// The edges, in the reference's order: first and last row from their
// neighbours (every column), then first and last column (every row), then
// the sign; one thread per output cell, reading the interior value the two
// copies end at.
__global__ void laplacian_edges_kernel(const double* __restrict__ g, float* __restrict__ out, int nz, int nx)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x >= nx || z >= nz) return;
    int xs = x;
    if (nx > 2) xs = x == 0 ? 1 : (x == nx - 1 ? nx - 2 : x);
    int zs = z;
    if (nz > 2) zs = z == 0 ? 1 : (z == nz - 1 ? nz - 2 : z);
    const bool inner = xs >= 1 && xs < nx - 1 && zs >= 1 && zs < nz - 1;
    out[(long long)z * nx + x] = inner ? (float)(-g[(long long)zs * nx + xs]) : 0.0f;
}

}  // namespace

extern "C" int pam_laplacian_filter(const float* image, int nz, int nx, float dz, float dx, float* out) {
    if (!image || !out || nz < 1 || nx < 1 || !(dz > 0.0f) || !(dx > 0.0f)) return PAM_E_ARG;
    const size_t n = (size_t)nz * nx;
    float *d_f = nullptr, *d_out = nullptr;
    double* d_g = nullptr;
    int rc = PAM_OK;
    if (cudaMalloc(&d_f, n * 4) != cudaSuccess || cudaMalloc(&d_g, n * 8) != cudaSuccess ||
        cudaMalloc(&d_out, n * 4) != cudaSuccess) {
        rc = PAM_E_CUDA;
    } else if (cudaMemcpy(d_f, image, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
               cudaMemset(d_g, 0, n * 8) != cudaSuccess) {
        rc = PAM_E_CUDA;
    } else {
        const dim3 grid((nx + 255) / 256, nz);
        const double dzd = dz, dxd = dx;
        laplacian_kernel<<<grid, 256>>>(d_f, d_g, nz, nx, dzd * dzd, dxd * dxd);
        laplacian_edges_kernel<<<grid, 256>>>(d_g, d_out, nz, nx);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, d_out, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = PAM_E_CUDA;
    }
    cudaFree(d_f);
    cudaFree(d_g);
    cudaFree(d_out);
    return rc;
}

extern "C" int pam_smooth_model(float* f, int nz, int nx, float sigma, int parameter, const float* water_model) {
    if (!f || nz < 1 || nx < 1 || !(sigma > 0.0f)) return PAM_E_ARG;
    int ks = (int)std::ceil(6.0f * sigma + 1.0f);
    if (ks % 2 == 0) ks++;
    if (ks > kMaxTaps) return PAM_E_ARG;
    const size_t n = (size_t)nz * nx;
    float fmin = f[0];
    for (size_t i = 1; i < n; i++) fmin = std::min(fmin, f[i]);
    if (!parameter && !(fmin > 0.0f)) return PAM_E_ARG;   // slowness of a non-positive velocity
    const float* w = water_model ? water_model : f;
    float wmin = w[0];
    for (size_t i = 1; i < n; i++) wmin = std::min(wmin, w[i]);
    const int half = ks / 2;
    std::vector<float> k(ks);
    float tot = 0.0f;
    for (int i = 0; i < ks; i++) {
        const int x = i - half;
        k[i] = std::exp(-(float)(x * x) / (2.0f * sigma * sigma));
        tot += k[i];
    }
    for (int i = 0; i < ks; i++) k[i] /= tot;
    float *d_f = nullptr, *d_w = nullptr, *d_tmp = nullptr, *d_out = nullptr, *d_k = nullptr;
    int rc = PAM_OK;
    if (cudaMalloc(&d_f, n * 4) != cudaSuccess || cudaMalloc(&d_tmp, n * 4) != cudaSuccess ||
        cudaMalloc(&d_out, n * 4) != cudaSuccess || cudaMalloc(&d_k, (size_t)ks * 4) != cudaSuccess ||
        (water_model && cudaMalloc(&d_w, n * 4) != cudaSuccess)) {
        rc = PAM_E_CUDA;
    } else if (cudaMemcpy(d_f, f, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
               (water_model && cudaMemcpy(d_w, water_model, n * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
               cudaMemcpy(d_k, k.data(), (size_t)ks * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = PAM_E_CUDA;
    } else {
        const dim3 grid((nx + 255) / 256, nz);
        smooth_rows_kernel<<<grid, 256>>>(d_f, d_k, ks, d_tmp, nz, nx, parameter);
        smooth_cols_kernel<<<grid, 256>>>(d_f, water_model ? d_w : d_f, d_tmp, d_k, ks, d_out, nz, nx, wmin,
                                          parameter);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(f, d_out, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = PAM_E_CUDA;
    }
    cudaFree(d_f);
    cudaFree(d_w);
    cudaFree(d_tmp);
    cudaFree(d_out);
    cudaFree(d_k);
    return rc;
}
