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
        acc += taps[i + half] * v;
    }
    tmp[(long long)z * nx + x] = acc;
}

__global__ void smooth_cols_kernel(const float* __restrict__ f, const float* __restrict__ tmp,
                                   const float* __restrict__ taps, int ks, float* __restrict__ out, int nz, int nx,
                                   float fmin, int parameter)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x >= nx || z >= nz) return;
    const int half = ks / 2;
    float acc = 0.0f;
    for (int i = -half; i <= half; i++) {
        const int zz = min(max(z + i, 0), nz - 1);
        acc += taps[i + half] * tmp[(long long)zz * nx + x];
    }
    const long long c = (long long)z * nx + x;
    const float s0 = parameter ? f[c] : 1.0f / f[c];
    const float v = fabsf(f[c] - fmin) < 1e-3f ? s0 : acc;
    out[c] = parameter ? v : 1.0f / v;
}

}  // namespace

extern "C" int pam_smooth_model(float* f, int nz, int nx, float sigma, int parameter) {
    if (!f || nz < 1 || nx < 1 || !(sigma > 0.0f)) return PAM_E_ARG;
    int ks = (int)std::ceil(6.0f * sigma + 1.0f);
    if (ks % 2 == 0) ks++;
    if (ks > kMaxTaps) return PAM_E_ARG;
    const size_t n = (size_t)nz * nx;
    float fmin = f[0];
    for (size_t i = 1; i < n; i++) fmin = std::min(fmin, f[i]);
    if (!parameter && !(fmin > 0.0f)) return PAM_E_ARG;   // slowness of a non-positive velocity
    const int half = ks / 2;
    std::vector<float> k(ks);
    float tot = 0.0f;
    for (int i = 0; i < ks; i++) {
        const int x = i - half;
        k[i] = std::exp(-(float)(x * x) / (2.0f * sigma * sigma));
        tot += k[i];
    }
    for (int i = 0; i < ks; i++) k[i] /= tot;
    float *d_f = nullptr, *d_tmp = nullptr, *d_out = nullptr, *d_k = nullptr;
    int rc = PAM_OK;
    if (cudaMalloc(&d_f, n * 4) != cudaSuccess || cudaMalloc(&d_tmp, n * 4) != cudaSuccess ||
        cudaMalloc(&d_out, n * 4) != cudaSuccess || cudaMalloc(&d_k, (size_t)ks * 4) != cudaSuccess) {
        rc = PAM_E_CUDA;
    } else if (cudaMemcpy(d_f, f, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
               cudaMemcpy(d_k, k.data(), (size_t)ks * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = PAM_E_CUDA;
    } else {
        const dim3 grid((nx + 255) / 256, nz);
        smooth_rows_kernel<<<grid, 256>>>(d_f, d_k, ks, d_tmp, nz, nx, parameter);
        smooth_cols_kernel<<<grid, 256>>>(d_f, d_tmp, d_k, ks, d_out, nz, nx, fmin, parameter);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(f, d_out, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = PAM_E_CUDA;
    }
    cudaFree(d_f);
    cudaFree(d_tmp);
    cudaFree(d_out);
    cudaFree(d_k);
    return rc;
}
