// L2 misfit of device-resident seismograms without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need a
// misfit: code running inside a memory budget that was fixed up front (a
// serving process with a pre-sized pool, a solver loop that must not touch
// the allocator between iterations, a job sharing the GPU under a hard
// per-process cap), where one more cudaMalloc would fail or fragment the
// pool.  pam_misfit_noalloc serves them: it computes the same quantity as the
// residual/misfit reduction inside the gradient jobs, but keeps its
// per-block partial sums in a fixed array that lives in this library's device
// image, so a call only launches kernels and copies eight bytes back.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/pam.h"
#include "pam_check.cuh"

namespace {

// Largest number of per-block partial sums one call can use: 65,536 doubles,
// 512 KiB of device memory held by every GPU that loads this library, for as
// long as the process runs.  With 2,048 samples reduced per block this bounds
// a call to PAM_MISFIT_NOALLOC_MAX_SAMPLES samples.
constexpr int kPartials = 65536;
constexpr int kThreads = 256;
constexpr int kPerThread = 8;
static_assert((long long)kPartials * kThreads * kPerThread == PAM_MISFIT_NOALLOC_MAX_SAMPLES,
              "limit in pam.h must match the scratch size");

// Slots [0, kPartials) hold block partials, slot kPartials the final sum.
static __device__ __align__(256) double g_misfit_scratch[kPartials + 1];

// Stage 1: block b writes sum over its 2,048 samples of 0.5 (dcal - dobs)^2 to
// scratch[b].  Every slot that stage 2 reads is written here first, so the
// contents a previous call left behind are never read.
__global__ void misfit_partials_kernel(const float* __restrict__ dcal, const float* __restrict__ dobs, long long n,
                                       double* __restrict__ scratch)
{
    __shared__ double red[kThreads];
    const long long base = (long long)blockIdx.x * kThreads * kPerThread + threadIdx.x;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < kPerThread; k++) {
        const long long i = base + (long long)k * kThreads;
        if (i < n) {
            const float r = *PAM_CHK(&dcal[i], dcal, n * 4, 4, 60) - *PAM_CHK(&dobs[i], dobs, n * 4, 4, 61);
            acc += 0.5 * (double)r * (double)r;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *PAM_CHK(&scratch[blockIdx.x], scratch, (kPartials + 1) * 8, 8, 62) = red[0];
}

// Stage 2: one block adds the `nb` partials in a fixed order and writes the
// total to scratch[kPartials].
__global__ void misfit_total_kernel(double* __restrict__ scratch, int nb)
{
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) acc += *PAM_CHK(&scratch[i], scratch, (kPartials + 1) * 8, 8, 63);
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *PAM_CHK(&scratch[kPartials], scratch, (kPartials + 1) * 8, 8, 64) = red[0];
}

// Device address of g_misfit_scratch, looked up once per device with that
// device current (the host-side symbol is only a stand-in, not an address a
// kernel may use).
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int scratch_for_current_device(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PAM_E_CUDA;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_misfit_scratch);
        if (rc != cudaSuccess || !p) return PAM_E_CUDA;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return PAM_OK;
}

}  // namespace

extern "C" int pam_misfit_noalloc(const float* d_dcal, const float* d_dobs, long long n, double* misfit, void* stream)
{
    if (!d_dcal || !d_dobs || !misfit) return PAM_E_ARG;
    if (n < 1 || n > PAM_MISFIT_NOALLOC_MAX_SAMPLES) {
        fprintf(stderr,
                "pam_misfit_noalloc: %lld samples requested; this entry point reduces at most %lld samples per call "
                "(its fixed scratch holds %d partial sums) - split the data or use the gradient entry points\n",
                n, (long long)PAM_MISFIT_NOALLOC_MAX_SAMPLES, kPartials);
        return PAM_E_ARG;
    }
    double* scratch = nullptr;
    if (int rc = scratch_for_current_device(&scratch)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nb = (int)((n + (long long)kThreads * kPerThread - 1) / ((long long)kThreads * kPerThread));
    misfit_partials_kernel<<<nb, kThreads, 0, s>>>(d_dcal, d_dobs, n, scratch);
    misfit_total_kernel<<<1, kThreads, 0, s>>>(scratch, nb);
    if (cudaGetLastError() != cudaSuccess) return PAM_E_CUDA;
    if (cudaMemcpyAsync(misfit, scratch + kPartials, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return PAM_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PAM_E_CUDA;
    return PAM_OK;
}
