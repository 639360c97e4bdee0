// Test infrastructure: runs the reference's own CUDA kernels.
//
// The reference's forward-modelling kernels (cpp/Modeling.cu:481-749:
// injectSource, updateWaveEquation{,VTI,TTI}, storeSeismogram) are compiled
// unmodified from the reference sources into a cubin by oracle/build.py
// (output in oracle/_ref/, never committed).  This file is the host side,
// written for this repository: it loads that cubin with the CUDA driver API
// and repeats the reference's shot loop (cpp/Modeling.cu:433-479) - reset the
// fields, then per time step injectSource on `current`, the update kernel
// (future from current, with the reference's in-place Cerjan damping),
// storeSeismogram of `current` once k >= itlag, and the buffer swap - with
// the launch shapes of cpp/Modeling.cu:43-44 (256 threads, one per cell).
//
// Host preparation (padding, radians, wavelet, Cerjan vector) is done by the
// caller with the oracle's restatements of cpp/Modeling.cu:84-182; only the
// device code and the loop come from the reference.  Used only by the tests,
// as a checker.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace {

char g_err[512] = "";

int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof g_err, "%s: %s", what, s ? s : "unknown CUDA error");
    return -1;
}

#define DRV(call)                                  \
    do {                                           \
        CUresult _r = (call);                      \
        if (_r != CUDA_SUCCESS) return fail(#call, _r); \
    } while (0)

struct Buffers {
    std::vector<CUdeviceptr> ptrs;
    ~Buffers() {
        for (CUdeviceptr p : ptrs) cuMemFree(p);
    }
    CUresult alloc(CUdeviceptr* p, size_t bytes) {
        CUresult r = cuMemAlloc(p, bytes < 4 ? 4 : bytes);
        if (r == CUDA_SUCCESS) ptrs.push_back(*p);
        return r;
    }
};

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err; }

// approx: 0 acoustic, 1 VTI, 2 TTI.  nz, nx: expanded grid.  Models are the
// expanded [nz][nx] arrays (theta in radians), A the Cerjan vector [N],
// source the wavelet [nt].  Shots run one after another; seis receives
// [nshots][nt - itlag][nrec].  gpu_ms: device time of the shot loops.
int ref_forward(const char* cubin, int approx, int nz, int nx, int N, float dz, float dx, float dt, int nt, int itlag,
                const float* vp, const float* eps, const float* del, const float* theta, const float* A,
                const float* source, int nshots, const int* sz, const int* sx, int nrec, const int* rz, const int* rx,
                float* seis, double* gpu_ms) {
    if (!cubin || !vp || !A || !source || !sz || !sx || !rz || !rx || !seis || nz < 9 || nx < 9 || nt < 1 ||
        itlag < 0 || itlag >= nt || nshots < 1 || nrec < 1 || approx < 0 || approx > 2 ||
        (approx >= 1 && (!eps || !del)) || (approx == 2 && !theta)) {
        std::snprintf(g_err, sizeof g_err, "invalid arguments");
        return -1;
    }
    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
    DRV(cuCtxPushCurrent(ctx));
    struct Pop {
        CUdevice d;
        ~Pop() {
            CUcontext c;
            cuCtxPopCurrent(&c);
            cuDevicePrimaryCtxRelease(d);
        }
    } pop{dev};

    CUmodule mod;
    DRV(cuModuleLoad(&mod, cubin));
    struct Unload {
        CUmodule m;
        ~Unload() { cuModuleUnload(m); }
    } unload{mod};
    // mangled names of the reference's kernels (cpp/Modeling.cuh:59-63)
    CUfunction f_inject, f_store, f_update;
    DRV(cuModuleGetFunction(&f_inject, mod, "_Z12injectSourcePfPKfiiiii"));
    DRV(cuModuleGetFunction(&f_store, mod, "_Z15storeSeismogramPKfPfPKiS3_iiii"));
    const char* upd = approx == 0 ? "_Z18updateWaveEquationPfS_PKfiifffS_i"
                    : approx == 1 ? "_Z21updateWaveEquationVTIPfS_iifffPKfS1_S1_S_i"
                                  : "_Z21updateWaveEquationTTIPfS_iifffPKfS1_S1_S1_S_i";
    DRV(cuModuleGetFunction(&f_update, mod, upd));

    const size_t ncell = (size_t)nz * nx;
    const int nt_data = nt - itlag;
    const size_t nseis = (size_t)nt_data * nrec;
    Buffers buf;
    CUdeviceptr d_vp, d_eps = 0, d_del = 0, d_th = 0, d_A, d_src, d_cur, d_fut, d_seis, d_rx, d_rz;
    DRV(buf.alloc(&d_vp, ncell * 4));
    DRV(buf.alloc(&d_A, (size_t)N * 4));
    DRV(buf.alloc(&d_src, (size_t)nt * 4));
    DRV(buf.alloc(&d_cur, ncell * 4));
    DRV(buf.alloc(&d_fut, ncell * 4));
    DRV(buf.alloc(&d_seis, nseis * 4));
    DRV(buf.alloc(&d_rx, (size_t)nrec * 4));
    DRV(buf.alloc(&d_rz, (size_t)nrec * 4));
    DRV(cuMemcpyHtoD(d_vp, vp, ncell * 4));
    DRV(cuMemcpyHtoD(d_A, A, (size_t)N * 4));
    DRV(cuMemcpyHtoD(d_src, source, (size_t)nt * 4));
    DRV(cuMemcpyHtoD(d_rx, rx, (size_t)nrec * 4));
    DRV(cuMemcpyHtoD(d_rz, rz, (size_t)nrec * 4));
    if (approx >= 1) {
        DRV(buf.alloc(&d_eps, ncell * 4));
        DRV(buf.alloc(&d_del, ncell * 4));
        DRV(cuMemcpyHtoD(d_eps, eps, ncell * 4));
        DRV(cuMemcpyHtoD(d_del, del, ncell * 4));
    }
    if (approx == 2) {
        DRV(buf.alloc(&d_th, ncell * 4));
        DRV(cuMemcpyHtoD(d_th, theta, ncell * 4));
    }

    for (int r = 0; r < nrec; r++)
        if (rz[r] < 0 || rz[r] >= nz || rx[r] < 0 || rx[r] >= nx) {
            std::snprintf(g_err, sizeof g_err, "receiver %d outside the grid", r);
            return -1;
        }
    CUstream st;
    DRV(cuStreamCreate(&st, CU_STREAM_DEFAULT));
    struct StreamGuard {
        CUstream s;
        ~StreamGuard() { cuStreamDestroy(s); }
    } sguard{st};
    CUevent e0, e1;
    DRV(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    DRV(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    struct EventGuard {
        CUevent a, b;
        ~EventGuard() {
            cuEventDestroy(a);
            cuEventDestroy(b);
        }
    } eguard{e0, e1};

    const unsigned expBlocks = (unsigned)((ncell + 255) / 256);
    const unsigned seisBlocks = (unsigned)((nrec + 255) / 256);
    double total_ms = 0.0;
    for (int shot = 0; shot < nshots; shot++) {
        int isx = sx[shot], isz = sz[shot];
        if (isx < 0 || isx >= nx || isz < 0 || isz >= nz) {
            std::snprintf(g_err, sizeof g_err, "source %d outside the grid", shot);
            return -1;
        }
        DRV(cuMemsetD32Async(d_cur, 0, ncell, st));
        DRV(cuMemsetD32Async(d_fut, 0, ncell, st));
        DRV(cuMemsetD32Async(d_seis, 0, nseis, st));
        DRV(cuEventRecord(e0, st));
        CUdeviceptr cur = d_cur, fut = d_fut;
        int N_abc = N, nzv = nz, nxv = nx, ntv = nt, itl = itlag, nr = nrec;
        float dzv = dz, dxv = dx, dtv = dt;
        for (int k = 0; k < nt; k++) {
            {
                void* p[] = {&cur, &d_src, &k, &ntv, &nxv, &isx, &isz};
                DRV(cuLaunchKernel(f_inject, 1, 1, 1, 1, 1, 1, 0, st, p, nullptr));
            }
            if (approx == 0) {
                void* p[] = {&fut, &cur, &d_vp, &nzv, &nxv, &dzv, &dxv, &dtv, &d_A, &N_abc};
                DRV(cuLaunchKernel(f_update, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            } else if (approx == 1) {
                void* p[] = {&fut, &cur, &nxv, &nzv, &dtv, &dxv, &dzv, &d_vp, &d_eps, &d_del, &d_A, &N_abc};
                DRV(cuLaunchKernel(f_update, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            } else {
                void* p[] = {&fut, &cur, &nxv, &nzv, &dtv, &dxv, &dzv, &d_vp, &d_eps, &d_del, &d_th, &d_A, &N_abc};
                DRV(cuLaunchKernel(f_update, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            }
            if (k >= itlag) {
                void* p[] = {&cur, &d_seis, &d_rx, &d_rz, &k, &itl, &nr, &nxv};
                DRV(cuLaunchKernel(f_store, seisBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            }
            std::swap(cur, fut);
        }
        DRV(cuEventRecord(e1, st));
        DRV(cuStreamSynchronize(st));
        float ms = 0.0f;
        DRV(cuEventElapsedTime(&ms, e0, e1));
        total_ms += ms;
        DRV(cuMemcpyDtoH(seis + (size_t)shot * nseis, d_seis, nseis * 4));
    }
    if (gpu_ms) *gpu_ms = total_ms;
    return 0;
}

}  // extern "C"
