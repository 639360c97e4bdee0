// Test infrastructure: runs the reference's own CUDA kernels (forward
// modelling, and the on-the-fly migration further below).
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

// The reference's on-the-fly migration (Migration::solveReverseTimeMigrationOntheFly,
// cpp/Migration.cu:359-397) with its own kernels: cubin_mod holds
// cpp/Modeling.cu's, cubin_mig cpp/Migration.cu's.  Per shot the forward loop
// above, saving `current` after each update (the reference copies it on a
// second stream while the next step already runs; here the copy is ordered
// after the update on the same stream, so the saved field is the one the
// reference means to save), then for t = nt-1 .. 0: injectAdjointSource of the
// observed sample t - itlag (t >= itlag), backward_step(t, saved U(t))
// (cpp/Migration.cu:238-250: the acoustic adjoint kernel, or the anisotropic
// products kernel then its update kernel, each with the imaging sums), and the
// buffer swap.  Image and illumination [nz - 2N][nx - 2N] accumulate over the
// shots; normalize != 0 applies normalizeImage (cpp/Migration.cu:470-484)
// at the end.  obs: [nshots][nt - itlag][nrec].
int ref_rtm(const char* cubin_mod, const char* cubin_mig, int approx, int nz, int nx, int N, float dz, float dx,
            float dt, int nt, int itlag, const float* vp, const float* eps, const float* del, const float* theta,
            const float* A, const float* source, int nshots, const int* sz, const int* sx, int nrec, const int* rz,
            const int* rx, const float* obs, int normalize, float* image, float* ilum, double* gpu_ms) {
    if (!cubin_mod || !cubin_mig || !vp || !A || !source || !sz || !sx || !rz || !rx || !obs || !image || !ilum ||
        nz < 2 * N + 1 || nx < 2 * N + 1 || N < 4 || nt < 1 || itlag < 0 || itlag >= nt || nshots < 1 || nrec < 1 ||
        approx < 0 || approx > 2 || (approx >= 1 && (!eps || !del)) || (approx == 2 && !theta)) {
        std::snprintf(g_err, sizeof g_err, "invalid arguments");
        return -1;
    }
    for (int r = 0; r < nrec; r++)
        if (rz[r] < 0 || rz[r] >= nz || rx[r] < 0 || rx[r] >= nx) {
            std::snprintf(g_err, sizeof g_err, "receiver %d outside the grid", r);
            return -1;
        }
    for (int s = 0; s < nshots; s++)
        if (sx[s] < 0 || sx[s] >= nx || sz[s] < 0 || sz[s] >= nz) {
            std::snprintf(g_err, sizeof g_err, "source %d outside the grid", s);
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
    CUmodule mod, mig;
    DRV(cuModuleLoad(&mod, cubin_mod));
    struct Unload {
        CUmodule m;
        ~Unload() { cuModuleUnload(m); }
    } unload_mod{mod};
    DRV(cuModuleLoad(&mig, cubin_mig));
    Unload unload_mig{mig};
    // mangled names of the reference's kernels (cpp/Modeling.cuh:59-63, cpp/Migration.cuh:68-75)
    CUfunction f_inject, f_update, f_adj_src, f_adj, f_prod = nullptr, f_norm;
    DRV(cuModuleGetFunction(&f_inject, mod, "_Z12injectSourcePfPKfiiiii"));
    DRV(cuModuleGetFunction(&f_update, mod,
                            approx == 0   ? "_Z18updateWaveEquationPfS_PKfiifffS_i"
                            : approx == 1 ? "_Z21updateWaveEquationVTIPfS_iifffPKfS1_S1_S_i"
                                          : "_Z21updateWaveEquationTTIPfS_iifffPKfS1_S1_S1_S_i"));
    DRV(cuModuleGetFunction(&f_adj_src, mig, "_Z19injectAdjointSourcePfPKfPKiS3_iiiff"));
    DRV(cuModuleGetFunction(&f_norm, mig, "_Z14normalizeImagePfPKfii"));
    if (approx == 0) {
        DRV(cuModuleGetFunction(&f_adj, mig, "_Z25updateAdjointWaveEquationPfS_S_S_S_PKfiifffS_i"));
    } else if (approx == 1) {
        DRV(cuModuleGetFunction(&f_prod, mig, "_Z27calculateAdjointVTIProductsPKfS0_PfS1_S1_S1_iiffS0_S0_"));
        DRV(cuModuleGetFunction(&f_adj, mig, "_Z28updateAdjointWaveEquationVTIPfS_S_S_S_S_S_S_S_iifffPKfS_i"));
    } else {
        DRV(cuModuleGetFunction(&f_prod, mig, "_Z27calculateAdjointTTIProductsPKfS0_PfS1_S1_S1_S1_iiffS0_S0_S0_"));
        DRV(cuModuleGetFunction(&f_adj, mig, "_Z28updateAdjointWaveEquationTTIPfS_S_S_S_PKfS1_S1_S1_S1_iifffS1_S_i"));
    }

    const size_t ncell = (size_t)nz * nx;
    const int nzi = nz - 2 * N, nxi = nx - 2 * N;
    const size_t nimg = (size_t)nzi * nxi;
    const int nt_data = nt - itlag;
    const size_t nseis = (size_t)nt_data * nrec;
    Buffers buf;
    CUdeviceptr d_vp, d_eps = 0, d_del = 0, d_th = 0, d_A, d_src, d_cur, d_fut, d_curb, d_futb, d_save, d_seis, d_rx,
        d_rz, d_img, d_ilum, d_AU = 0, d_BU = 0, d_HU = 0, d_QX = 0, d_QZ = 0;
    DRV(buf.alloc(&d_vp, ncell * 4));
    DRV(buf.alloc(&d_A, (size_t)N * 4));
    DRV(buf.alloc(&d_src, (size_t)nt * 4));
    DRV(buf.alloc(&d_cur, ncell * 4));
    DRV(buf.alloc(&d_fut, ncell * 4));
    DRV(buf.alloc(&d_curb, ncell * 4));
    DRV(buf.alloc(&d_futb, ncell * 4));
    DRV(buf.alloc(&d_save, ncell * 4 * (size_t)nt));
    DRV(buf.alloc(&d_seis, nseis * 4));
    DRV(buf.alloc(&d_rx, (size_t)nrec * 4));
    DRV(buf.alloc(&d_rz, (size_t)nrec * 4));
    DRV(buf.alloc(&d_img, nimg * 4));
    DRV(buf.alloc(&d_ilum, nimg * 4));
    DRV(cuMemcpyHtoD(d_vp, vp, ncell * 4));
    DRV(cuMemcpyHtoD(d_A, A, (size_t)N * 4));
    DRV(cuMemcpyHtoD(d_src, source, (size_t)nt * 4));
    DRV(cuMemcpyHtoD(d_rx, rx, (size_t)nrec * 4));
    DRV(cuMemcpyHtoD(d_rz, rz, (size_t)nrec * 4));
    DRV(cuMemsetD32(d_img, 0, nimg));
    DRV(cuMemsetD32(d_ilum, 0, nimg));
    if (approx >= 1) {
        DRV(buf.alloc(&d_eps, ncell * 4));
        DRV(buf.alloc(&d_del, ncell * 4));
        DRV(cuMemcpyHtoD(d_eps, eps, ncell * 4));
        DRV(cuMemcpyHtoD(d_del, del, ncell * 4));
        DRV(buf.alloc(&d_AU, ncell * 4));
        DRV(buf.alloc(&d_BU, ncell * 4));
        DRV(buf.alloc(&d_QX, ncell * 4));
        DRV(buf.alloc(&d_QZ, ncell * 4));
    }
    if (approx == 2) {
        DRV(buf.alloc(&d_th, ncell * 4));
        DRV(cuMemcpyHtoD(d_th, theta, ncell * 4));
        DRV(buf.alloc(&d_HU, ncell * 4));
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
    const unsigned nBlocks = (unsigned)((nimg + 255) / 256);
    int N_abc = N, nzv = nz, nxv = nx, ntv = nt, nr = nrec;
    float dzv = dz, dxv = dx, dtv = dt;
    double total_ms = 0.0;
    for (int shot = 0; shot < nshots; shot++) {
        int isx = sx[shot], isz = sz[shot];
        DRV(cuMemsetD32Async(d_cur, 0, ncell, st));
        DRV(cuMemsetD32Async(d_fut, 0, ncell, st));
        DRV(cuMemsetD32Async(d_curb, 0, ncell, st));
        DRV(cuMemsetD32Async(d_futb, 0, ncell, st));
        DRV(cuMemcpyHtoDAsync(d_seis, obs + (size_t)shot * nseis, nseis * 4, st));
        DRV(cuEventRecord(e0, st));
        CUdeviceptr cur = d_cur, fut = d_fut;
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
            DRV(cuMemcpyDtoDAsync(d_save + (size_t)k * ncell * 4, cur, ncell * 4, st));
            std::swap(cur, fut);
        }
        CUdeviceptr curb = d_curb, futb = d_futb;
        for (int t = nt - 1; t >= 0; t--) {
            if (t >= itlag) {
                int it = t - itlag;
                void* p[] = {&curb, &d_seis, &d_rx, &d_rz, &it, &nr, &nxv, &dxv, &dzv};
                DRV(cuLaunchKernel(f_adj_src, seisBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            }
            CUdeviceptr P = d_save + (size_t)t * ncell * 4;
            if (approx == 0) {
                void* p[] = {&futb, &curb, &P, &d_img, &d_ilum, &d_vp, &nzv, &nxv, &dzv, &dxv, &dtv, &d_A, &N_abc};
                DRV(cuLaunchKernel(f_adj, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            } else if (approx == 1) {
                void* pp[] = {&curb, &P, &d_AU, &d_BU, &d_QX, &d_QZ, &nxv, &nzv, &dxv, &dzv, &d_eps, &d_del};
                DRV(cuLaunchKernel(f_prod, expBlocks, 1, 1, 256, 1, 1, 0, st, pp, nullptr));
                void* p[] = {&futb, &curb, &P, &d_img, &d_ilum, &d_AU, &d_BU, &d_QX, &d_QZ,
                             &nxv,  &nzv,  &dtv, &dxv,  &dzv,    &d_vp, &d_A,  &N_abc};
                DRV(cuLaunchKernel(f_adj, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            } else {
                void* pp[] = {&curb, &P, &d_AU, &d_BU, &d_HU, &d_QX, &d_QZ, &nxv, &nzv, &dxv, &dzv, &d_eps, &d_del,
                              &d_th};
                DRV(cuLaunchKernel(f_prod, expBlocks, 1, 1, 256, 1, 1, 0, st, pp, nullptr));
                void* p[] = {&futb, &curb, &P,   &d_img, &d_ilum, &d_AU, &d_BU, &d_HU, &d_QX,
                             &d_QZ, &nxv,  &nzv, &dtv,   &dxv,    &dzv,  &d_vp, &d_A,  &N_abc};
                DRV(cuLaunchKernel(f_adj, expBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
            }
            std::swap(curb, futb);
        }
        DRV(cuEventRecord(e1, st));
        DRV(cuStreamSynchronize(st));
        float ms = 0.0f;
        DRV(cuEventElapsedTime(&ms, e0, e1));
        total_ms += ms;
    }
    if (normalize) {
        int nxi_v = nxi, nzi_v = nzi;
        void* p[] = {&d_img, &d_ilum, &nxi_v, &nzi_v};
        DRV(cuLaunchKernel(f_norm, nBlocks, 1, 1, 256, 1, 1, 0, st, p, nullptr));
    }
    DRV(cuStreamSynchronize(st));
    DRV(cuMemcpyDtoH(image, d_img, nimg * 4));
    DRV(cuMemcpyDtoH(ilum, d_ilum, nimg * 4));
    if (gpu_ms) *gpu_ms = total_ms;
    return 0;
}

}  // extern "C"
