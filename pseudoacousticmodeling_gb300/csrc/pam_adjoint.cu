// Receiver-side propagation: reverse-time migration, FWI gradients and the
// exact discrete adjoint, with checkpointed reconstruction of the source
// wavefield.
//
// A job on a batch of shots runs
//   1. a forward sweep that records the modelled data and saves the state
//      (U(t), U(t-1) and, for CPML, the memory variables) every K steps into
//      HBM, the wavefields in FP32, BF16 or FP16 with a per-shot, per-snapshot
//      scale;
//   2. a backward sweep over the segments, last first: restore the segment's
//      checkpoint, rerun its K forward steps while copying every U(t) into a
//      segment buffer, then step the receiver field back through the segment,
//      applying the imaging condition or gradient at each step.
// The forward sweep writes the steps of the last segment straight into the
// segment buffer, so that segment needs neither a checkpoint nor a
// recomputation: one recomputed forward pass costs (nt - last segment) steps,
// and a large K (a segment buffer sized to the free HBM) saves that share.
// K = 0 (or K >= nt) stores every step: one segment, no recomputation, the
// reference's "onthefly" mode (cpp/Migration.cu:359-397).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/pam.h"
#include "pam_adjgrad.cuh"
#include "pam_adjoint_kernels.cuh"
#include "pam_engine.h"

using namespace pam;

#define CU(call)                                                                                 \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return e->fail(PAM_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),    \
                           __FILE__, __LINE__);                                                  \
    } while (0)

namespace {

enum Mode { kRTM = 0, kFWIRef = 1, kExact = 2 };

size_t store_bytes(int store) { return store == PAM_STORE_F32 ? 4 : 2; }

GridDims dims(const pam_engine* e) {
    GridDims g;
    g.nz = e->nza;
    g.nx = e->nxa;
    g.P = e->P;
    g.N = e->N;
    g.stride = e->shot_stride;
    g.cerjan = e->cfg.boundary == PAM_CERJAN ? e->d_cerjan : nullptr;
    return g;
}

dim3 grid2d(int nx, int nz, int B) { return dim3((nx + 31) / 32, (nz + 7) / 8, B); }

}  // namespace

// Allocate the migration / inversion buffers for checkpoint interval K
// (already clamped to [1, nt]) and storage type `store`.
int pam_engine::ensure_adjoint(int K, int store) {
    pam_engine* e = this;
    const size_t field = (size_t)shot_stride;
    const size_t interior = (size_t)cfg.nz * cfg.nx;
    if (!adj_base_ready) {
        if (dalloc_bytes((void**)&d_ub[0], field * B * 4) || dalloc_bytes((void**)&d_ub[1], field * B * 4) ||
            dalloc_bytes((void**)&d_ilum_b, interior * 4) || dalloc_bytes((void**)&d_img, interior * 4) ||
            dalloc_bytes((void**)&d_img_ilum, interior * 4) || dalloc_bytes((void**)&d_grad, interior * 4) ||
            dalloc_bytes((void**)&d_grad_ilum, interior * 4))
            return PAM_E_CUDA;
        CU(cudaMemset(d_img, 0, interior * 4));
        CU(cudaMemset(d_img_ilum, 0, interior * 4));
        CU(cudaMemset(d_grad, 0, interior * 4));
        CU(cudaMemset(d_grad_ilum, 0, interior * 4));
        if (cfg.boundary == PAM_CPML) {
            if (dalloc_bytes((void**)&d_bpsix, (size_t)xs_stride * B * 4) ||
                dalloc_bytes((void**)&d_bzetax, (size_t)xs_stride * B * 4) ||
                dalloc_bytes((void**)&d_bxaux, (size_t)xs_stride * B * 8) ||
                dalloc_bytes((void**)&d_bpsiz, (size_t)zs_stride * B * 4) ||
                dalloc_bytes((void**)&d_bzetaz, (size_t)zs_stride * B * 4) ||
                dalloc_bytes((void**)&d_bzaux, (size_t)zs_stride * B * 8))
                return PAM_E_CUDA;
        }
        if (cfg.approximation != PAM_ACOUSTIC) {
            if (dalloc_bytes((void**)&d_mp, interior * 3 * 4)) return PAM_E_CUDA;
            CU(cudaMemset(d_mp, 0, interior * 3 * 4));
        } else {
            // G, and the partial sums of the fused adjoint + gradient pass per group of four shots
            const size_t groups = (size_t)(B + kWarpsPerBlock - 1) / kWarpsPerBlock;
            if (dalloc_bytes((void**)&d_gk, field * 4) || dalloc_bytes((void**)&d_gp, groups * field * 4) ||
                dalloc_bytes((void**)&d_ip, groups * field * 4))
                return PAM_E_CUDA;
        }
        adj_base_ready = true;
    }
    if (K != adj_K || store != adj_store) {
        // release the buffers of the previous interval / format first (cudaFree
        // waits for the work still using them)
        dfree(d_seg);
        dfree(d_ckpt);
        dfree(d_ckpt_amax);
        dfree(d_ckpt_cpml);
        dfree(d_band);
        dfree(d_band_scale);
        d_seg = nullptr;
        d_ckpt = nullptr;
        d_ckpt_amax = nullptr;
        d_ckpt_cpml = nullptr;
        d_band = nullptr;
        d_band_scale = nullptr;
        if (K == PAM_RANDOM_BOUNDARY) {
            if (!d_u3 && dalloc_bytes((void**)&d_u3, field * B * 4)) return PAM_E_CUDA;
            if (!d_kap_rbc && dalloc_bytes((void**)&d_kap_rbc, field * 4)) return PAM_E_CUDA;
            if (!d_ones) {
                if (dalloc_bytes((void**)&d_ones, (size_t)N * sizeof(float))) return PAM_E_CUDA;
                const std::vector<float> ones((size_t)N, 1.0f);
                CU(cudaMemcpy(d_ones, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice));
            }
            adj_K = K;
            adj_store = store;
            adj_nseg = 0;
            return PAM_OK;
        }
        if (K == PAM_BOUNDARY_SAVING) {
            const long long nb = band_cells(cfg.nz, cfg.nx);
            const size_t nchunk = (size_t)((nb + kBandChunk - 1) / kBandChunk);
            const size_t slots = (size_t)std::max(cfg.nt - 1, 1);
            if (dalloc_bytes(&d_band, slots * B * (size_t)nb * store_bytes(store)) ||
                dalloc_bytes((void**)&d_band_scale, slots * B * nchunk * sizeof(float)))
                return PAM_E_CUDA;
            if (!d_u3 && dalloc_bytes((void**)&d_u3, field * B * 4)) return PAM_E_CUDA;
            if (!d_ones) {
                if (dalloc_bytes((void**)&d_ones, (size_t)N * sizeof(float))) return PAM_E_CUDA;
                const std::vector<float> ones((size_t)N, 1.0f);
                CU(cudaMemcpy(d_ones, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice));
            }
            adj_K = K;
            adj_store = store;
            adj_nseg = 0;
            return PAM_OK;
        }
        const int nseg = (cfg.nt + K - 1) / K;
        if (dalloc_bytes((void**)&d_seg, field * (size_t)B * (size_t)(K + 2) * 4)) return PAM_E_CUDA;
        // the stepping kernels write the update region only: the outer rows
        // and columns of a slot (read by the stencils of the rows and columns
        // next to them) must start at zero, and only whole-field copies of
        // zero-bordered fields write them afterwards
        CU(cudaMemset(d_seg, 0, field * (size_t)B * (size_t)(K + 2) * 4));
        if (nseg > 1) {
            // checkpoints of every segment but the last (kept in the segment buffer)
            const size_t nck = (size_t)nseg - 1;
            if (dalloc_bytes(&d_ckpt, field * (size_t)B * 2 * nck * store_bytes(store)) ||
                dalloc_bytes((void**)&d_ckpt_amax, nck * 2 * B * sizeof(unsigned)))
                return PAM_E_CUDA;
            if (cfg.boundary == PAM_CPML &&
                dalloc_bytes((void**)&d_ckpt_cpml, nck * B * (2 * xs_stride + 2 * zs_stride) * 4))
                return PAM_E_CUDA;
        }
        adj_K = K;
        adj_store = store;
        adj_nseg = nseg;
    }
    return PAM_OK;
}

namespace {

// Save / restore of the forward state before step k (U(k) = cur, U(k-1) =
// prev) into checkpoint `s`.
int save_checkpoint(pam_engine* e, int s, int nshots, cudaStream_t st, const float* cur, const float* prev) {
    const long long n = e->shot_stride;
    const size_t sb = store_bytes(e->adj_store);
    unsigned* amax = e->d_ckpt_amax + (size_t)s * 2 * e->B;
    const int blocks = std::min<long long>((n + 255) / 256, 1024);
    for (int f = 0; f < 2; f++) {
        const float* src = f == 0 ? cur : prev;
        char* dst = (char*)e->d_ckpt + (((size_t)s * 2 + f) * e->B) * (size_t)n * sb;
        if (e->adj_store == PAM_STORE_F32) {
            CU(cudaMemcpyAsync(dst, src, (size_t)nshots * n * 4, cudaMemcpyDeviceToDevice, st));
        } else {
            unsigned* am = amax + (size_t)f * e->B;
            CU(cudaMemsetAsync(am, 0, nshots * sizeof(unsigned), st));
            absmax_kernel<<<dim3(blocks, nshots), 256, 0, st>>>(src, n, nshots, n, am);
            if (e->adj_store == PAM_STORE_BF16)
                pack_kernel<__nv_bfloat16><<<dim3(blocks, nshots), 256, 0, st>>>(src, (__nv_bfloat16*)dst, n, nshots,
                                                                                 n, am, 1.0f);
            else
                pack_kernel<__half><<<dim3(blocks, nshots), 256, 0, st>>>(src, (__half*)dst, n, nshots, n, am,
                                                                          16384.0f);
        }
    }
    if (e->cfg.boundary == PAM_CPML) {
        const size_t per = (size_t)2 * e->xs_stride + 2 * e->zs_stride;
        float* c = e->d_ckpt_cpml + (size_t)s * e->B * per;
        const size_t xb = (size_t)e->xs_stride * nshots * 4, zb = (size_t)e->zs_stride * nshots * 4;
        CU(cudaMemcpyAsync(c, e->d_psix, xb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(c + (size_t)e->xs_stride * e->B, e->d_zetax, xb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(c + (size_t)2 * e->xs_stride * e->B, e->d_psiz, zb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(c + (size_t)(2 * e->xs_stride + e->zs_stride) * e->B, e->d_zetaz, zb,
                           cudaMemcpyDeviceToDevice, st));
    }
    CU(cudaGetLastError());
    return PAM_OK;
}

int restore_checkpoint(pam_engine* e, int s, int nshots, cudaStream_t st, float* cur, float* prev) {
    const long long n = e->shot_stride;
    const size_t sb = store_bytes(e->adj_store);
    const unsigned* amax = e->d_ckpt_amax + (size_t)s * 2 * e->B;
    const int blocks = std::min<long long>((n + 255) / 256, 1024);
    for (int f = 0; f < 2; f++) {
        float* dst = f == 0 ? cur : prev;
        const char* src = (const char*)e->d_ckpt + (((size_t)s * 2 + f) * e->B) * (size_t)n * sb;
        if (e->adj_store == PAM_STORE_F32) {
            CU(cudaMemcpyAsync(dst, src, (size_t)nshots * n * 4, cudaMemcpyDeviceToDevice, st));
        } else if (e->adj_store == PAM_STORE_BF16) {
            unpack_kernel<__nv_bfloat16><<<dim3(blocks, nshots), 256, 0, st>>>(
                (const __nv_bfloat16*)src, dst, n, nshots, n, amax + (size_t)f * e->B, 1.0f);
        } else {
            unpack_kernel<__half><<<dim3(blocks, nshots), 256, 0, st>>>((const __half*)src, dst, n, nshots, n,
                                                                        amax + (size_t)f * e->B, 16384.0f);
        }
    }
    if (e->cfg.boundary == PAM_CPML) {
        const size_t per = (size_t)2 * e->xs_stride + 2 * e->zs_stride;
        const float* c = e->d_ckpt_cpml + (size_t)s * e->B * per;
        const size_t xb = (size_t)e->xs_stride * nshots * 4, zb = (size_t)e->zs_stride * nshots * 4;
        CU(cudaMemcpyAsync(e->d_psix, c, xb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(e->d_zetax, c + (size_t)e->xs_stride * e->B, xb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(e->d_psiz, c + (size_t)2 * e->xs_stride * e->B, zb, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(e->d_zetaz, c + (size_t)(2 * e->xs_stride + e->zs_stride) * e->B, zb,
                           cudaMemcpyDeviceToDevice, st));
    }
    CU(cudaGetLastError());
    return PAM_OK;
}

// Boundary saving: save / write back the band of a source-field buffer.
int save_band(pam_engine* e, const float* field, int slot, int nshots, cudaStream_t st) {
    const GridDims g = dims(e);
    const long long nb = band_cells(e->cfg.nz, e->cfg.nx);
    const int nchunk = (int)((nb + kBandChunk - 1) / kBandChunk);
    const size_t sb = store_bytes(e->adj_store);
    char* dst = (char*)e->d_band + (size_t)slot * e->B * (size_t)nb * sb;
    float* sc = e->d_band_scale + (size_t)slot * e->B * nchunk;
    const dim3 grid(nchunk, nshots);
    if (e->adj_store == PAM_STORE_F32)
        band_save_kernel<float><<<grid, kBandChunk, 0, st>>>(field, (float*)dst, sc, g, e->cfg.nz, e->cfg.nx, 0.0f);
    else if (e->adj_store == PAM_STORE_BF16)
        band_save_kernel<__nv_bfloat16><<<grid, kBandChunk, 0, st>>>(field, (__nv_bfloat16*)dst, sc, g, e->cfg.nz,
                                                                     e->cfg.nx, 1.0f);
    else
        band_save_kernel<__half><<<grid, kBandChunk, 0, st>>>(field, (__half*)dst, sc, g, e->cfg.nz, e->cfg.nx,
                                                              16384.0f);
    CU(cudaGetLastError());
    return PAM_OK;
}

int restore_band(pam_engine* e, float* field, int slot, int nshots, cudaStream_t st) {
    const GridDims g = dims(e);
    const long long nb = band_cells(e->cfg.nz, e->cfg.nx);
    const int nchunk = (int)((nb + kBandChunk - 1) / kBandChunk);
    const size_t sb = store_bytes(e->adj_store);
    const char* src = (const char*)e->d_band + (size_t)slot * e->B * (size_t)nb * sb;
    const float* sc = e->d_band_scale + (size_t)slot * e->B * nchunk;
    const dim3 grid(nchunk, nshots);
    if (e->adj_store == PAM_STORE_F32)
        band_restore_kernel<float><<<grid, kBandChunk, 0, st>>>((const float*)src, sc, field, g, e->cfg.nz,
                                                                e->cfg.nx, 0);
    else if (e->adj_store == PAM_STORE_BF16)
        band_restore_kernel<__nv_bfloat16><<<grid, kBandChunk, 0, st>>>((const __nv_bfloat16*)src, sc, field, g,
                                                                        e->cfg.nz, e->cfg.nx, 1);
    else
        band_restore_kernel<__half><<<grid, kBandChunk, 0, st>>>((const __half*)src, sc, field, g, e->cfg.nz,
                                                                 e->cfg.nx, 1);
    CU(cudaGetLastError());
    return PAM_OK;
}

}  // namespace

// ---- the single-pass anisotropic adjoint (reference form)

// The kernel stages its operands with 16-byte cp.async from quads that start
// at columns that are multiples of 4: every base must be 16-byte aligned and
// every row pitch and shot stride a multiple of 4 floats.  (The engine's
// fields, models and segment slots always are; a false here is a bug.)
static bool aniso_operands_aligned(const AnisoArgs& aa, const float* nxt, const float* kap) {
    auto al = [](const void* p) { return p == nullptr || ((uintptr_t)p & 15) == 0; };
    return al(aa.ub) && al(aa.pf) && al(aa.eps) && al(aa.del) && al(aa.cth) && al(aa.sth) && al(nxt) && al(kap) &&
           aa.g.P % 4 == 0 && aa.g.stride % 4 == 0 && aa.pstride % 4 == 0;
}

static cudaError_t launch_aniso_adjoint(const AnisoArgs& aa, float* nxt, const float* kap, cudaStream_t s) {
    if (!aniso_operands_aligned(aa, nxt, kap)) return cudaErrorMisalignedAddress;
    static bool configured[2][64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    const int smem = aniso_tile_smem_bytes(aa.tti);
    const dim3 grid((aa.g.nx + kAnTX - 1) / kAnTX, (aa.g.nz + kAnTZ - 1) / kAnTZ, aa.B);
    const dim3 block(32, 8);
    if (aa.tti) {
        if (dev < 0 || dev >= 64 || !configured[1][dev]) {
            cudaFuncSetAttribute(aniso_adjoint_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (dev >= 0 && dev < 64) configured[1][dev] = true;
        }
        aniso_adjoint_tile_kernel<true><<<grid, block, smem, s>>>(aa, nxt, kap);
    } else {
        if (dev < 0 || dev >= 64 || !configured[0][dev]) {
            cudaFuncSetAttribute(aniso_adjoint_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (dev >= 0 && dev < 64) configured[0][dev] = true;
        }
        aniso_adjoint_tile_kernel<false><<<grid, block, smem, s>>>(aa, nxt, kap);
    }
    return cudaSuccess;
}

// ---- the fused adjoint + gradient kernel of the exact gradient

static int adjgrad_height(const pam_engine* e, int nshots) {
    const auto it = e->adjgrad_height_by_shots.find(nshots);
    return it == e->adjgrad_height_by_shots.end() ? e->seg_height(nshots) : it->second;
}

static AdjGradArgs adjgrad_args(const pam_engine* e, int t, int nshots, const float* wcur, float* wnxt,
                                const float* U, int grad, int H) {
    AdjGradArgs ag;
    ag.s = e->step_args(t, nshots, wcur, wnxt, 0);
    ag.s.H = H;
    ag.s.nseg = (e->nza - 8 + H - 1) / H;
    ag.U = U;
    ag.gp = e->d_gp;
    ag.ip = e->d_ip;
    ag.Bp = (nshots + kWarpsPerBlock - 1) / kWarpsPerBlock * kWarpsPerBlock;
    ag.grad = grad;
    return ag;
}

static void launch_adjgrad_kernel(const pam_engine* e, const AdjGradArgs& ag, cudaStream_t s) {
    static bool configured[64] = {};
    int dev = e->device;
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        cudaFuncSetAttribute(adjgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, adjgrad_smem_bytes());
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    const long long warps = (long long)ag.Bp * ag.s.ntiles * ag.s.nseg;
    adjgrad_kernel<<<(int)(warps / kWarpsPerBlock), 32 * kWarpsPerBlock, adjgrad_smem_bytes(), s>>>(ag);
}

// Segment height of adjgrad_kernel for this batch size: the candidates are
// timed on the receiver-field and partial-sum buffers before the job resets
// them (they hold garbage afterwards).  The arithmetic per cell does not
// depend on the height, so the gradient is bitwise the same whatever wins.
int pam_engine::tune_adjgrad(int nshots, cudaStream_t s) {
    pam_engine* e = this;
    if (!autotune || adjgrad_height_by_shots.count(nshots)) return PAM_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return PAM_OK;
    static const int cand[] = {8, 16, 24, 32, 48, 64, 96, 128};
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    int best = seg_height(nshots);
    float best_ms = 1e30f;
    for (int h : cand) {
        if (h > nza - 8 && h != cand[0]) break;
        const AdjGradArgs ag = adjgrad_args(this, 1, nshots, d_ub[0], d_ub[1], d_ub[0], 1, h);
        launch_adjgrad_kernel(this, ag, s);          // warm-up
        cudaEventRecord(e0, s);
        for (int i = 0; i < 3; i++) launch_adjgrad_kernel(this, ag, s);
        cudaEventRecord(e1, s);
        cudaError_t err = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(PAM_E_CUDA, "adjoint segment tuning failed: %s", cudaGetErrorString(err));
        }
        if (ms < best_ms) { best_ms = ms; best = h; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CU(cudaGetLastError());
    adjgrad_height_by_shots[nshots] = best;
    return PAM_OK;
}

// mode: kRTM (reference imaging), kFWIRef (reference gradient), kExact (exact
// gradient of 0.5 |d - dobs|^2 with respect to vp).
int pam_engine::run_adjoint_job(int mode, int nshots, const int* sz, const int* sx, const float* dobs, int K, int store,
                                double* misfit, float* grad_vp, cudaStream_t st) {
    pam_engine* e = this;
    if (!models_set) return fail(PAM_E_STATE, "pam_set_models has not been called");
    if (nrec < 1) return fail(PAM_E_STATE, "pam_set_receivers has not been called");
    if (int rc = check_sources(nshots, sz, sx)) return rc;
    if (!dobs) return fail(PAM_E_ARG, "observed data is NULL");
    if (store < PAM_STORE_F32 || store > PAM_STORE_F16) return fail(PAM_E_ARG, "unknown checkpoint storage %d", store);
    if (mode == kExact && cfg.approximation != PAM_ACOUSTIC)
        return fail(PAM_E_UNSUPPORTED, "the exact gradient is implemented for the acoustic approximation");
    if (mode == kFWIRef && cfg.approximation != PAM_ACOUSTIC && cfg.boundary == PAM_CPML)
        return fail(PAM_E_UNSUPPORTED, "anisotropic FWI follows the reference, which has Cerjan boundaries only");
    if (mode == kRTM && cfg.approximation != PAM_ACOUSTIC && cfg.boundary == PAM_CPML)
        return fail(PAM_E_UNSUPPORTED, "anisotropic RTM follows the reference, which has Cerjan boundaries only");
    if (mode == kExact && cfg.boundary != PAM_CERJAN)
        return fail(PAM_E_UNSUPPORTED, "the exact adjoint is implemented for Cerjan boundaries");
    const bool sb = K == PAM_BOUNDARY_SAVING;
    const bool rbc = K == PAM_RANDOM_BOUNDARY;
    if (sb && mode == kExact)
        return fail(PAM_E_UNSUPPORTED, "boundary saving rebuilds the physical region only, and the exact gradient "
                                       "needs the absorbing border too: use checkpoints");
    if (rbc && mode == kExact)
        return fail(PAM_E_UNSUPPORTED, "a random boundary changes the source field, and the exact gradient is "
                                       "that of the absorbing scheme: use checkpoints");
    if (sb && (cfg.nz < 9 || cfg.nx < 9)) return fail(PAM_E_ARG, "boundary saving needs nz, nx >= 9");
    if (!sb && !rbc && (K <= 0 || K > cfg.nt)) K = cfg.nt;
    CU(cudaSetDevice(device));
    if (int rc = tune_segments(nshots, st)) return rc;
    if (int rc = ensure_adjoint(K, store)) return rc;
    if (mode == kExact)
        if (int rc = tune_adjgrad(nshots, st)) return rc;
    const int nseg = adj_nseg;
    if (rbc) {
        // the random border (random_boundary.cpp), velocities capped at 95% of the
        // leapfrog limit v dt sqrt(S (1/dx^2 + 1/dz^2)) <= 2, S = 6.50158 the largest
        // symbol of the 8th-order second derivative, slowed by sqrt(1 + 2 eps) for
        // the anisotropic operators
        double emax = 0.0;
        for (float v : h_eps) emax = std::max(emax, (double)v);
        const double S = 6.50158;
        const double inv_h2 = 1.0 / ((double)cfg.dx * cfg.dx) + 1.0 / ((double)cfg.dz * cfg.dz);
        const double vcap = 0.95 * 2.0 / ((double)cfg.dt * std::sqrt(S * inv_h2)) / std::sqrt(1.0 + 2.0 * emax);
        std::vector<float> vr((size_t)nza * nxa);
        if (pam_random_boundary(h_vp.data(), cfg.nz, cfg.nx, N, cfg.dx, cfg.dz, rbc_dvel, rbc_ratio, (float)vcap,
                                rbc_seed, vr.data()) < 0)
            return fail(PAM_E_ARG, "invalid random-boundary parameters (dvel %g, ratio %g)", rbc_dvel, rbc_ratio);
        const float dt2 = cfg.dt * cfg.dt;
        std::vector<float> kr((size_t)shot_stride, 0.0f);
        for (int z = 0; z < nza; z++)
            for (int x = 0; x < nxa; x++) {
                const float v = vr[(size_t)z * nxa + x];
                kr[(size_t)z * P + x] = (v * v) * dt2;
            }
        CU(cudaMemcpyAsync(d_kap_rbc, kr.data(), kr.size() * 4, cudaMemcpyHostToDevice, st));
        CU(cudaStreamSynchronize(st));
    }
    const size_t nseis = (size_t)nshots * nt_data * nrec;
    if (!d_seis_own || seis_own_nrec < nrec) {
        if (dalloc_bytes((void**)&d_seis_own, (size_t)B * nt_data * nrec * 4)) return PAM_E_CUDA;
        seis_own_shots = B;
        seis_own_nrec = nrec;
    }
    if (!d_obs || partial_cap < (nseis + 255) / 256) {
        if (dalloc_bytes((void**)&d_obs, (size_t)B * nt_data * nrec * 4)) return PAM_E_CUDA;
        partial_cap = ((size_t)B * nt_data * nrec + 255) / 256;
        if (dalloc_bytes((void**)&d_partial, partial_cap * sizeof(double))) return PAM_E_CUDA;
    }
    CU(cudaMemcpyAsync(d_sz, sz, nshots * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_sx, sx, nshots * sizeof(int), cudaMemcpyHostToDevice, st));
    // The observed data are first read after the forward sweep (residual, or
    // the receiver injection of migration).  From pinned memory they upload on
    // the copy stream while the sweep runs; st waits for them before that read.
    cudaPointerAttributes obs_attr{};
    const bool obs_pinned = cudaPointerGetAttributes(&obs_attr, dobs) == cudaSuccess &&
                            obs_attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    bool obs_pending = false;
    // migration with an armed mute (pam_set_mute): mute on the device after the upload
    const bool mute = mode == kRTM && mute_shots > 0;
    if (mute && mute_shots != nshots)
        return fail(PAM_E_ARG, "the mute was armed for %d shots, the migration call has %d", mute_shots, nshots);
    if (mute && mute_nrec != nrec)
        return fail(PAM_E_ARG, "the mute was armed for %d receivers, the engine has %d", mute_nrec, nrec);
    auto launch_mute = [&](cudaStream_t ms) -> int {
        constexpr int kRows = 64;
        const dim3 grid((nrec + 255) / 256, (nt_data + kRows - 1) / kRows, nshots);
        mute_kernel<<<grid, 256, 0, ms>>>(d_obs, d_mute, nshots, nt_data, nrec, mute_per_shot, cfg.dt, mute_v0,
                                          mute_shift, mute_window, kRows);
        CU(cudaGetLastError());
        mute_shots = 0;   // used up
        return PAM_OK;
    };
    if (obs_pinned) {
        if (!copy_stream) CU(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& ev : obs_events)
            if (!ev) CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CU(cudaEventRecord(obs_events[0], st));            // after earlier work on st
        CU(cudaStreamWaitEvent(copy_stream, obs_events[0], 0));
        CU(cudaMemcpyAsync(d_obs, dobs, nseis * 4, cudaMemcpyHostToDevice, copy_stream));
        if (mute)
            if (int rc = launch_mute(copy_stream)) return rc;
        CU(cudaEventRecord(obs_events[1], copy_stream));
        obs_pending = true;
    } else {
        CU(cudaMemcpyAsync(d_obs, dobs, nseis * 4, cudaMemcpyHostToDevice, st));
        if (mute)
            if (int rc = launch_mute(st)) return rc;
    }
    auto wait_obs = [&]() -> int {
        if (obs_pending) CU(cudaStreamWaitEvent(st, obs_events[1], 0));
        obs_pending = false;
        return PAM_OK;
    };

    const GridDims g = dims(this);
    GridDims gnod = g;          // receiver injection of the reference adjoint: no damping factor
    gnod.cerjan = nullptr;
    prof_reset();
    const int nzi = cfg.nz, nxi = cfg.nx;
    const size_t interior = (size_t)nzi * nxi;
    const long long field = shot_stride;
    const float inv_dxdz = 1.0f / (cfg.dx * cfg.dz);
    const int itlag = cfg.itlag, nt = cfg.nt;

    CU(cudaMemsetAsync(d_ilum_b, 0, interior * 4, st));     // the exact gradient's illumination of this call
    const bool mp = mode == kFWIRef && multiparameter && cfg.approximation != PAM_ACOUSTIC;
    if (mode == kExact) CU(cudaMemsetAsync(d_gk, 0, (size_t)field * 4, st));

    // ---- 1. forward sweep: modelled data and checkpoints
    // the exact adjoint of a given adjoint source (pam_adjoint_gradient) needs
    // no modelled data: the uploaded array is the residual itself
    const bool need_data = mode != kRTM && !(mode == kExact && adjoint_source_given);
    // an undamped step of the source field with the random border (rbc)
    auto rbc_step = [&](int k, const float* cur, const float* prev, float* nxt) {
        StepArgs a = step_args(k, nshots, cur, nxt, 1);
        a.prev = prev;
        a.kap = d_kap_rbc;
        a.cerjan = d_ones;
        launch_step(a, st, PAM_CERJAN);
    };
    if (rbc) {
        if (need_data) {
            // the modelled data come from the absorbing scheme
            if (int rc = reset_fields(nshots, st)) return rc;
            for (int k = 0; k < nt; k++) enqueue_forward_step(k, nshots, d_seis_own, st);
        }
        if (int rc = reset_fields(nshots, st)) return rc;
        for (int k = 0; k < nt; k++) rbc_step(k, d_u[k & 1], nullptr, d_u[(k + 1) & 1]);
        CU(cudaGetLastError());
    } else if (sb) {
        // every step's band of U(t), t = 0 .. nt-2; U(nt-1) and U(nt) stay in the buffers
        if (int rc = reset_fields(nshots, st)) return rc;
        if (nt >= 2)
            if (int rc = save_band(this, d_u[0], 0, nshots, st)) return rc;
        for (int k = 0; k < nt; k++) {
            enqueue_forward_step(k, nshots, need_data ? d_seis_own : nullptr, st);
            if (k + 1 <= nt - 2)
                if (int rc = save_band(this, d_u[(k + 1) & 1], k + 1, nshots, st)) return rc;
        }
        CU(cudaGetLastError());
    } else if (nseg > 1) {
        // steps before the last segment rotate through the two field buffers
        // and checkpoint every K steps; the last segment's steps write into
        // the segment buffer (slot j holds U(tl - 1 + j)), where the backward
        // sweep reads them without recomputing
        if (int rc = reset_fields(nshots, st)) return rc;
        const int tl = (nseg - 1) * K;
        auto lslot = [&](int t) { return d_seg + (size_t)(t - tl + 1) * B * field; };
        float* seis = need_data ? d_seis_own : nullptr;
        for (int k = 0; k < tl; k++) {
            if (k % K == 0)
                if (int rc = save_checkpoint(this, k / K, nshots, st, d_u[k & 1], d_u[(k + 1) & 1])) return rc;
            enqueue_forward_step(k, nshots, seis, st);
        }
        CU(cudaMemcpyAsync(lslot(tl - 1), d_u[(tl + 1) & 1], (size_t)field * nshots * 4, cudaMemcpyDeviceToDevice,
                           st));
        CU(cudaMemcpyAsync(lslot(tl), d_u[tl & 1], (size_t)field * nshots * 4, cudaMemcpyDeviceToDevice, st));
        for (int k = tl; k < nt; k++) enqueue_forward_step(k, nshots, seis, st, lslot(k), lslot(k - 1), lslot(k + 1));
        CU(cudaGetLastError());
    }

    // ---- receiver-side state
    CU(cudaMemsetAsync(d_ub[0], 0, (size_t)field * nshots * 4, st));
    CU(cudaMemsetAsync(d_ub[1], 0, (size_t)field * nshots * 4, st));
    if (cfg.boundary == PAM_CPML) {
        CU(cudaMemsetAsync(d_bpsix, 0, (size_t)xs_stride * nshots * 4, st));
        CU(cudaMemsetAsync(d_bzetax, 0, (size_t)xs_stride * nshots * 4, st));
        CU(cudaMemsetAsync(d_bxaux, 0, (size_t)xs_stride * nshots * 8, st));
        CU(cudaMemsetAsync(d_bpsiz, 0, (size_t)zs_stride * nshots * 4, st));
        CU(cudaMemsetAsync(d_bzetaz, 0, (size_t)zs_stride * nshots * 4, st));
        CU(cudaMemsetAsync(d_bzaux, 0, (size_t)zs_stride * nshots * 8, st));
    }
    int ubc = 0;   // index of the receiver field's current buffer
    bool residual_ready = false;
    double mis = 0.0;
    auto make_residual = [&]() -> int {
        // Exact: dJ/dd = dcal - dobs.  Reference: adjoint source dobs - dcal
        // (src/Inversion.py:49).  Misfit 0.5 sum r^2 either way.
        if (int rc = wait_obs()) return rc;
        const long long n = (long long)nseis;
        const int blocks = (int)((n + 255) / 256);
        residual_kernel<<<blocks, 256, 0, st>>>(d_seis_own, d_obs, d_obs, n, mode == kExact ? 1.0f : -1.0f,
                                                d_partial);
        CU(cudaGetLastError());
        std::vector<double> part(blocks);
        CU(cudaMemcpyAsync(part.data(), d_partial, blocks * sizeof(double), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        for (double v : part) mis += v;
        if (!std::isfinite(mis))
            return fail(PAM_E_NUMERIC, "non-finite misfit: the modelled data overflowed (an unstable dt or grid for "
                                       "this model, see pam_check_stability) or the observed data hold NaN/Inf");
        residual_ready = true;
        return PAM_OK;
    };
    if (need_data && (nseg > 1 || sb || rbc))
        if (int rc = make_residual()) return rc;

    const dim3 blk(32, 8);
    const dim3 gsum = grid2d(nxi, nzi, 1);     // kernels that sum the batch per cell
    const dim3 gquad = grid2d((N + nxi + 3) / 4, nzi, 1);   // ... per 16-byte quad of field columns
    const int ngroups = (nshots + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (mode == kExact) {
        CU(cudaMemsetAsync(d_gp, 0, (size_t)ngroups * field * 4, st));
        CU(cudaMemsetAsync(d_ip, 0, (size_t)ngroups * field * 4, st));
    }
    auto launch_adjgrad = [&](int t, int n, const float* wcur, float* wnxt, const float* U, int grad,
                              cudaStream_t s) {
        launch_adjgrad_kernel(this, adjgrad_args(this, t, n, wcur, wnxt, U, grad, adjgrad_height(this, n)), s);
    };

    bool aniso_misaligned = false;   // set when an anisotropic adjoint launch was refused
    // receiver side of backward step t, given the source field at t - 1, t, t + 1
    auto receiver_step = [&](int t, const float* Pm1, const float* Pt, const float* Pp1) {
        float* ucur = d_ub[ubc];
        float* uprv = d_ub[ubc ^ 1];
        const long long pstride = field;
        if (mode == kRTM) {
            // C++ loop (cpp/Migration.cu:383-390): t = nt-1 .. 0
            if (t >= itlag) {
                const long long n = (long long)nrec * nshots;
                inject_receivers_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(
                    ucur, d_obs, d_rz, d_rx, nrec, nshots, t - itlag, nt_data, rec_per_shot, inv_dxdz, gnod);
            }
            {
                cudaEvent_t pend;
                prof_begin(t, 4, st, &pend);
                imaging_sum_kernel<<<gquad, blk, 0, st>>>(ucur, Pt, d_img, d_img_ilum, g, nzi, nxi, pstride, nshots);
                if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
            }
            if (cfg.approximation == PAM_ACOUSTIC) {
                if (cfg.boundary == PAM_CPML)
                    launch_cpml(nshots, ucur, st, d_bpsix, d_bzetax, d_bxaux, d_bpsiz, d_bzetaz, d_bzaux);
                StepArgs a = step_args(t, nshots, ucur, uprv, 0);
                a.xaux = d_bxaux;
                a.zaux = d_bzaux;
                {
                    cudaEvent_t pend;
                    prof_begin(t, 3, st, &pend);
                    launch_step(a, st);
                    if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
                }
            } else {
                AnisoArgs aa;
                aa.ub = ucur;
                aa.pf = Pt;
                aa.pstride = pstride;
                aa.eps = d_eps;
                aa.del = d_del;
                aa.cth = d_cth;
                aa.sth = d_sth;
                aa.g = g;
                aa.B = nshots;
                aa.tti = cfg.approximation == PAM_TTI;
                aa.inv_dx = 1.0f / cfg.dx;
                aa.inv_dz = 1.0f / cfg.dz;
                aa.inv_dx2 = 1.0f / (cfg.dx * cfg.dx);
                aa.inv_dz2 = 1.0f / (cfg.dz * cfg.dz);
                {
                    cudaEvent_t pend;
                    prof_begin(t, 3, st, &pend);
                    if (launch_aniso_adjoint(aa, uprv, d_kap, st) != cudaSuccess) aniso_misaligned = true;
                    if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
                }
            }
            ubc ^= 1;
        } else if (mode == kFWIRef) {
            // Python loop (src/Migration.py:1030-1049): illumination over every
            // forward step, gradient for t = nt-2 .. 1
            ilum_sum_kernel<<<gsum, blk, 0, st>>>(Pt, d_grad_ilum, g, nzi, nxi, pstride, nshots);
            if (t <= nt - 2 && t >= 1) {
                if (t >= itlag) {
                    const long long n = (long long)nrec * nshots;
                    inject_receivers_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(
                        ucur, d_obs, d_rz, d_rx, nrec, nshots, t - itlag, nt_data, rec_per_shot, inv_dxdz, gnod);
                }
                {
                    cudaEvent_t pend;
                    prof_begin(t, 4, st, &pend);
                    fwi_ref_grad_sum_kernel<<<gsum, blk, 0, st>>>(ucur, Pm1, Pt, Pp1, d_grad, g, nzi, nxi, pstride,
                                                                  nshots, 1.0f / (cfg.dt * cfg.dt));
                    if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
                }
                if (mp)
                    mp_grad_kernel<<<gsum, blk, 0, st>>>(Pt, ucur, pstride, d_eps, d_del, d_cth, d_sth, d_mp,
                                                         d_mp + interior,
                                                         cfg.approximation == PAM_TTI ? d_mp + 2 * interior : nullptr,
                                                         g, nzi, nxi, nshots, 1.0f / cfg.dx, 1.0f / cfg.dz,
                                                         1.0f / (cfg.dx * cfg.dx), 1.0f / (cfg.dz * cfg.dz));
                if (cfg.approximation == PAM_ACOUSTIC) {
                    if (cfg.boundary == PAM_CPML)
                        launch_cpml(nshots, ucur, st, d_bpsix, d_bzetax, d_bxaux, d_bpsiz, d_bzetaz, d_bzaux);
                    StepArgs a = step_args(t, nshots, ucur, uprv, 0);
                    a.xaux = d_bxaux;
                    a.zaux = d_bzaux;
                    {
                        cudaEvent_t pend;
                        prof_begin(t, 3, st, &pend);
                        launch_step(a, st);
                        if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
                    }
                } else {
                    // the reference's anisotropic adjoint (cpp/Migration.cu:573-973)
                    AnisoArgs aa;
                    aa.ub = ucur;
                    aa.pf = Pt;
                    aa.pstride = pstride;
                    aa.eps = d_eps;
                    aa.del = d_del;
                    aa.cth = d_cth;
                    aa.sth = d_sth;
                    aa.g = g;
                    aa.B = nshots;
                    aa.tti = cfg.approximation == PAM_TTI;
                    aa.inv_dx = 1.0f / cfg.dx;
                    aa.inv_dz = 1.0f / cfg.dz;
                    aa.inv_dx2 = 1.0f / (cfg.dx * cfg.dx);
                    aa.inv_dz2 = 1.0f / (cfg.dz * cfg.dz);
                    {
                        cudaEvent_t pend;
                        prof_begin(t, 3, st, &pend);
                        if (launch_aniso_adjoint(aa, uprv, d_kap, st) != cudaSuccess) aniso_misaligned = true;
                        if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
                    }
                }
                ubc ^= 1;
            }
        } else {
            // exact adjoint on w = kappa D lambda: ucur = w(t+1), uprv = w(t+2);
            // the illumination of every step is kept for the preconditioned gradient
            // one fused pass: w(t) into uprv, G += w(t+1) L U(t) (t <= nt-2) and
            // ilum += U(t)^2 into the shot groups' partial sums
            {
                cudaEvent_t pend;
                prof_begin(t, 3, st, &pend);
                launch_adjgrad(t, nshots, ucur, uprv, Pt, t <= nt - 2 ? 1 : 0, st);
                if (pend) cudaEventRecordWithFlags(pend, st, prof_flags);
            }
            if (t >= itlag) {
                const long long n = (long long)nrec * nshots;
                inject_adjoint_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(
                    uprv, d_obs, d_rz, d_rx, nrec, nshots, t - itlag, nt_data, rec_per_shot, d_kap, g);
            }
            ubc ^= 1;
        }
    };

    // ---- 2. backward sweep
    if (sb || rbc) {
        // S(t-1) = 2 S(t) - S(t+1) + kappa L S(t) + w(t+1): the stepping kernel with
        // the time direction reversed and no damping, then (boundary saving) the
        // saved band of S(t-1); with the random border the whole grid reverses
        float* Sp1 = d_u[nt & 1];           // U(nt)
        float* S0 = d_u[(nt - 1) & 1];      // U(nt-1)
        float* X = d_u3;
        // the steps write only the update region: keep the rest of the third buffer zero
        CU(cudaMemsetAsync(X, 0, (size_t)field * nshots * 4, st));
        if (int rc = wait_obs()) return rc;
        for (int t = nt - 1; t >= 0; t--) {
            float* Sm1 = nullptr;
            if (t >= 1) {
                if (rbc) {
                    rbc_step(t, S0, Sp1, X);
                } else {
                    StepArgs a = step_args(t, nshots, S0, X, 1);
                    a.prev = Sp1;
                    a.cerjan = d_ones;
                    launch_step(a, st, PAM_CERJAN);
                    if (int rc = restore_band(this, X, t - 1, nshots, st)) return rc;
                }
                Sm1 = X;
            }
            receiver_step(t, Sm1 ? Sm1 : S0, S0, Sp1);
            if (Sm1) {
                X = Sp1;
                Sp1 = S0;
                S0 = Sm1;
            }
        }
        CU(cudaGetLastError());
        if (aniso_misaligned) return fail(PAM_E_CUDA, "anisotropic adjoint: operands not 16-byte aligned");
    }
    for (int s = nseg - 1; s >= 0; s--) {
        const int t0 = s * K, t1 = std::min(t0 + K, nt);
        // slot j of the segment buffer holds U(t0 - 1 + j); the steps write
        // straight into the slots (U(t-1) and U(t) read from the two before)
        auto slot = [&](int t) { return d_seg + (size_t)(t - t0 + 1) * B * field; };
        // the last segment of a checkpointed sweep is already in the slots
        const bool kept = nseg > 1 && s == nseg - 1;
        if (!kept) {
            if (nseg > 1) {
                if (int rc = restore_checkpoint(this, s, nshots, st, slot(t0), slot(t0 - 1))) return rc;
            } else {
                if (int rc = reset_fields(nshots, st)) return rc;
                CU(cudaMemcpyAsync(slot(t0 - 1), d_u[(t0 + 1) & 1], (size_t)field * nshots * 4,
                                   cudaMemcpyDeviceToDevice, st));
                CU(cudaMemcpyAsync(slot(t0), d_u[t0 & 1], (size_t)field * nshots * 4, cudaMemcpyDeviceToDevice, st));
            }
            for (int k = t0; k < t1; k++)
                enqueue_forward_step(k, nshots, (need_data && nseg == 1) ? d_seis_own : nullptr, st, slot(k),
                                     slot(k - 1), slot(k + 1));
        }
        CU(cudaGetLastError());
        if (need_data && !residual_ready)
            if (int rc = make_residual()) return rc;

        if (int rc = wait_obs()) return rc;
        for (int t = t1 - 1; t >= t0; t--) receiver_step(t, slot(t - 1), slot(t), slot(t + 1));
        CU(cudaGetLastError());
        if (aniso_misaligned) return fail(PAM_E_CUDA, "anisotropic adjoint: operands not 16-byte aligned");
    }

    // ---- 3. fold the per-shot accumulators into the totals (and never return
    // while the observed data may still be uploading from the caller's buffer)
    if (int rc = wait_obs()) return rc;
    {
        const long long n = (long long)interior;
        const int blocks = (int)((n + 255) / 256);
        // (migration images, reference-form and multiparameter gradients were
        // summed into the totals step by step)
        if (mode == kExact) {
            // the shot groups' partial sums into G (expanded grid) and this
            // call's illumination, then into the illumination pam_fwi_result returns
            const dim3 fg((nxa + 255) / 256, nza);
            adjgrad_fold_kernel<<<fg, 256, 0, st>>>(d_gp, d_ip, ngroups, field, nza, nxa, P, N, nzi, nxi, d_gk,
                                                    d_ilum_b);
            reduce_shots_kernel<<<blocks, 256, 0, st>>>(d_ilum_b, d_grad_ilum, n, 1);   // already summed
        }
        CU(cudaGetLastError());
    }
    if (mode == kExact) {
        // G = kappa dJ/dkappa on the expanded grid, summed over the batch; the
        // transpose of the edge-replicating padding folds it onto the model,
        // where kappa = (vp vp)(dt dt) is constant along each folded line, then
        // the chain rule d kappa / d vp = 2 vp dt^2
        std::vector<float> gk((size_t)field);
        CU(cudaMemcpyAsync(gk.data(), d_gk, gk.size() * 4, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        const int nz = cfg.nz, nx = cfg.nx;
        std::vector<double> acc((size_t)nz * nx, 0.0);
        for (int z = 0; z < nza; z++) {
            const int zi = std::min(std::max(z - N, 0), nz - 1);
            for (int x = 0; x < nxa; x++) {
                const int xi = std::min(std::max(x - N, 0), nx - 1);
                acc[(size_t)zi * nx + xi] += (double)gk[(size_t)z * P + x];
            }
        }
        const float dt2f = cfg.dt * cfg.dt;
        const double dt2 = (double)cfg.dt * cfg.dt;
        for (size_t i = 0; i < acc.size(); i++) {
            const float kap = (h_vp[i] * h_vp[i]) * dt2f;
            grad_vp[i] += (float)(acc[i] / (double)kap * 2.0 * (double)h_vp[i] * dt2);
        }
    }
    CU(cudaStreamSynchronize(st));
    if (misfit) *misfit += mis;
    return PAM_OK;
}

namespace {

int finish_result(pam_engine* e, const float* d_num, const float* d_den, float* out, float* ilum_out, int norm) {
    const size_t n = (size_t)e->cfg.nz * e->cfg.nx;
    std::vector<float> num(n), den(n);
    CU(cudaMemcpy(num.data(), d_num, n * 4, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(den.data(), d_den, n * 4, cudaMemcpyDeviceToHost));
    if (ilum_out) std::copy(den.begin(), den.end(), ilum_out);
    if (!out) return PAM_OK;
    if (norm == PAM_NORM_NONE) {
        std::copy(num.begin(), num.end(), out);
    } else if (norm == PAM_NORM_CPP) {
        // cpp/Migration.cu:470-484
        for (size_t i = 0; i < n; i++) out[i] = den[i] > 1e-12f ? num[i] / den[i] : 0.0f;
    } else {
        // src/Migration.py:1086
        float mx = 0.0f;
        for (size_t i = 0; i < n; i++) mx = std::max(mx, den[i]);
        for (size_t i = 0; i < n; i++) out[i] = num[i] / (den[i] + 1e-5f * mx);
    }
    return PAM_OK;
}

}  // namespace

// ---------------------------------------------------------------- C ABI

extern "C" {

#define PAM_GUARD(e)                                                                   \
    do {                                                                               \
        if (!(e)) return PAM_E_ARG;                                                    \
        if ((e)->broken) return (e)->fail(PAM_E_STATE, "engine failed to initialise"); \
        (e)->err.clear();                                                              \
    } while (0)

int pam_rtm(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs, int ckpt_interval, int store,
            void* stream) {
    PAM_GUARD(e);
    if (!sz || !sx) return e->fail(PAM_E_ARG, "null host pointer");
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    return e->run_adjoint_job(kRTM, nshots, sz, sx, dobs, ckpt_interval, store, nullptr, nullptr, s);
}

int pam_rtm_result(pam_engine* e, float* image, float* ilum, int norm) {
    PAM_GUARD(e);
    if (!e->adj_base_ready) return e->fail(PAM_E_STATE, "no migration has run");
    if (norm < PAM_NORM_NONE || norm > PAM_NORM_PY) return e->fail(PAM_E_ARG, "unknown normalisation %d", norm);
    CU(cudaSetDevice(e->device));
    CU(cudaStreamSynchronize(e->stream));
    return finish_result(e, e->d_img, e->d_img_ilum, image, ilum, norm);
}

int pam_rtm_reset(pam_engine* e) {
    PAM_GUARD(e);
    if (!e->adj_base_ready) return PAM_OK;
    const size_t n = (size_t)e->cfg.nz * e->cfg.nx * 4;
    CU(cudaSetDevice(e->device));
    CU(cudaMemset(e->d_img, 0, n));
    CU(cudaMemset(e->d_img_ilum, 0, n));
    CU(cudaMemset(e->d_grad, 0, n));
    CU(cudaMemset(e->d_grad_ilum, 0, n));
    if (e->d_mp) CU(cudaMemset(e->d_mp, 0, 3 * n));
    return PAM_OK;
}

int pam_set_mute(pam_engine* e, int nshots, const float* shot_x, const float* shot_z, int nrec, const float* rec_x,
                 const float* rec_z, int per_shot, float v0, float shift, float window) {
    PAM_GUARD(e);
    if (nshots == 0) {
        e->mute_shots = 0;
        return PAM_OK;
    }
    if (nshots < 0 || nshots > e->B) return e->fail(PAM_E_ARG, "nshots=%d outside [0, %d]", nshots, e->B);
    if (nrec < 1 || !shot_x || !shot_z || !rec_x || !rec_z) return e->fail(PAM_E_ARG, "missing mute coordinates");
    if (!(v0 > 0.0f)) return e->fail(PAM_E_ARG, "v0=%g is not a positive velocity", v0);
    const size_t R = per_shot ? (size_t)nshots * nrec : (size_t)nrec;
    const size_t need = 2 * (size_t)nshots + 2 * R;
    CU(cudaSetDevice(e->device));
    if (need > e->mute_cap) {
        if (e->d_mute) e->dfree(e->d_mute);
        e->d_mute = nullptr;
        e->mute_cap = 0;
        if (e->dalloc_bytes((void**)&e->d_mute, need * sizeof(float))) return PAM_E_CUDA;
        e->mute_cap = need;
    }
    std::vector<float> c(need);
    std::copy(shot_x, shot_x + nshots, c.begin());
    std::copy(shot_z, shot_z + nshots, c.begin() + nshots);
    std::copy(rec_x, rec_x + R, c.begin() + 2 * nshots);
    std::copy(rec_z, rec_z + R, c.begin() + 2 * nshots + R);
    CU(cudaDeviceSynchronize());   // an earlier migration may still read the old coordinates
    CU(cudaMemcpy(e->d_mute, c.data(), need * sizeof(float), cudaMemcpyHostToDevice));
    e->mute_shots = nshots;
    e->mute_nrec = nrec;
    e->mute_per_shot = per_shot ? 1 : 0;
    e->mute_v0 = v0;
    e->mute_shift = shift;
    e->mute_window = window;
    return PAM_OK;
}

int pam_set_multiparameter(pam_engine* e, int enable) {
    PAM_GUARD(e);
    e->multiparameter = enable != 0;
    return PAM_OK;
}

int pam_fwi_multiparameter_result(pam_engine* e, float* g_eps, float* g_delta, float* g_theta) {
    PAM_GUARD(e);
    if (e->cfg.approximation == PAM_ACOUSTIC) return e->fail(PAM_E_UNSUPPORTED, "no anisotropy parameters");
    if (!e->adj_base_ready || !e->d_mp) return e->fail(PAM_E_STATE, "no gradient has run");
    const size_t n = (size_t)e->cfg.nz * e->cfg.nx;
    CU(cudaSetDevice(e->device));
    CU(cudaStreamSynchronize(e->stream));
    if (g_eps) CU(cudaMemcpy(g_eps, e->d_mp, n * 4, cudaMemcpyDeviceToHost));
    if (g_delta) CU(cudaMemcpy(g_delta, e->d_mp + n, n * 4, cudaMemcpyDeviceToHost));
    if (g_theta && e->cfg.approximation == PAM_TTI) CU(cudaMemcpy(g_theta, e->d_mp + 2 * n, n * 4, cudaMemcpyDeviceToHost));
    return PAM_OK;
}

int pam_fwi_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs, int ckpt_interval,
                     int store, double* misfit, void* stream) {
    PAM_GUARD(e);
    if (!sz || !sx) return e->fail(PAM_E_ARG, "null host pointer");
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    return e->run_adjoint_job(kFWIRef, nshots, sz, sx, dobs, ckpt_interval, store, misfit, nullptr, s);
}

int pam_fwi_result(pam_engine* e, float* grad, float* ilum) {
    PAM_GUARD(e);
    if (!e->adj_base_ready) return e->fail(PAM_E_STATE, "no gradient has run");
    CU(cudaSetDevice(e->device));
    CU(cudaStreamSynchronize(e->stream));
    return finish_result(e, e->d_grad, e->d_grad_ilum, grad, ilum, PAM_NORM_NONE);
}

int pam_plan_checkpoints(const pam_engine* e, long long budget_bytes, int store, int* ckpt_interval,
                         int* recomputed) {
    if (!e || !ckpt_interval || store < PAM_STORE_F32 || store > PAM_STORE_F16) return PAM_E_ARG;
    const long long nt = e->cfg.nt;
    const long long slot = (long long)e->shot_stride * e->B * 4;
    const long long ck = (long long)e->shot_stride * e->B * 2 * (long long)store_bytes(store);
    // fewer segments recompute fewer steps ((nseg - 1) K of them): the first
    // segment count whose buffers fit wins
    for (long long nseg = 1; nseg <= nt; nseg++) {
        const long long K = (nt + nseg - 1) / nseg;
        const long long real = (nt + K - 1) / K;   // segments K actually makes
        if (real != nseg) continue;
        const long long bytes = (K + 2) * slot + (real - 1) * ck;
        if (bytes <= budget_bytes) {
            *ckpt_interval = real == 1 ? 0 : (int)K;
            if (recomputed) *recomputed = (int)((real - 1) * K);
            return PAM_OK;
        }
    }
    return PAM_E_ARG;
}

int pam_misfit_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs, int ckpt_interval,
                        int store, double* misfit, float* grad_vp, void* stream) {
    PAM_GUARD(e);
    if (!sz || !sx || !grad_vp) return e->fail(PAM_E_ARG, "null host pointer");
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    return e->run_adjoint_job(kExact, nshots, sz, sx, dobs, ckpt_interval, store, misfit, grad_vp, s);
}

int pam_adjoint_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* adjoint_source,
                         int ckpt_interval, int store, float* grad_vp, void* stream) {
    PAM_GUARD(e);
    if (!sz || !sx || !grad_vp) return e->fail(PAM_E_ARG, "null host pointer");
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    double unused = 0.0;
    e->adjoint_source_given = true;
    const int rc = e->run_adjoint_job(kExact, nshots, sz, sx, adjoint_source, ckpt_interval, store, &unused, grad_vp, s);
    e->adjoint_source_given = false;
    return rc;
}

}  // extern "C"
