// Host side of the engine: device buffers, model preparation, the time loop
// (captured into a CUDA graph), and the C ABI declared in include/pam.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pam.h"
#include "pam_engine.h"
#include "pam_kernels.cuh"
#include "stability.hpp"

using namespace pam;

// ---------------------------------------------------------------- errors

int pam_engine::fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
}

#define CU(call)                                                                                 \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return e->fail(PAM_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),    \
                           __FILE__, __LINE__);                                                  \
    } while (0)

namespace {

const float kPi = 3.14159265358979323846f;

template <typename T>
int dalloc(pam_engine* e, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) return PAM_OK;
    cudaError_t s = cudaMalloc((void**)p, n * sizeof(T));
    if (s != cudaSuccess)
        return e->fail(PAM_E_CUDA, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(s));
    e->allocs.push_back((void*)*p);
    e->bytes_allocated += n * sizeof(T);
    return PAM_OK;
}

// Edge-replicating padding of Modeling::expandModel (cpp/Modeling.cu:130-182)
// straight into the pitched device layout [nz_a][P] (padding columns zero).
std::vector<float> expand_pitched(const float* m, int nz, int nx, int N, int P) {
    const int nza = nz + 2 * N, nxa = nx + 2 * N;
    std::vector<float> out((size_t)nza * P, 0.0f);
    for (int z = 0; z < nza; z++) {
        const int zi = std::min(std::max(z - N, 0), nz - 1);
        for (int x = 0; x < nxa; x++) {
            const int xi = std::min(std::max(x - N, 0), nx - 1);
            out[(size_t)z * P + x] = m[(size_t)zi * nx + xi];
        }
    }
    return out;
}

}  // namespace

void pam_engine::dfree(void* p) {
    if (!p) return;
    for (size_t i = 0; i < allocs.size(); i++)
        if (allocs[i] == p) {
            cudaFree(p);
            allocs.erase(allocs.begin() + (long)i);
            return;
        }
}

int pam_engine::dalloc_bytes(void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return PAM_OK;
    cudaError_t s = cudaMalloc(p, bytes);
    if (s != cudaSuccess) return fail(PAM_E_CUDA, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(s));
    allocs.push_back(*p);
    bytes_allocated += bytes;
    return PAM_OK;
}

pam_engine::~pam_engine() {
    for (GraphSet& gs : graph_sets) drop_graphs(gs);
    for (cudaEvent_t ev : chunk_events) cudaEventDestroy(ev);
    for (cudaEvent_t ev : strip_events)
        if (ev) cudaEventDestroy(ev);
    if (strip_stream) cudaStreamDestroy(strip_stream);
    for (cudaEvent_t ev : obs_events)
        if (ev) cudaEventDestroy(ev);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (auto& p : prof) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    if (cap_stream) cudaStreamDestroy(cap_stream);
    for (void* p : allocs) cudaFree(p);
    for (void* p : host_allocs) cudaFreeHost(p);
    if (own_stream) cudaStreamDestroy(own_stream);
}

// ---------------------------------------------------------------- setup

int pam_engine::init(const pam_config& c, int dev) {
    pam_engine* e = this;
    cfg = c;
    device = dev;
    if (c.nz < 1 || c.nx < 1 || c.n_abc < 8 || c.nt < 1 || c.itlag < 0 || c.itlag >= c.nt || c.max_shots < 1)
        return fail(PAM_E_ARG, "invalid config: nz=%d nx=%d n_abc=%d nt=%d itlag=%d max_shots=%d (n_abc must be >= 8)",
                    c.nz, c.nx, c.n_abc, c.nt, c.itlag, c.max_shots);
    if (!(c.dx > 0 && c.dz > 0 && c.dt > 0))
        return fail(PAM_E_ARG, "invalid spacing dx=%g dz=%g dt=%g", c.dx, c.dz, c.dt);
    if (c.approximation < PAM_ACOUSTIC || c.approximation > PAM_TTI)
        return fail(PAM_E_ARG, "unknown approximation %d", c.approximation);
    if (c.boundary != PAM_CERJAN && c.boundary != PAM_CPML)
        return fail(PAM_E_ARG, "unknown boundary %d", c.boundary);
    N = c.n_abc;
    nza = c.nz + 2 * N;
    nxa = c.nx + 2 * N;
    if (N - 4 > kCpmlMaxStrip) return fail(PAM_E_ARG, "n_abc=%d exceeds the supported %d", N, kCpmlMaxStrip + 4);
    if (2 * N > nxa - 8 || 2 * N > nza - 8) return fail(PAM_E_ARG, "absorbing layers overlap");
    nt_data = c.nt - c.itlag;
    if (c.approximation == PAM_TTI) {
        // 120 written columns per tile starting at column 4, loads from column 0
        ntiles = (nxa - 8 + kTileOut - 1) / kTileOut;
        P = ((ntiles * kTileOut + 8) + 31) / 32 * 32;
    } else {
        // 128-aligned tiles covering columns [0, nxa - 4), plus the right halo quad
        ntiles = (nxa - 4 + kTileWide - 1) / kTileWide;
        P = ((ntiles * kTileWide + 4) + 31) / 32 * 32;
    }
    H = 64;
    nseg = (nza - 8 + H - 1) / H;
    B = c.max_shots;

    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
    if (c.boundary == PAM_CPML) {
        CU(cudaStreamCreateWithFlags(&strip_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& ev : strip_events) CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }

    const size_t field = (size_t)nza * P;
    shot_stride = (long long)field;
    if (dalloc(this, &d_kap, field)) return PAM_E_CUDA;
    if (c.approximation != PAM_ACOUSTIC) {
        if (dalloc(this, &d_eps, field) || dalloc(this, &d_del, field) || dalloc(this, &d_e2, field) ||
            dalloc(this, &d_m1, field) || dalloc(this, &d_m2, field))
            return PAM_E_CUDA;
    }
    if (c.approximation == PAM_TTI) {
        if (dalloc(this, &d_cth, field) || dalloc(this, &d_sth, field)) return PAM_E_CUDA;
    }
    if (dalloc(this, &d_u[0], field * B) || dalloc(this, &d_u[1], field * B)) return PAM_E_CUDA;
    if (c.boundary == PAM_CERJAN) {
        if (dalloc(this, &d_cerjan, (size_t)N)) return PAM_E_CUDA;
        // Cerjan factors, float arithmetic of Modeling::createCerjanVector (cpp/Modeling.cu:111-120)
        std::vector<float> A(N);
        const float sb = 3.0f * N;
        for (int i = 0; i < N; i++) {
            const float fb = (N - i) / (1.4142f * sb);
            A[i] = std::exp(-fb * fb);
        }
        h_cerjan = A;
        CU(cudaMemcpy(d_cerjan, A.data(), N * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        xs_stride = (long long)nza * 2 * N;
        zs_stride = (long long)2 * N * P;
        if (dalloc(this, &d_psix, (size_t)xs_stride * B) || dalloc(this, &d_zetax, (size_t)xs_stride * B) ||
            dalloc(this, &d_xaux, (size_t)xs_stride * B) || dalloc(this, &d_psiz, (size_t)zs_stride * B) ||
            dalloc(this, &d_zetaz, (size_t)zs_stride * B) || dalloc(this, &d_zaux, (size_t)zs_stride * B) ||
            dalloc(this, &d_cxab, (size_t)xs_stride) || dalloc(this, &d_czab, (size_t)zs_stride))
            return PAM_E_CUDA;
    }
    if (dalloc(this, &d_sz, (size_t)B) || dalloc(this, &d_sx, (size_t)B) || dalloc(this, &d_status, (size_t)1))
        return PAM_E_CUDA;
    CU(cudaMemset(d_status, 0, sizeof(int)));

    // Ricker wavelet, float arithmetic of Modeling::createWavelet (cpp/Modeling.cu:84-100)
    wavelet.assign(c.nt, 0.0f);
    const float tlag = 2.0f * std::sqrt(kPi) / c.fcut;
    const float scale = 1.0f / (c.dx * c.dz);
    const float fc = c.fcut / (3.0f * std::sqrt(kPi));
    for (int n = 0; n < c.nt; n++) {
        const float td = n * c.dt - tlag;
        const float arg = kPi * kPi * kPi * fc * fc * td * td;
        wavelet[n] = (1.0f - 2.0f * arg) * std::exp(-arg) * scale;
    }
    if (dalloc(this, &d_wavelet, (size_t)c.nt)) return PAM_E_CUDA;
    CU(cudaMemcpy(d_wavelet, wavelet.data(), (size_t)c.nt * sizeof(float), cudaMemcpyHostToDevice));
    return PAM_OK;
}

int pam_engine::set_models(const float* vp, const float* eps, const float* del, const float* theta_deg) {
    pam_engine* e = this;
    if (!vp) return fail(PAM_E_ARG, "vp is required");
    const int nz = cfg.nz, nx = cfg.nx;
    const size_t n = (size_t)nz * nx;
    for (size_t i = 0; i < n; i++)
        if (!(vp[i] > 0.0f) || !std::isfinite(vp[i])) return fail(PAM_E_ARG, "vp[%zu]=%g is not a positive finite velocity", i, vp[i]);
    const bool aniso = cfg.approximation != PAM_ACOUSTIC;
    if (aniso && (!eps || !del)) return fail(PAM_E_ARG, "epsilon and delta are required for VTI/TTI");
    if (cfg.approximation == PAM_TTI && !theta_deg) return fail(PAM_E_ARG, "theta is required for TTI");
    CU(cudaSetDevice(device));

    h_vp.assign(vp, vp + n);
    // kappa = (vp*vp)*(dt*dt), the product order of cpp/Modeling.cu:519,533
    std::vector<float> ex = expand_pitched(vp, nz, nx, N, P);
    const float dt2 = cfg.dt * cfg.dt;
    std::vector<float> kap(ex.size(), 0.0f);
    for (int z = 0; z < nza; z++)
        for (int x = 0; x < nxa; x++) {
            const size_t i = (size_t)z * P + x;
            kap[i] = (ex[i] * ex[i]) * dt2;
        }
    // the engine's streams are non-blocking, so the synchronous copies below
    // would not wait for a modelling call still running on one of them
    CU(cudaDeviceSynchronize());
    CU(cudaMemcpy(d_kap, kap.data(), kap.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (aniso) {
        h_eps.assign(eps, eps + n);
        h_del.assign(del, del + n);
        const std::vector<float> ea = expand_pitched(eps, nz, nx, N, P);
        const std::vector<float> da = expand_pitched(del, nz, nx, N, P);
        CU(cudaMemcpy(d_eps, ea.data(), ea.size() * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_del, da.data(), da.size() * sizeof(float), cudaMemcpyHostToDevice));
        // the per-cell coefficients of the VTI/TTI update, each rounded as the
        // reference's expressions round them (cpp/Modeling.cu:605-613):
        // 1.0f + 2.0f*eps, -2.0f*(eps - delta), 2.0f*(1.0f + delta)
        std::vector<float> e2(ea.size()), m1(ea.size()), m2(ea.size());
        for (size_t i = 0; i < ea.size(); i++) {
            e2[i] = 1.0f + 2.0f * ea[i];
            m1[i] = -2.0f * (ea[i] - da[i]);
            m2[i] = 2.0f * (1.0f + da[i]);
        }
        CU(cudaMemcpy(d_e2, e2.data(), e2.size() * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_m1, m1.data(), m1.size() * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_m2, m2.data(), m2.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (cfg.approximation == PAM_TTI) {
        std::vector<float> th(n);
        for (size_t i = 0; i < n; i++) th[i] = theta_deg[i] * kPi / 180.0f;   // cpp/Modeling.cu:364-367
        h_theta.assign(th.begin(), th.end());
        std::vector<float> a = expand_pitched(th.data(), nz, nx, N, P);
        std::vector<float> c(a.size(), 0.0f), s(a.size(), 0.0f);
        for (int z = 0; z < nza; z++)
            for (int x = 0; x < nxa; x++) {
                const size_t i = (size_t)z * P + x;
                c[i] = (float)std::cos((double)a[i]);
                s[i] = (float)std::sin((double)a[i]);
            }
        CU(cudaMemcpy(d_cth, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_sth, s.data(), s.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (cfg.boundary == PAM_CPML) {
        // CPML profiles of src/utils.py:198-240 with d0 = -3 ln R,
        // R = 1e-3^(N/10), f_pico = fcut/3 (src/Modeling2D.py:110-126), in double.
        const double R = N < 200 ? std::pow(1e-3, N / 10.0) : std::pow(1e-3, 15.0);
        const double d0 = -3.0 * std::log(R);
        const double fp = cfg.fcut / 3.0;
        const double dt = cfg.dt;
        auto prof = [&](int i, int n, double h, double v, float2* out) {
            double pts = 0.0;
            bool in = false;
            if (i < N) { pts = (N - i - 1.0) * h; in = true; }
            else if (i >= n - N) { pts = (i - n + N) * h; in = true; }
            double d = 0.0, al = 0.0;
            if (in) {
                const double rr = pts / (N * h);
                d = d0 / (2.0 * N * h) * rr * rr * v;
                al = M_PI * fp * (1.0 - rr * rr);
            }
            const double a = std::exp(-(d + al) * dt);
            const double b = std::fabs(d + al) > 1e-10 ? d / (d + al) * (a - 1.0) : 0.0;
            *out = make_float2((float)a, (float)b);
        };
        std::vector<float2> cx((size_t)xs_stride), cz((size_t)zs_stride, make_float2(1.f, 0.f));
        for (int z = 0; z < nza; z++)
            for (int c2 = 0; c2 < 2 * N; c2++) {
                const int x = c2 < N ? c2 : nxa - 2 * N + c2;
                prof(x, nxa, cfg.dx, ex[(size_t)z * P + x], &cx[(size_t)z * 2 * N + c2]);
            }
        for (int r2 = 0; r2 < 2 * N; r2++) {
            const int z = r2 < N ? r2 : nza - 2 * N + r2;
            for (int x = 0; x < nxa; x++) prof(z, nza, cfg.dz, ex[(size_t)z * P + x], &cz[(size_t)r2 * P + x]);
        }
        CU(cudaMemcpy(d_cxab, cx.data(), cx.size() * sizeof(float2), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_czab, cz.data(), cz.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    models_set = true;
    return PAM_OK;
}

int pam_engine::set_receivers(int n, const int* rz, const int* rx, int per_shot) {
    pam_engine* e = this;
    if (n < 1 || !rz || !rx) return fail(PAM_E_ARG, "receiver list is empty");
    const size_t cnt = (size_t)n * (per_shot ? B : 1);
    for (size_t i = 0; i < cnt; i++)
        if (rz[i] < 0 || rz[i] >= nza || rx[i] < 0 || rx[i] >= nxa)
            return fail(PAM_E_ARG, "receiver %zu at (%d,%d) lies outside the %dx%d expanded grid", i, rz[i], rx[i], nza, nxa);
    CU(cudaSetDevice(device));
    if (cnt > rec_cap) {
        if (dalloc(this, &d_rz, cnt) || dalloc(this, &d_rx, cnt)) return PAM_E_CUDA;
        rec_cap = cnt;
    }
    CU(cudaMemcpy(d_rz, rz, cnt * sizeof(int), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(d_rx, rx, cnt * sizeof(int), cudaMemcpyHostToDevice));
    nrec = n;
    rec_per_shot = per_shot ? 1 : 0;
    invalidate_graph();
    return PAM_OK;
}

int pam_engine::check_sources(int nshots, const int* sz, const int* sx) {
    if (nshots < 1 || nshots > B) return fail(PAM_E_ARG, "nshots=%d outside [1, %d]", nshots, B);
    for (int i = 0; i < nshots; i++)
        if (sz[i] < 4 || sz[i] >= nza - 4 || sx[i] < 4 || sx[i] >= nxa - 4)
            return fail(PAM_E_ARG, "source %d at (%d,%d) lies outside the update region of the %dx%d grid", i, sz[i],
                        sx[i], nza, nxa);
    return PAM_OK;
}

void pam_engine::invalidate_graph() {
    for (GraphSet& gs : graph_sets) drop_graphs(gs);
}

void pam_engine::drop_graphs(GraphSet& gs) {
    for (cudaGraphExec_t g : gs.execs) cudaGraphExecDestroy(g);
    gs.execs.clear();
    gs.bounds.clear();
    gs.shots = -1;
    gs.seis = nullptr;
}

// ---------------------------------------------------------------- stepping

StepArgs pam_engine::step_args(int k, int nshots, const float* cur, float* nxt, int fwd_src) const {
    StepArgs a;
    a.cur = cur;
    a.nxt = nxt;
    a.prev = nullptr;
    a.kap = d_kap;
    a.eps = d_eps;
    a.del = d_del;
    a.e2 = d_e2;
    a.m1 = d_m1;
    a.m2 = d_m2;
    a.cth = d_cth;
    a.sth = d_sth;
    a.cerjan = d_cerjan;
    a.xaux = d_xaux;
    a.zaux = d_zaux;
    a.src_z = d_sz;
    a.src_x = d_sx;
    a.src_amp = (fwd_src && k + 1 < cfg.nt) ? wavelet[k + 1] : 0.0f;
    a.nz = nza;
    a.nx = nxa;
    a.P = P;
    a.N = N;
    a.shot_stride = shot_stride;
    a.xaux_stride = xs_stride;
    a.zaux_stride = zs_stride;
    a.B = nshots;
    a.ntiles = ntiles;
    a.H = seg_height(nshots);
    a.nseg = (nza - 8 + a.H - 1) / a.H;
    a.inv_dx = 1.0f / cfg.dx;
    a.inv_dz = 1.0f / cfg.dz;
    a.inv_dx2 = 1.0f / (cfg.dx * cfg.dx);
    a.inv_dz2 = 1.0f / (cfg.dz * cfg.dz);
    const float A[4] = {0.8f, -0.2f, 0.03809523809f, -0.00357142857f};
    for (int i = 0; i < 4; i++) { a.cx1[i] = A[i] * a.inv_dx; a.cz1[i] = A[i] * a.inv_dz; }
    return a;
}

int pam_engine::seg_height(int nshots) const {
    const auto it = seg_height_by_shots.find(nshots);
    return it == seg_height_by_shots.end() ? H : it->second;
}

// Autotuner of the stepping kernel's tile height: each candidate segment
// height (rows a warp marches) is launched on the live field buffers and timed
// with events; the fastest is kept for this batch size.  Short segments give
// more warps and shorter dependency chains (small batches), long ones less
// halo re-reading (large batches).  The arithmetic per cell does not depend on
// the height, so results are bitwise identical whatever is chosen.  The
// buffers hold garbage afterwards: callers tune before resetting the fields.
// Skipped (default height) while the stream is being captured into a graph.
int pam_engine::tune_segments(int nshots, cudaStream_t s) {
    pam_engine* e = this;
    if (!autotune || seg_height_by_shots.count(nshots)) return PAM_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return PAM_OK;
    static const int cand[] = {8, 16, 24, 32, 48, 64, 96, 128};
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    int best = H;
    float best_ms = 1e30f;
    for (int h : cand) {
        if (h > nza - 8 && h != cand[0]) break;
        StepArgs a = step_args(1, nshots, d_u[0], d_u[1], 0);
        a.H = h;
        a.nseg = (nza - 8 + h - 1) / h;
        launch_step(a, s);                       // warm-up
        cudaEventRecord(e0, s);
        for (int i = 0; i < 3; i++) launch_step(a, s);
        cudaEventRecord(e1, s);
        cudaError_t err = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(PAM_E_CUDA, "segment tuning failed: %s", cudaGetErrorString(err));
        }
        if (ms < best_ms) { best_ms = ms; best = h; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CU(cudaGetLastError());
    seg_height_by_shots[nshots] = best;
    return PAM_OK;
}

constexpr int kMaxDevices = 64;

template <int A, int BC>
static void launch_step_t(const StepArgs& a, cudaStream_t s) {
    const long long warps = (long long)a.B * a.ntiles * a.nseg;
    const int blocks = (int)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock);
    constexpr int smem = step_smem_bytes<A>();
    // the shared-memory opt-in is a per-device attribute of the kernel
    static bool configured[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices || !configured[dev]) {
        cudaFuncSetAttribute(step_kernel<A, BC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (dev >= 0 && dev < kMaxDevices) configured[dev] = true;
    }
    step_kernel<A, BC><<<blocks, 32 * kWarpsPerBlock, smem, s>>>(a);
}

void pam_engine::launch_step(const StepArgs& a, cudaStream_t s, int boundary) const {
    const int A = cfg.approximation, BC = boundary >= 0 ? boundary : cfg.boundary;
    if (A == PAM_ACOUSTIC && BC == PAM_CERJAN) launch_step_t<kAcoustic, kCerjan>(a, s);
    else if (A == PAM_ACOUSTIC) launch_step_t<kAcoustic, kCPML>(a, s);
    else if (A == PAM_VTI && BC == PAM_CERJAN) launch_step_t<kVTI, kCerjan>(a, s);
    else if (A == PAM_VTI) launch_step_t<kVTI, kCPML>(a, s);
    else if (BC == PAM_CERJAN) launch_step_t<kTTI, kCerjan>(a, s);
    else launch_step_t<kTTI, kCPML>(a, s);
}

void pam_engine::launch_cpml(int nshots, const float* cur, cudaStream_t s, float* psix, float* zetax, float2* xaux,
                             float* psiz, float* zetaz, float2* zaux) const {
    CpmlArgs c;
    c.cur = cur;
    c.psix = psix;
    c.zetax = zetax;
    c.xaux = xaux;
    c.psiz = psiz;
    c.zetaz = zetaz;
    c.zaux = zaux;
    c.cxab = d_cxab;
    c.czab = d_czab;
    c.nz = nza;
    c.nx = nxa;
    c.P = P;
    c.N = N;
    c.B = nshots;
    c.shot_stride = shot_stride;
    c.xs_stride = xs_stride;
    c.zs_stride = zs_stride;
    c.inv_dx = 1.0f / cfg.dx;
    c.inv_dz = 1.0f / cfg.dz;
    c.inv_dx2 = 1.0f / (cfg.dx * cfg.dx);
    c.inv_dz2 = 1.0f / (cfg.dz * cfg.dz);
    const CpmlXShape xs = cpml_x_shape(N);
    const dim3 xgrid(2, (nza - 8 + xs.rows - 1) / xs.rows, nshots);
    // the x and z strips write disjoint arrays and both only read U(t): the
    // x strips (latency-bound, small blocks) run on strip_stream beside the z
    // strips, joined back into s before anything reads the strip terms
    cudaEventRecord(strip_events[0], s);
    cudaStreamWaitEvent(strip_stream, strip_events[0], 0);
    if (N % 2 == 0) {
        const CpmlXPairShape xp = cpml_x_pair_shape(N);
        const dim3 xpgrid(2, (nza - 8 + xp.rows - 1) / xp.rows, nshots);
        cpml_x_pair_kernel<<<xpgrid, dim3(xp.bx, xp.rows), xp.rows * (2 * xp.bx + 8) * sizeof(float), strip_stream>>>(
            c);
    } else {
        cpml_x_kernel<<<xgrid, dim3(xs.bx, xs.rows), xs.rows * (xs.bx + 8) * sizeof(float), strip_stream>>>(c);
    }
    const int nslab = (nxa - 8 + kCpmlZCols - 1) / kCpmlZCols;
    const dim3 zgrid(nslab, 2, nshots);
    const int zrows = cpml_z_block_rows(N), R = cpml_z_rows_per_thread(N);
    const dim3 zblock(kCpmlZCols, zrows);
    const size_t zsmem = (size_t)(zrows * R + 8) * kCpmlZCols * sizeof(float);
    if (cpml_z_pairs_usable(N)) {
        const int zprows = cpml_z_pair_block_rows(N);
        const size_t zpsmem = (size_t)(zprows * kCpmlZPairRows + 8) * kCpmlZCols * sizeof(float);
        cpml_z_pair_kernel<<<zgrid, dim3(kCpmlZCols / 2, zprows), zpsmem, s>>>(c);
    } else if (R == 6) {
        cpml_z_kernel<6><<<zgrid, zblock, zsmem, s>>>(c);
    } else {
        cpml_z_kernel<8><<<zgrid, zblock, zsmem, s>>>(c);
    }
    cudaEventRecord(strip_events[1], strip_stream);
    cudaStreamWaitEvent(s, strip_events[1], 0);
}

void pam_engine::launch_record(int nshots, const float* cur, float* seis, int it, cudaStream_t s) const {
    RecordArgs r;
    r.cur = cur;
    r.seis = seis;
    r.rz = d_rz;
    r.rx = d_rx;
    r.cerjan = d_cerjan;
    r.status = d_status;
    r.nrec = nrec;
    r.B = nshots;
    r.it = it;
    r.nt_data = nt_data;
    r.per_shot = rec_per_shot;
    r.nz = nza;
    r.nx = nxa;
    r.P = P;
    r.N = N;
    r.cerjan_on = cfg.boundary == PAM_CERJAN;
    r.shot_stride = shot_stride;
    const long long n = (long long)nrec * nshots;
    record_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(r);
}

// Reset fields and memory variables and inject the step-0 source sample.
// After a modelling run has completed: PAM_E_NUMERIC if the recording saw a
// non-finite value (an unstable time step or grid for the model overflows the
// fields within a few dozen steps).
int pam_engine::check_numeric() {
    pam_engine* e = this;
    int v = 0;
    CU(cudaMemcpy(&v, d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (v & 1)
        return fail(PAM_E_NUMERIC, "non-finite values in the seismograms: the scheme is unstable for this model, dt and "
                                   "grid spacing (see pam_check_stability)");
    return PAM_OK;
}

int pam_engine::reset_fields(int nshots, cudaStream_t s) {
    pam_engine* e = this;
    const size_t fb = (size_t)shot_stride * nshots * sizeof(float);
    CU(cudaMemsetAsync(d_status, 0, sizeof(int), s));
    CU(cudaMemsetAsync(d_u[0], 0, fb, s));
    CU(cudaMemsetAsync(d_u[1], 0, fb, s));
    if (cfg.boundary == PAM_CPML) {
        const size_t xb = (size_t)xs_stride * nshots, zb = (size_t)zs_stride * nshots;
        CU(cudaMemsetAsync(d_psix, 0, xb * sizeof(float), s));
        CU(cudaMemsetAsync(d_zetax, 0, xb * sizeof(float), s));
        CU(cudaMemsetAsync(d_xaux, 0, xb * sizeof(float2), s));
        CU(cudaMemsetAsync(d_psiz, 0, zb * sizeof(float), s));
        CU(cudaMemsetAsync(d_zetaz, 0, zb * sizeof(float), s));
        CU(cudaMemsetAsync(d_zaux, 0, zb * sizeof(float2), s));
    }
    inject_first_kernel<<<(nshots + 127) / 128, 128, 0, s>>>(d_u[0], d_sz, d_sx, wavelet[0], nshots, P, shot_stride,
                                                             nza, nxa);
    CU(cudaGetLastError());
    return PAM_OK;
}

// Records the opening event of a sampled launch; *end receives the event to
// record after it (nullptr when step k is not sampled).
void pam_engine::prof_begin(int k, int cls, cudaStream_t s, cudaEvent_t* end) {
    *end = nullptr;
    if (prof_stride <= 0 || k % prof_stride != 0) return;
    if (prof_used == prof.size()) {
        ProfPair p{};
        if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) return;
        prof.push_back(p);
    }
    ProfPair& p = prof[prof_used];
    p.cls = cls;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    prof_flags = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (cudaEventRecordWithFlags(p.a, s, prof_flags) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    prof_used++;
    *end = p.b;
}

// One forward step k for `nshots` shots: CPML memory variables, the stencil
// update into the other buffer, and the recording of U(k).
void pam_engine::enqueue_forward_step(int k, int nshots, float* seis, cudaStream_t s, const float* cur_in,
                                      const float* prev_in, float* nxt_in) {
    // default: the two-buffer rotation (U(t-1) read from and U(t+1) written to
    // the same buffer); explicit buffers write U(t+1) into a third one
    const float* cur = cur_in ? cur_in : d_u[k & 1];
    float* nxt = nxt_in ? nxt_in : d_u[(k + 1) & 1];
    cudaEvent_t end;
    if (cfg.boundary == PAM_CPML) {
        prof_begin(k, 1, s, &end);
        launch_cpml(nshots, cur, s, d_psix, d_zetax, d_xaux, d_psiz, d_zetaz, d_zaux);
        if (end) cudaEventRecordWithFlags(end, s, prof_flags);
    }
    prof_begin(k, 0, s, &end);
    StepArgs a = step_args(k, nshots, cur, nxt, 1);
    a.prev = prev_in;
    launch_step(a, s);
    if (end) cudaEventRecordWithFlags(end, s, prof_flags);
    if (k >= cfg.itlag && seis) {
        prof_begin(k, 2, s, &end);
        launch_record(nshots, cur, seis, k - cfg.itlag, s);
        if (end) cudaEventRecordWithFlags(end, s, prof_flags);
    }
}

// The forward time loop.  With h_seis (pinned host memory, [nshots][nt_data]
// [nrec]) the loop runs as a chain of graphs over kSeisChunks time chunks and
// each chunk's seismogram rows are copied to the host on copy_stream while
// the next chunk computes, so only the last chunk's copy is exposed; the
// caller synchronises s, which waits for the copies.
int pam_engine::run_forward(int nshots, float* d_seis, cudaStream_t s, float* h_seis) {
    pam_engine* e = this;
    if (!models_set) return fail(PAM_E_STATE, "pam_set_models has not been called");
    if (nrec < 1) return fail(PAM_E_STATE, "pam_set_receivers has not been called");
    CU(cudaSetDevice(device));
    const bool use_graph = std::getenv("PAM_NO_GRAPH") == nullptr;
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(s, &capturing));
    const int persist_h = use_graph && capturing == cudaStreamCaptureStatusNone ? persistent_height(nshots) : 0;
    if (!persist_h)   // the persistent path sets its own segment height
        if (int rc = tune_segments(nshots, s)) return rc;
    if (int rc = reset_fields(nshots, s)) return rc;
    if (!use_graph) {
        prof_reset();
        for (int k = 0; k < cfg.nt; k++) enqueue_forward_step(k, nshots, d_seis, s);
        CU(cudaGetLastError());
        if (h_seis)
            CU(cudaMemcpyAsync(h_seis, d_seis, (size_t)nshots * nt_data * nrec * sizeof(float), cudaMemcpyDeviceToHost,
                               s));
        return PAM_OK;
    }
    constexpr int kSeisChunks = 16;
    const int nchunks = h_seis ? std::max(1, std::min(kSeisChunks, nt_data)) : 1;
    if (int H = persist_h) {
        // small run: each chunk of steps is one cooperative launch
        const int per = (nt_data + nchunks - 1) / nchunks;
        std::vector<int> bounds(1, 0);
        for (int c = 1; c < nchunks; c++) bounds.push_back(std::min(cfg.nt, cfg.itlag + c * per));
        bounds.push_back(cfg.nt);
        if (h_seis && !copy_stream) CU(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
        while (h_seis && chunk_events.size() < (size_t)nchunks + 1) {
            cudaEvent_t ev;
            CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            chunk_events.push_back(ev);
        }
        const size_t pitch = (size_t)nt_data * nrec * sizeof(float);
        for (int c = 0; c < nchunks; c++) {
            if (int rc = launch_persistent(nshots, H, d_seis, bounds[c], bounds[c + 1], s)) return rc;
            if (!h_seis) continue;
            const int j0 = std::max(bounds[c] - cfg.itlag, 0), j1 = bounds[c + 1] - cfg.itlag;
            if (j1 <= j0) continue;
            CU(cudaEventRecord(chunk_events[c], s));
            CU(cudaStreamWaitEvent(copy_stream, chunk_events[c], 0));
            const size_t off = (size_t)j0 * nrec;
            CU(cudaMemcpy2DAsync(h_seis + off, pitch, d_seis + off, pitch, (size_t)(j1 - j0) * nrec * sizeof(float),
                                 nshots, cudaMemcpyDeviceToHost, copy_stream));
        }
        if (h_seis) {
            CU(cudaEventRecord(chunk_events[nchunks], copy_stream));
            CU(cudaStreamWaitEvent(s, chunk_events[nchunks], 0));
        }
        return PAM_OK;
    }
    GraphSet& gs = graph_sets[h_seis ? 1 : 0];
    if (gs.execs.size() != (size_t)nchunks || gs.shots != nshots || gs.seis != d_seis) {
        drop_graphs(gs);
        cudaStream_t cs = capture_stream();
        if (!cs) return fail(PAM_E_CUDA, "could not create the capture stream");
        // chunk c ends at the step that records sample c * ceil(nt_data / nchunks)
        const int per = (nt_data + nchunks - 1) / nchunks;
        gs.bounds.assign(1, 0);
        for (int c = 1; c < nchunks; c++) gs.bounds.push_back(std::min(cfg.nt, cfg.itlag + c * per));
        gs.bounds.push_back(cfg.nt);
        prof_reset();
        for (int c = 0; c < nchunks; c++) {
            cudaGraph_t g = nullptr;
            CU(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            for (int k = gs.bounds[c]; k < gs.bounds[c + 1]; k++) enqueue_forward_step(k, nshots, d_seis, cs);
            cudaError_t le = cudaGetLastError();
            cudaError_t ce = cudaStreamEndCapture(cs, &g);
            if (le != cudaSuccess || ce != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                drop_graphs(gs);
                return fail(PAM_E_CUDA, "graph capture failed: %s / %s", cudaGetErrorString(le), cudaGetErrorString(ce));
            }
            cudaGraphExec_t x = nullptr;
            cudaError_t ie = cudaGraphInstantiate(&x, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                drop_graphs(gs);
                return fail(PAM_E_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(ie));
            }
            gs.execs.push_back(x);
        }
        gs.shots = nshots;
        gs.seis = d_seis;
    }
    if (!h_seis) {
        CU(cudaGraphLaunch(gs.execs[0], s));
        return PAM_OK;
    }
    if (!copy_stream) CU(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    while (chunk_events.size() < (size_t)nchunks + 1) {
        cudaEvent_t ev;
        CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        chunk_events.push_back(ev);
    }
    const size_t pitch = (size_t)nt_data * nrec * sizeof(float);
    for (int c = 0; c < nchunks; c++) {
        CU(cudaGraphLaunch(gs.execs[c], s));
        const int j0 = std::max(gs.bounds[c] - cfg.itlag, 0), j1 = gs.bounds[c + 1] - cfg.itlag;
        if (j1 <= j0) continue;
        CU(cudaEventRecord(chunk_events[c], s));
        CU(cudaStreamWaitEvent(copy_stream, chunk_events[c], 0));
        const size_t off = (size_t)j0 * nrec;
        CU(cudaMemcpy2DAsync(h_seis + off, pitch, d_seis + off, pitch, (size_t)(j1 - j0) * nrec * sizeof(float), nshots,
                             cudaMemcpyDeviceToHost, copy_stream));
    }
    CU(cudaEventRecord(chunk_events[nchunks], copy_stream));
    CU(cudaStreamWaitEvent(s, chunk_events[nchunks], 0));
    return PAM_OK;
}

// ---------------------------------------------------------------- persistent small runs

template <int A, int BC>
static cudaError_t launch_persistent_t(const PersistArgs& p, int blocks, cudaStream_t s) {
    constexpr int smem = step_smem_bytes<A>();
    static bool configured[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices || !configured[dev]) {
        cudaFuncSetAttribute(step_persistent_kernel<A, BC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (dev >= 0 && dev < kMaxDevices) configured[dev] = true;
    }
    PersistArgs q = p;
    void* args[] = {&q};
    return cudaLaunchCooperativeKernel((const void*)step_persistent_kernel<A, BC>, dim3(blocks), dim3(32 * kWarpsPerBlock),
                                       args, smem, s);
}

template <int A, int BC>
static int persistent_capacity() {
    // resident blocks of the persistent kernel on this device (0: unknown)
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    constexpr int smem = step_smem_bytes<A>();
    cudaFuncSetAttribute(step_persistent_kernel<A, BC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_persistent_kernel<A, BC>, 32 * kWarpsPerBlock,
                                                      smem) != cudaSuccess)
        return 0;
    return sms * per_sm;
}

// Segment height of the persistent path for this batch, or 0 to use the
// graph of one-step launches.  Only Cerjan runs whose step is small (at most
// kPersistCells cell updates) qualify, with the shortest segments whose
// blocks all stay resident: a step then costs the latency of a short march
// (each warp reloads its nine-row window from L2) plus one grid barrier.
// Single-shot 301 x 501 expanded grid, 2237 steps: 6.55 ms with one row per
// warp, 7.12 with two, 8.68 with four; 13.95 ms as a graph of one-step
// launches.
int pam_engine::persistent_height(int nshots) {
    constexpr long long kPersistCells = 1LL << 20;
    if (cfg.boundary != PAM_CERJAN || prof_stride > 0 || std::getenv("PAM_NO_PERSISTENT")) return 0;
    if ((long long)nshots * nza * nxa > kPersistCells) return 0;
    if (persist_capacity < 0) {
        const int A = cfg.approximation;
        persist_capacity = A == PAM_ACOUSTIC ? persistent_capacity<kAcoustic, kCerjan>()
                         : A == PAM_VTI      ? persistent_capacity<kVTI, kCerjan>()
                                             : persistent_capacity<kTTI, kCerjan>();
        cudaGetLastError();
    }
    for (int h : {1, 2, 4, 8, 16, 32, 64}) {
        const long long nseg_h = (nza - 8 + h - 1) / h;
        const long long blocks = ((long long)nshots * ntiles * nseg_h + kWarpsPerBlock - 1) / kWarpsPerBlock;
        if (blocks <= persist_capacity) return h;
    }
    return 0;
}

int pam_engine::launch_persistent(int nshots, int H, float* d_seis, int k0, int k1, cudaStream_t s) {
    PersistArgs p;
    p.base = step_args(0, nshots, d_u[0], d_u[1], 1);
    p.base.H = H;
    p.base.nseg = (nza - 8 + H - 1) / H;
    p.u[0] = d_u[0];
    p.u[1] = d_u[1];
    p.wavelet = d_wavelet;
    p.rec.cur = nullptr;
    p.rec.seis = d_seis;
    p.rec.rz = d_rz;
    p.rec.rx = d_rx;
    p.rec.cerjan = d_cerjan;
    p.rec.status = d_status;
    p.rec.nrec = nrec;
    p.rec.B = nshots;
    p.rec.it = 0;
    p.rec.nt_data = nt_data;
    p.rec.per_shot = rec_per_shot;
    p.rec.nz = nza;
    p.rec.nx = nxa;
    p.rec.P = P;
    p.rec.N = N;
    p.rec.cerjan_on = 1;
    p.rec.shot_stride = shot_stride;
    p.nt = cfg.nt;
    p.itlag = cfg.itlag;
    p.k0 = k0;
    p.k1 = k1;
    const long long warps = (long long)nshots * ntiles * p.base.nseg;
    const int blocks = (int)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock);
    // enough threads for the recording as well
    const int rec_blocks = (int)(((long long)nrec * nshots + 32 * kWarpsPerBlock - 1) / (32 * kWarpsPerBlock));
    const int grid = std::max(blocks, rec_blocks);
    if (grid > persist_capacity) return fail(PAM_E_CUDA, "persistent launch of %d blocks exceeds %d", grid, persist_capacity);
    const int A = cfg.approximation;
    cudaError_t err = A == PAM_ACOUSTIC ? launch_persistent_t<kAcoustic, kCerjan>(p, grid, s)
                    : A == PAM_VTI      ? launch_persistent_t<kVTI, kCerjan>(p, grid, s)
                                        : launch_persistent_t<kTTI, kCerjan>(p, grid, s);
    if (err != cudaSuccess) return fail(PAM_E_CUDA, "cooperative launch failed: %s", cudaGetErrorString(err));
    return PAM_OK;
}

cudaStream_t pam_engine::capture_stream() {
    if (!cap_stream) {
        if (cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    }
    return cap_stream;
}

// ---------------------------------------------------------------- stability check

int pam_engine::check_stability(float* dt_lim_out, float* dx_lim_out) {
    // Modeling::checkDispersionAndStability (cpp/Modeling.cu:184-327), on the host.
    if (!models_set) return fail(PAM_E_STATE, "pam_set_models has not been called");
    return pam::stability_limits(cfg.approximation, h_vp.size(), h_vp.data(), h_eps.data(), h_del.data(),
                                 h_theta.empty() ? nullptr : h_theta.data(), cfg.dx, cfg.dz, cfg.dt, cfg.fcut,
                                 dt_lim_out, dx_lim_out);
}

// ---------------------------------------------------------------- C ABI

extern "C" {

int pam_create(const pam_config* cfg, int device, pam_engine** out) {
    if (!cfg || !out) return PAM_E_ARG;
    *out = nullptr;
    pam_engine* e = new (std::nothrow) pam_engine();
    if (!e) return PAM_E_ARG;
    int rc = e->init(*cfg, device);
    if (rc != PAM_OK) {
        // keep the handle so the caller can read the error, but mark it unusable
        e->broken = true;
    }
    *out = e;
    return rc;
}

void pam_destroy(pam_engine* e) { delete e; }

const char* pam_last_error(const pam_engine* e) { return e ? e->err.c_str() : "null engine"; }

#define PAM_GUARD(e)                                                                   \
    do {                                                                               \
        if (!(e)) return PAM_E_ARG;                                                    \
        if ((e)->broken) return (e)->fail(PAM_E_STATE, "engine failed to initialise"); \
        (e)->err.clear();                                                              \
    } while (0)

int pam_set_models(pam_engine* e, const float* vp, const float* eps, const float* delta, const float* theta_deg) {
    PAM_GUARD(e);
    return e->set_models(vp, eps, delta, theta_deg);
}

int pam_set_random_boundary(pam_engine* e, float dvel, float ratio, unsigned long long seed) {
    PAM_GUARD(e);
    if (!(dvel >= 0.0f) || !(ratio > 0.0f)) return e->fail(PAM_E_ARG, "dvel must be >= 0 and ratio > 0");
    e->rbc_dvel = dvel;
    e->rbc_ratio = ratio;
    e->rbc_seed = seed;
    return PAM_OK;
}

int pam_autotune(pam_engine* e, int enable) {
    PAM_GUARD(e);
    e->autotune = enable != 0;
    return PAM_OK;
}

int pam_segment_height(const pam_engine* e, int nshots) {
    if (!e) return PAM_E_ARG;
    const auto it = e->seg_height_by_shots.find(nshots);
    return it == e->seg_height_by_shots.end() ? 0 : it->second;
}

int pam_set_wavelet(pam_engine* e, const float* w) {
    PAM_GUARD(e);
    if (!w) return e->fail(PAM_E_ARG, "wavelet is NULL");
    e->wavelet.assign(w, w + e->cfg.nt);
    CU(cudaMemcpy(e->d_wavelet, w, (size_t)e->cfg.nt * sizeof(float), cudaMemcpyHostToDevice));
    e->invalidate_graph();
    return PAM_OK;
}

int pam_set_damping(pam_engine* e, const float* factors) {
    PAM_GUARD(e);
    if (!factors) return e->fail(PAM_E_ARG, "damping factors are NULL");
    if (e->cfg.boundary != PAM_CERJAN) return e->fail(PAM_E_STATE, "damping factors apply to Cerjan boundaries");
    for (int i = 0; i < e->N; i++)
        if (!(factors[i] > 0.0f && factors[i] <= 1.0f))
            return e->fail(PAM_E_ARG, "damping factor %d = %g outside (0, 1]", i, factors[i]);
    CU(cudaSetDevice(e->device));
    // the engine's streams are non-blocking: wait for work that may read the factors
    CU(cudaDeviceSynchronize());
    e->h_cerjan.assign(factors, factors + e->N);
    CU(cudaMemcpy(e->d_cerjan, factors, e->N * sizeof(float), cudaMemcpyHostToDevice));
    return PAM_OK;
}

int pam_set_receivers(pam_engine* e, int nrec, const int* rz, const int* rx, int per_shot) {
    PAM_GUARD(e);
    return e->set_receivers(nrec, rz, rx, per_shot);
}

int pam_forward_device(pam_engine* e, int nshots, const int* d_sz, const int* d_sx, float* d_seis, void* stream) {
    PAM_GUARD(e);
    if (nshots < 1 || nshots > e->B) return e->fail(PAM_E_ARG, "nshots=%d outside [1, %d]", nshots, e->B);
    if (!d_sz || !d_sx || !d_seis) return e->fail(PAM_E_ARG, "null device pointer");
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    CU(cudaSetDevice(e->device));
    CU(cudaMemcpyAsync(e->d_sz, d_sz, nshots * sizeof(int), cudaMemcpyDeviceToDevice, s));
    CU(cudaMemcpyAsync(e->d_sx, d_sx, nshots * sizeof(int), cudaMemcpyDeviceToDevice, s));
    return e->run_forward(nshots, d_seis, s);
}

int pam_forward(pam_engine* e, int nshots, const int* sz, const int* sx, float* seis, void* stream) {
    PAM_GUARD(e);
    if (!sz || !sx || !seis) return e->fail(PAM_E_ARG, "null host pointer");
    if (int rc = e->check_sources(nshots, sz, sx)) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    CU(cudaSetDevice(e->device));
    if (!e->d_seis_own || e->seis_own_shots < e->B) {
        if (dalloc(e, &e->d_seis_own, (size_t)e->B * e->nt_data * std::max(e->nrec, 1))) return PAM_E_CUDA;
        e->seis_own_shots = e->B;
        e->seis_own_nrec = e->nrec;
    }
    if (e->seis_own_nrec < e->nrec) return e->fail(PAM_E_STATE, "receiver count grew after the first forward call");
    CU(cudaMemcpyAsync(e->d_sz, sz, nshots * sizeof(int), cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(e->d_sx, sx, nshots * sizeof(int), cudaMemcpyHostToDevice, s));
    // pinned output: the copies overlap the time loop; pageable: one copy after it
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, seis) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (int rc = e->run_forward(nshots, e->d_seis_own, s, pinned ? seis : nullptr)) return rc;
    if (!pinned) {
        const size_t bytes = (size_t)nshots * e->nt_data * e->nrec * sizeof(float);
        CU(cudaMemcpyAsync(seis, e->d_seis_own, bytes, cudaMemcpyDeviceToHost, s));
    }
    CU(cudaStreamSynchronize(s));
    return e->check_numeric();
}

int pam_begin(pam_engine* e, int nshots, const int* sz, const int* sx) {
    PAM_GUARD(e);
    if (!sz || !sx) return e->fail(PAM_E_ARG, "null host pointer");
    if (int rc = e->check_sources(nshots, sz, sx)) return rc;
    if (!e->models_set) return e->fail(PAM_E_STATE, "pam_set_models has not been called");
    if (e->nrec < 1) return e->fail(PAM_E_STATE, "pam_set_receivers has not been called");
    CU(cudaSetDevice(e->device));
    if (!e->d_seis_own || e->seis_own_nrec < e->nrec) {
        if (dalloc(e, &e->d_seis_own, (size_t)e->B * e->nt_data * e->nrec)) return PAM_E_CUDA;
        e->seis_own_shots = e->B;
        e->seis_own_nrec = e->nrec;
    }
    CU(cudaMemcpyAsync(e->d_sz, sz, nshots * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(e->d_sx, sx, nshots * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemsetAsync(e->d_seis_own, 0, (size_t)nshots * e->nt_data * e->nrec * sizeof(float), e->stream));
    e->step_shots = nshots;
    e->next_step = 0;
    if (int rc = e->tune_segments(nshots, e->stream)) return rc;
    return e->reset_fields(nshots, e->stream);
}

int pam_step(pam_engine* e, int k) {
    PAM_GUARD(e);
    if (e->step_shots < 1) return e->fail(PAM_E_STATE, "pam_begin has not been called");
    if (k != e->next_step || k >= e->cfg.nt) return e->fail(PAM_E_ARG, "step %d out of order (expected %d)", k, e->next_step);
    e->enqueue_forward_step(k, e->step_shots, e->d_seis_own, e->stream);
    CU(cudaGetLastError());
    e->next_step = k + 1;
    return PAM_OK;
}

int pam_read_seismograms(pam_engine* e, float* out) {
    PAM_GUARD(e);
    if (e->step_shots < 1 || !out) return e->fail(PAM_E_STATE, "no shots in flight");
    CU(cudaMemcpyAsync(out, e->d_seis_own, (size_t)e->step_shots * e->nt_data * e->nrec * sizeof(float),
                       cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return e->check_numeric();
}

int pam_read_wavefield(pam_engine* e, int shot, float* out) {
    PAM_GUARD(e);
    if (shot < 0 || shot >= std::max(e->step_shots, 1) || !out) return e->fail(PAM_E_ARG, "bad shot index %d", shot);
    // U(next_step) lives in buffer next_step & 1
    const float* src = e->d_u[e->next_step & 1] + (long long)shot * e->shot_stride;
    CU(cudaMemcpy2DAsync(out, e->nxa * sizeof(float), src, e->P * sizeof(float), e->nxa * sizeof(float), e->nza,
                         cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return PAM_OK;
}

int pam_check_stability(pam_engine* e, float* dt_lim, float* dx_lim) {
    PAM_GUARD(e);
    return e->check_stability(dt_lim, dx_lim);
}

int pam_profile_enable(pam_engine* e, int stride) {
    PAM_GUARD(e);
    if (stride < 0) return e->fail(PAM_E_ARG, "negative profiling stride");
    if (stride != e->prof_stride) {
        e->prof_stride = stride;
        e->invalidate_graph();
    }
    return PAM_OK;
}

int pam_profile_read(pam_engine* e, double* ms, int* count, int nclasses) {
    PAM_GUARD(e);
    if (!ms || !count || nclasses < 1) return e->fail(PAM_E_ARG, "bad output arrays");
    for (int c = 0; c < nclasses; c++) { ms[c] = 0.0; count[c] = 0; }
    for (size_t i = 0; i < e->prof_used; i++) {
        const auto& p = e->prof[i];
        float t = 0.0f;
        cudaError_t r = cudaEventSynchronize(p.b);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&t, p.a, p.b);
        if (r != cudaSuccess) return e->fail(PAM_E_CUDA, "cudaEventElapsedTime: %s", cudaGetErrorString(r));
        if (p.cls < nclasses) { ms[p.cls] += t; count[p.cls] += 1; }
    }
    return PAM_OK;
}

int pam_grid_info(const pam_engine* e, int* nz_abc, int* nx_abc, int* pitch) {
    if (!e) return PAM_E_ARG;
    if (nz_abc) *nz_abc = e->nza;
    if (nx_abc) *nx_abc = e->nxa;
    if (pitch) *pitch = e->P;
    return PAM_OK;
}

}  // extern "C"
