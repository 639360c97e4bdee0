// Engine state shared by the translation units of the library (not part of
// the public C ABI; include/pam.h is).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pam.h"
#include "pam_types.h"

struct pam_engine {
    pam_config cfg{};
    int device = 0;
    bool broken = false;
    std::string err;
    int fail(int code, const char* fmt, ...);

    // geometry
    int N = 0, nza = 0, nxa = 0, P = 0, ntiles = 0, nseg = 0, H = 64, B = 0, nt_data = 0;
    long long shot_stride = 0, xs_stride = 0, zs_stride = 0;

    // shared model and boundary tables
    float *d_kap = nullptr, *d_eps = nullptr, *d_del = nullptr, *d_cth = nullptr, *d_sth = nullptr;
    float* d_cerjan = nullptr;
    float2 *d_cxab = nullptr, *d_czab = nullptr;
    std::vector<float> h_vp, h_eps, h_del, h_theta, h_cerjan;
    bool models_set = false;

    // per-shot state
    float* d_u[2] = {nullptr, nullptr};
    float *d_psix = nullptr, *d_zetax = nullptr, *d_psiz = nullptr, *d_zetaz = nullptr;
    float2 *d_xaux = nullptr, *d_zaux = nullptr;
    int *d_sz = nullptr, *d_sx = nullptr;
    int *d_rz = nullptr, *d_rx = nullptr;
    size_t rec_cap = 0;
    int nrec = 0, rec_per_shot = 0;
    float* d_seis_own = nullptr;
    int seis_own_shots = 0, seis_own_nrec = 0;
    std::vector<float> wavelet;

    // step-level interface
    int step_shots = 0, next_step = 0;

    // streams and graph
    cudaStream_t own_stream = nullptr, stream = nullptr, cap_stream = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_key_shots = -1;
    const float* graph_key_seis = nullptr;

    // sampled kernel timing (events captured into the graph)
    int prof_stride = 0;
    struct ProfPair { cudaEvent_t a, b; int cls; };
    std::vector<ProfPair> prof;
    size_t prof_used = 0;
    unsigned prof_flags = 0;
    void prof_begin(int k, int cls, cudaStream_t s, cudaEvent_t* end);
    void prof_reset() { prof_used = 0; }

    std::vector<void*> allocs, host_allocs;
    size_t bytes_allocated = 0;

    ~pam_engine();
    int init(const pam_config& c, int dev);
    int set_models(const float* vp, const float* eps, const float* del, const float* theta_deg);
    int set_receivers(int n, const int* rz, const int* rx, int per_shot);
    int check_sources(int nshots, const int* sz, const int* sx);
    int check_stability(float* dt_lim, float* dx_lim);
    void invalidate_graph();
    pam::StepArgs step_args(int k, int nshots, const float* cur, float* nxt, int fwd_src) const;
    void launch_step(const pam::StepArgs& a, cudaStream_t s) const;
    void launch_cpml(int nshots, const float* cur, cudaStream_t s, float* psix, float* zetax, float2* xaux,
                     float* psiz, float* zetaz, float2* zaux) const;
    void launch_record(int nshots, const float* cur, float* seis, int it, cudaStream_t s) const;
    int reset_fields(int nshots, cudaStream_t s);
    void enqueue_forward_step(int k, int nshots, float* seis, cudaStream_t s);
    int run_forward(int nshots, float* d_seis, cudaStream_t s);
    cudaStream_t capture_stream();
};
