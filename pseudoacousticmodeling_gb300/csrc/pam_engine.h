// Engine state shared by the translation units of the library (not part of
// the public C ABI; include/pam.h is).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <map>
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
    float *d_e2 = nullptr, *d_m1 = nullptr, *d_m2 = nullptr;   // 1+2eps, -2(eps-delta), 2(1+delta)
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
    int* d_status = nullptr;             // bit 0: a non-finite seismogram sample was recorded
    int check_numeric();                 // PAM_E_NUMERIC (with a message) if that bit is set
    int seis_own_shots = 0, seis_own_nrec = 0;
    std::vector<float> wavelet;
    float* d_wavelet = nullptr;          // [nt], the persistent path's source samples

    // step-level interface
    int step_shots = 0, next_step = 0;

    // streams and graph
    cudaStream_t own_stream = nullptr, stream = nullptr, cap_stream = nullptr;
    // the CPML x strips run on strip_stream beside the z strips (fork / join
    // by the two events around each strip update)
    cudaStream_t strip_stream = nullptr;
    cudaEvent_t strip_events[2] = {nullptr, nullptr};
    // the forward time loop as a chain of graphs over consecutive time chunks:
    // set 0 one chunk (device output), set 1 the chunks of a run streaming its
    // seismograms to pinned host memory; both stay cached
    struct GraphSet {
        std::vector<cudaGraphExec_t> execs;
        std::vector<int> bounds;         // chunk c covers steps [bounds[c], bounds[c+1])
        int shots = -1;
        const float* seis = nullptr;
    };
    GraphSet graph_sets[2];
    void drop_graphs(GraphSet& gs);
    cudaStream_t copy_stream = nullptr;  // seismogram downloads overlapping the next chunk,
                                         // observed-data uploads overlapping the forward sweep
    std::vector<cudaEvent_t> chunk_events;
    cudaEvent_t obs_events[2] = {nullptr, nullptr};

    // sampled kernel timing (events captured into the graph)
    int prof_stride = 0;
    struct ProfPair { cudaEvent_t a, b; int cls; };
    std::vector<ProfPair> prof;
    size_t prof_used = 0;
    unsigned prof_flags = 0;
    void prof_begin(int k, int cls, cudaStream_t s, cudaEvent_t* end);
    void prof_reset() { prof_used = 0; }

    // migration / inversion state (allocated on first use, see pam_adjoint.cu)
    int adj_K = 0, adj_store = -1, adj_nseg = 0, adj_shots = 0;
    void* d_ckpt = nullptr;              // [nseg][2][B][stride] in the storage type
    unsigned* d_ckpt_amax = nullptr;     // [nseg][2][B] per-snapshot |max| (ordered float bits)
    float* d_ckpt_cpml = nullptr;        // [nseg][B][2 xs + 2 zs] CPML memory variables (FP32)
    float* d_seg = nullptr;              // [K+2][B][stride] stored U(t), t = t0-1 .. t0+K
    void* d_band = nullptr;              // boundary saving: [nt-1][B][nband] saved bands in the storage type
    float* d_band_scale = nullptr;       // [nt-1][B][nchunk] inverse scales of the compressed bands
    float* d_u3 = nullptr;               // [B][stride] third source-field buffer of the reverse sweep
    float* d_ones = nullptr;             // [N] unit damping factors (undamped steps)
    float* d_kap_rbc = nullptr;          // [stride] kappa with the random border (source field)
    bool multiparameter = false;         // reference-form gradient also for epsilon, delta (theta)
    float* d_mp = nullptr;               // [3][nz*nx] epsilon, delta, theta gradients, summed over shots
    // mute armed for the next migration call (pam_set_mute)
    int mute_shots = 0, mute_nrec = 0, mute_per_shot = 0;
    float mute_v0 = 0.0f, mute_shift = 0.0f, mute_window = 0.0f;
    float* d_mute = nullptr;             // [sx: shots][sz: shots][rx: R][rz: R], R = nrec or shots * nrec
    size_t mute_cap = 0;
    float rbc_dvel = 1000.0f, rbc_ratio = 200.0f;
    unsigned long long rbc_seed = 0;
    float* d_ub[2] = {nullptr, nullptr};
    float *d_bpsix = nullptr, *d_bzetax = nullptr, *d_bpsiz = nullptr, *d_bzetaz = nullptr;
    float2 *d_bxaux = nullptr, *d_bzaux = nullptr;
    float* d_gk = nullptr;               // [stride]: kappa dJ/dkappa summed over the batch
    float* d_gp = nullptr;               // [ceil(B/4)][stride] partial sums of the fused adjoint +
    float* d_ip = nullptr;               // gradient pass per group of four shots (G and illumination)
    float* d_ilum_b = nullptr;           // [nz][nx] illumination of one exact-gradient call
    float *d_img = nullptr, *d_img_ilum = nullptr, *d_grad = nullptr, *d_grad_ilum = nullptr;   // [nz][nx]
    float* d_obs = nullptr;              // [B][nt_data][nrec], becomes the residual
    double* d_partial = nullptr;
    size_t partial_cap = 0;
    bool adj_base_ready = false;
    int dalloc_bytes(void** p, size_t bytes);
    void dfree(void* p);   // free one tracked allocation (implicitly waits for the device)
    int ensure_adjoint(int K, int store);
    int run_adjoint_job(int mode, int nshots, const int* sz, const int* sx, const float* dobs, int K, int store,
                        double* misfit, float* grad_vp, cudaStream_t s);

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
    void launch_step(const pam::StepArgs& a, cudaStream_t s, int boundary = -1) const;
    void launch_cpml(int nshots, const float* cur, cudaStream_t s, float* psix, float* zetax, float2* xaux,
                     float* psiz, float* zetaz, float2* zaux) const;
    void launch_record(int nshots, const float* cur, float* seis, int it, cudaStream_t s) const;
    int reset_fields(int nshots, cudaStream_t s);
    // Segment height of the stepping kernel per batch size, chosen by
    // timing the candidates on the live buffers (tune_segments); 64 until tuned.
    std::map<int, int> seg_height_by_shots;
    bool autotune = true;
    int seg_height(int nshots) const;
    int tune_segments(int nshots, cudaStream_t s);
    // The persistent path of small Cerjan runs (step_persistent_kernel): the
    // segment height to use for this batch, 0 for the graph path
    int persist_capacity = -1;
    // set by pam_adjoint_gradient: the exact job's data are the adjoint source
    bool adjoint_source_given = false;
    int persistent_height(int nshots);
    int launch_persistent(int nshots, int H, float* d_seis, int k0, int k1, cudaStream_t s);
    // The same for the fused adjoint + gradient kernel of the exact gradient
    // (fewer resident warps per SM than the stepping kernel, so its own
    // height); the stepping kernel's until tuned.
    std::map<int, int> adjgrad_height_by_shots;
    int tune_adjgrad(int nshots, cudaStream_t s);
    void enqueue_forward_step(int k, int nshots, float* seis, cudaStream_t s, const float* cur = nullptr,
                              const float* prev = nullptr, float* nxt = nullptr);
    int run_forward(int nshots, float* d_seis, cudaStream_t s, float* h_seis = nullptr);
    cudaStream_t capture_stream();
};
