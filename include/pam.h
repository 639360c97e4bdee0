/*
 * pam.h - C ABI of the GB300 finite-difference wave-propagation engine.
 *
 * Drop-in for the hot path of PseudoAcousticModeling: 2-D 8th-order-space /
 * 2nd-order-time acoustic, VTI and TTI pseudo-acoustic propagation with
 * Cerjan or CPML absorbing boundaries, source injection, receiver recording,
 * reverse-time-migration imaging and the FWI gradient.
 *
 * Conventions
 *   - Every function returns PAM_OK (0) or a negative PAM_E* code; the text
 *     of the last error of a handle is available from pam_last_error().
 *     Nothing throws across this boundary.
 *   - Host arrays are caller-owned, row-major float32.  Models are on the
 *     interior grid [nz][nx] (Survey nz, nx); seismograms are [shot][nt_data][nrec].
 *   - Grid indices (source/receiver rows and columns) are on the expanded
 *     grid, i.e. round(coord/d) + N_abc as Survey::readGeometry computes them
 *     (cpp/Survey.cpp:145-175).
 *   - Device memory is owned by the engine.  One handle per host thread.
 *   - `stream` is a cudaStream_t (NULL = the engine's own stream).
 */
#ifndef PAM_H
#define PAM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PAM_OK 0
#define PAM_E_ARG (-1)       /* invalid argument or size */
#define PAM_E_CUDA (-2)      /* CUDA runtime error */
#define PAM_E_STATE (-3)     /* call made in the wrong order (e.g. no model set) */
#define PAM_E_UNSUPPORTED (-4)
#define PAM_E_NUMERIC (-5)   /* non-finite seismograms or misfit (an unstable dt or grid) */

enum pam_approximation { PAM_ACOUSTIC = 0, PAM_VTI = 1, PAM_TTI = 2 };
enum pam_boundary { PAM_CERJAN = 0, PAM_CPML = 1 };
enum pam_store { PAM_STORE_F32 = 0, PAM_STORE_BF16 = 1, PAM_STORE_F16 = 2 };
enum pam_image_norm { PAM_NORM_NONE = 0, PAM_NORM_CPP = 1, PAM_NORM_PY = 2 };

/* Grid, time axis and operator of one job.  Field meanings follow the Survey
 * class (cpp/Survey.hpp:11-125); nt = itlag + nt_data. */
typedef struct pam_config {
    int nz, nx;            /* interior grid */
    int n_abc;             /* absorbing-layer width N_abc */
    float dz, dx, dt;
    int nt;                /* total steps, itlag + nt_data */
    int itlag;             /* source delay in steps */
    float fcut;            /* wavelet cut-off frequency; also sets the CPML alpha */
    int approximation;     /* pam_approximation */
    int boundary;          /* pam_boundary */
    int max_shots;         /* shots per batch; device buffers are sized for it */
} pam_config;

typedef struct pam_engine pam_engine;

/* Create an engine on CUDA device `device`.  Replaces Modeling::Modeling +
 * initializeFields + createWavelet + createCerjanVector
 * (cpp/Modeling.cu:8-120).  The wavelet defaults to the reference Ricker. */
int pam_create(const pam_config* cfg, int device, pam_engine** out);
void pam_destroy(pam_engine* e);
const char* pam_last_error(const pam_engine* e);

/* Models on the interior grid; eps/delta for VTI and TTI, theta in degrees for
 * TTI (NULL otherwise).  Pads by edge replication and builds the boundary
 * tables.  Replaces Modeling::setModel (cpp/Modeling.cu:329-382) minus the
 * file read.  Prints nothing; pam_check_stability reports the CFL check.
 * Waits for the work in flight on the device before replacing the models. */
int pam_set_models(pam_engine* e, const float* vp, const float* eps, const float* delta,
                   const float* theta_deg);

/* Override the source wavelet ([nt] samples, already scaled). Replaces
 * Modeling::createWavelet (cpp/Modeling.cu:84-100). */
int pam_set_wavelet(pam_engine* e, const float* wavelet);

/* Override the Cerjan damping factors ([n_abc] floats, index 0 at the outer
 * edge) of a Cerjan engine.  Replaces Modeling::createCerjanVector
 * (cpp/Modeling.cu:111-120); all ones gives an undamped (reflecting) border,
 * the case in which the reference's update kernels, whose in-place damping
 * races with their neighbours' reads (cpp/Modeling.cu:535-550), are
 * deterministic.  PAM_E_STATE for a CPML engine. */
int pam_set_damping(pam_engine* e, const float* factors);

/* Receivers (expanded-grid indices).  per_shot = 0: one list shared by every
 * shot, arrays [nrec]; per_shot = 1: arrays [max_shots][nrec] giving each shot
 * of a batch its own spread.  Replaces the rx/rz upload of
 * Modeling::initializeFields (cpp/Modeling.cu:78-81). */
int pam_set_receivers(pam_engine* e, int nrec, const int* rz, const int* rx, int per_shot);

/* Forward modelling of a batch of shots: the time loop of
 * Modeling::solveWaveEquation (cpp/Modeling.cu:433-479) for `nshots` shots at
 * once (source cells sz[i], sx[i]).  seis receives [nshots][nt_data][nrec].
 * pam_forward takes host arrays and copies inside; pam_forward_device takes
 * device arrays (sz, sx, seis all on the device).  The loop runs as a CUDA
 * graph of one-step launches, or, for small Cerjan batches (at most 2^20 cell
 * updates per step) on a stream that is not being captured, as one
 * cooperative launch per time chunk with a grid-wide barrier between steps;
 * the seismograms are the same bit for bit. */
int pam_forward(pam_engine* e, int nshots, const int* sz, const int* sx, float* seis, void* stream);
int pam_forward_device(pam_engine* e, int nshots, const int* d_sz, const int* d_sx, float* d_seis,
                       void* stream);

/* Step-level interface, mirroring Modeling::forward_step(k)
 * (cpp/Modeling.cu:421-431) inside the reference's own loop:
 *   pam_begin(e, n, sz, sx)     reset fields, inject step 0
 *   pam_step(e, k)              advance one step, record if k >= itlag
 *   pam_read_seismograms(e, out)  [n][nt_data][nrec]
 *   pam_read_wavefield(e, shot, out)  current U(k+1) on the expanded grid [nz_abc][nx_abc]
 * Arrays are host arrays. */
int pam_begin(pam_engine* e, int nshots, const int* sz, const int* sx);
int pam_step(pam_engine* e, int k);
int pam_read_seismograms(pam_engine* e, float* out);
int pam_read_wavefield(pam_engine* e, int shot, float* out);

/* Source-field strategy value for ckpt_interval: boundary saving
 * (src/Migration.py:288-298, 714-834).  The forward sweep saves the outer
 * four rows and columns of the physical region every step (in `store`
 * format, compressed formats with one scale per 256 cells); the backward
 * sweep rebuilds the source field by stepping backwards in time from the last
 * two states and writing the saved band back after each step.  Exact up to
 * rounding inside the physical region; for pam_rtm and pam_fwi_gradient. */
#define PAM_BOUNDARY_SAVING (-1)

/* Source-field strategy value for ckpt_interval: random boundary (the
 * reference's "RBC", src/Migration.py:327-458, 837-959).  The source field
 * runs undamped through a border of random velocities (pam_set_random_boundary)
 * and is rebuilt by running the same undamped scheme backwards in time:
 * nothing is stored.  The receiver field keeps the absorbing border.  For
 * pam_rtm and pam_fwi_gradient (whose modelled data then come from an extra
 * forward run with the absorbing border). */
#define PAM_RANDOM_BOUNDARY (-2)

/* Random border parameters (Parameters.json "dvel", "ratio"; defaults 1000
 * m/s and 200 m) and the seed of its generator (default 0). */
int pam_set_random_boundary(pam_engine* e, float dvel, float ratio, unsigned long long seed);

/* The random border itself, a host utility with no device work: vp is the
 * interior model [nz][nx]; out receives the expanded model [nz+2N][nx+2N]
 * with the border's velocities drawn as described in pam_set_random_boundary,
 * clipped to vcap.  Returns the number of velocity blobs placed (>= 0), or
 * -1 on invalid arguments.  No counterpart in the reference's C++ (its
 * generator is src/Migration.py:327-458, unseeded). */
int pam_random_boundary(const float* vp, int nz, int nx, int N, float dx, float dz, float dvel, float ratio,
                        float vcap, unsigned long long seed, float* out);

/* Reverse-time migration of a batch (Migration::solveReverseTimeMigration*,
 * cpp/Migration.cu:359-468) with the zero-lag cross-correlation imaging
 * condition and source illumination, accumulated into the engine's image.
 * dobs: host [nshots][nt_data][nrec], muted by the caller (Migration::Mute)
 * or on the GPU by an armed pam_set_mute; from pinned memory the upload
 * overlaps the source field's forward sweep.
 * The source field is rebuilt from checkpoints every `ckpt_interval` steps
 * (0 = store every step, the reference's "onthefly"; PAM_BOUNDARY_SAVING =
 * from saved boundary bands), stored as `store`. */
int pam_rtm(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs,
            int ckpt_interval, int store, void* stream);
/* Image and illumination [nz][nx]; norm = PAM_NORM_CPP divides by the
 * illumination where it exceeds 1e-12 (cpp/Migration.cu:470-484),
 * PAM_NORM_PY by illumination + 1e-5 max (src/Migration.py:563). */
int pam_rtm_result(pam_engine* e, float* image, float* ilum, int norm);
int pam_rtm_reset(pam_engine* e);

/* FWI gradient of the L2 misfit for a batch, reference form: adjoint field
 * driven by the residual dobs - dcal, g += adj(t) (P(t+1) - 2P(t) + P(t-1))/dt^2
 * (cpp/inversion.cu:142-213, loop of src/Migration.py:1030-1049).
 * Accumulates into the engine's gradient; misfit (0.5 sum r^2) is added to
 * *misfit.  Read with pam_fwi_result. */
/* Multiparameter FWI (the reference's "multiparameter" key): with enable != 0,
 * pam_fwi_gradient of a VTI/TTI engine also accumulates the epsilon, delta
 * (and, for TTI, theta in radians) gradients of src/utils.py:1309-1463,
 * read with pam_fwi_multiparameter_result (un-normalised, [nz][nx] each;
 * g_theta may be NULL for VTI).  The anisotropic gradient uses the reference's
 * anisotropic adjoint (cpp/Migration.cu:573-973), Cerjan boundaries only. */
int pam_set_multiparameter(pam_engine* e, int enable);
int pam_fwi_multiparameter_result(pam_engine* e, float* g_eps, float* g_delta, float* g_theta);

int pam_fwi_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs,
                     int ckpt_interval, int store, double* misfit, void* stream);
int pam_fwi_result(pam_engine* e, float* grad, float* ilum);

/* Exact discrete gradient of J = 0.5 sum (d - dobs)^2 with respect to vp on
 * the interior grid (transpose of the forward scheme, Cerjan boundaries; no
 * reference counterpart).  grad_vp [nz][nx] is accumulated into (+=); the
 * misfit is added to *misfit; the source illumination of the batch is added
 * to the illumination pam_fwi_result returns.  Acoustic only. */
int pam_misfit_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* dobs,
                        int ckpt_interval, int store, double* misfit, float* grad_vp, void* stream);

/* The exact adjoint of the forward map d = F(vp) applied to a given adjoint
 * source: grad_vp += (dF/dvp)^T adjoint_source, adjoint_source
 * [nshots][nt_data][nrec] (e.g. dL/dd of any loss).  The job of
 * pam_misfit_gradient with adjoint_source in place of the residual
 * d - dobs: no modelled data are recorded and nothing is subtracted, so the
 * adjoint source enters the adjoint exactly.  Acoustic, Cerjan. */
int pam_adjoint_gradient(pam_engine* e, int nshots, const int* sz, const int* sx, const float* adjoint_source,
                         int ckpt_interval, int store, float* grad_vp, void* stream);

/* Checkpoint planner for pam_rtm / pam_fwi_gradient / pam_misfit_gradient
 * (no counterpart in the reference, whose checkpoint step is a fixed user
 * parameter: src/Migration.py:148-201, cpp/Migration.cu:399-468).  The
 * forward sweep keeps its last segment in the segment buffer, so a job
 * recomputes (nt - last segment) steps; this returns in *ckpt_interval the
 * interval K with the fewest recomputed steps whose buffers - K + 2 field
 * slots for the engine's max_shots plus two `store` fields per earlier
 * segment - fit in budget_bytes (0 when storing every step fits), and in
 * *recomputed (may be NULL) the number of steps that K recomputes.
 * PAM_E_ARG when not even the smallest plan fits. */
int pam_plan_checkpoints(const pam_engine* e, long long budget_bytes, int store, int* ckpt_interval,
                         int* recomputed);

/* Dispersion / stability check of Modeling::checkDispersionAndStability
 * (cpp/Modeling.cu:184-327): writes dt_lim, dx_lim, and returns 1 if both
 * conditions hold, 0 if not, <0 on error. */
int pam_check_stability(pam_engine* e, float* dt_lim, float* dx_lim);

/* The same check without an engine (host only, no GPU needed), for models
 * [nz][nx] as pam_set_models takes them (theta in degrees, TTI only;
 * eps/delta for VTI and TTI). */
int pam_stability_limits(int approximation, int nz, int nx, const float* vp, const float* eps, const float* delta,
                         const float* theta_deg, float dx, float dz, float dt, float fcut, float* dt_lim,
                         float* dx_lim);

/* Kernel timing.  pam_profile_enable(e, stride) makes every `stride`-th
 * forward step bracket its stepping kernel (and, for CPML, the strip kernels)
 * with CUDA events, captured into the step graph, and every `stride`-th
 * backward step of a migration or gradient job its receiver-side kernels;
 * stride 0 turns it off.  After a run has completed, pam_profile_read
 * returns the summed milliseconds and the number of sampled launches of each
 * kernel class (index 0: stepping kernel, 1: CPML strip kernels, 2: receiver
 * recording, 3: the backward step's adjoint kernel (receiver-field step,
 * anisotropic adjoint, or the fused adjoint + gradient pass), 4: the
 * imaging condition or reference-form gradient sum). */
int pam_profile_enable(pam_engine* e, int stride);
int pam_profile_read(pam_engine* e, double* ms, int* count, int nclasses);

/* L2 misfit 0.5 * sum (dcal - dobs)^2 of n float samples that are already in
 * device memory, computed without allocating any device memory.  This entry
 * point has no counterpart in the reference: it exists for callers that
 * cannot allocate where they need the number - a solver loop or serving
 * process whose device memory was sized once up front (a pre-reserved pool,
 * a hard per-process cap shared with other jobs on the GPU), where a
 * cudaMalloc at that point would fail or fragment the pool.
 *
 * The partial sums live in a fixed 512 KiB array inside this library's device
 * image (every GPU that loads the library holds it until the process exits),
 * which limits one call to PAM_MISFIT_NOALLOC_MAX_SAMPLES samples; larger
 * inputs are rejected with PAM_E_ARG and a message on stderr.  The first call
 * on a device looks up that array's device address.  All calls share the one
 * array: calls that overlap on the GPU (from different streams or threads)
 * race and must be serialised by the caller.  `misfit` is a host pointer; the
 * call waits for its stream. */
#define PAM_MISFIT_NOALLOC_MAX_SAMPLES 134217728LL   /* 65,536 partials x 2,048 samples */
int pam_misfit_noalloc(const float* d_dcal, const float* d_dobs, long long n, double* misfit, void* stream);

/* Tile-shape autotuner (no counterpart in the reference, whose kernels use
 * fixed 2-D blocks: cpp/Modeling.cu:448-449).  The first modelling, migration
 * or gradient call for a batch size times the stepping kernel with every
 * candidate segment height (the rows one warp marches: 8 ... 128) and keeps
 * the fastest; results do not depend on the choice.  pam_autotune(e, 0)
 * keeps the default height of 64 for batch sizes not yet tuned.
 * pam_segment_height returns the height chosen for `nshots`, 0 if none yet. */
int pam_autotune(pam_engine* e, int enable);
int pam_segment_height(const pam_engine* e, int nshots);

/* Model smoothing of the migration (Migration::setModel / smoothModel,
 * cpp/Migration.cu:131-236, 252-309) on the GPU, in place on a host array
 * [nz][nx]: separable Gaussian of ceil(6 sigma + 1) taps (made odd), edge
 * indices clamped, applied to the slowness 1/v (parameter = 0) or to the
 * value (parameter != 0, anisotropy); the cells of the water mask keep their
 * value.  The mask is Migration::createMask of `water_model`: its cells
 * within 1e-3 of its minimum.  The reference builds it once from the
 * unsmoothed velocity and uses it for vp, epsilon, delta and theta alike, so
 * pass that velocity (NULL: the model itself, which is the same thing when
 * smoothing the velocity).  Every tap sum is accumulated in float from the
 * first tap to the last, each product and sum rounded on its own, as the
 * reference's host loops are.  Uses the current CUDA device; no engine
 * needed. */
int pam_smooth_model(float* model, int nz, int nx, float sigma, int parameter, const float* water_model);

/* Laplacian post-filter of a migrated image on the GPU (the reference's
 * laplacian_filter, src/Viewdata.py:23-41): out = -(d2/dz2 + d2/dx2) of
 * image [nz][nx] with second-order differences evaluated in double, the
 * first and last rows then columns copied from their neighbours, rounded to
 * float.  Host arrays; uses the current CUDA device; no engine needed. */
int pam_laplacian_filter(const float* image, int nz, int nx, float dz, float dx, float* out);

/* Mute of the observed data on the GPU (Migration::Mute, cpp/Migration.cu:
 * 86-115): samples before the direct arrival t1 = |r - s| / v0 + shift are
 * zeroed and those in [t1, t1 + window) scaled by (t - t1) / window, in the
 * reference's float32 operations (no fused multiply-add).  Arms the mute for
 * the next pam_rtm call, which must model exactly `nshots` shots: it is
 * applied on the device right after the observed data are uploaded (instead
 * of on the host before the call, per shot), then cleared.  Coordinates in
 * metres as in the survey files: shot_x/shot_z [nshots]; rec_x/rec_z [nrec],
 * or [nshots][nrec] with per_shot.  nshots = 0 disarms it. */
int pam_set_mute(pam_engine* e, int nshots, const float* shot_x, const float* shot_z, int nrec,
                 const float* rec_x, const float* rec_z, int per_shot, float v0, float shift, float window);

/* Sizes: expanded grid and row pitch used on the device. */
int pam_grid_info(const pam_engine* e, int* nz_abc, int* nx_abc, int* pitch);

#ifdef __cplusplus
}
#endif
#endif /* PAM_H */
