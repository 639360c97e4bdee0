// Argument blocks and launch constants shared by the translation units of the
// engine (kernels themselves live in pam_kernels.cuh / pam_adjoint_kernels.cuh).
#pragma once
#include <cuda_runtime.h>

namespace pam {

constexpr int kTileOut = 120;    // columns written per warp with halo lanes (TTI)
constexpr int kTileLoad = 128;   // columns loaded per warp (all lanes)
constexpr int kTileWide = 128;   // columns covered per warp with fetched halos (acoustic, VTI)
constexpr int kWarpsPerBlock = 4;
constexpr int kCpmlMaxStrip = 256;   // N - 4 <= 256

enum Approx { kAcoustic = 0, kVTI = 1, kTTI = 2 };
enum Boundary { kCerjan = 0, kCPML = 1 };

struct StepArgs {
    const float* __restrict__ cur;   // U(t), source of step t already added
    float* __restrict__ nxt;         // in: U(t-1) as stored (unless prev is set); out: U(t+1) (+ source t+1)
    const float* prev;               // U(t-1) in a buffer of its own, or nullptr (then read from nxt)
    const float* __restrict__ kap;   // vp^2 dt^2
    const float* __restrict__ eps;   // unused by the stepping kernel (adjoint products read it)
    const float* __restrict__ del;
    const float* __restrict__ e2;    // 1 + 2 eps         per-cell coefficients of the VTI/TTI
    const float* __restrict__ m1;    // -2 (eps - delta)  update, precomputed with the reference's
    const float* __restrict__ m2;    // 2 (1 + delta)     expressions (cpp/Modeling.cu:605-613)
    const float* __restrict__ cth;   // cos(theta)
    const float* __restrict__ sth;   // sin(theta)
    const float* __restrict__ cerjan;    // [N] Cerjan factors
    const float2* __restrict__ xaux;     // CPML x strip terms
    const float2* __restrict__ zaux;     // CPML z strip terms
    const int* __restrict__ src_z;       // [B] source row (expanded grid)
    const int* __restrict__ src_x;       // [B] source column
    float src_amp;                       // wavelet sample t+1 (0 past the end)
    int nz, nx, P, N;
    long long shot_stride;               // nz * P
    long long xaux_stride;               // nz * 2N
    long long zaux_stride;               // 2N * P
    int B, ntiles, nseg, H;
    float inv_dx, inv_dz, inv_dx2, inv_dz2;
    // first-derivative coefficients A_k / d (k = 1..4); the second derivative
    // uses the literal C_k and multiplies by 1/d^2 after the sum, as the
    // reference does
    float cx1[4], cz1[4];
};

struct CpmlArgs {
    const float* __restrict__ cur;   // U(t)
    float* __restrict__ psix; float* __restrict__ zetax; float2* __restrict__ xaux;   // [B][nz][2N]
    float* __restrict__ psiz; float* __restrict__ zetaz; float2* __restrict__ zaux;   // [B][2N][P]
    const float2* __restrict__ cxab;   // [nz][2N]  (a, b) for x strips
    const float2* __restrict__ czab;   // [2N][P]   (a, b) for z strips
    int nz, nx, P, N, B;
    long long shot_stride, xs_stride, zs_stride;
    float inv_dx, inv_dz, inv_dx2, inv_dz2;
};

struct RecordArgs {
    const float* __restrict__ cur;
    float* __restrict__ seis;        // [B][nt_data][nrec]
    const int* __restrict__ rz;      // [nrec] or [B][nrec]
    const int* __restrict__ rx;
    const float* __restrict__ cerjan;
    int* status;                     // bit 0 set when a recorded value is not finite
    int nrec, B, it, nt_data, per_shot, nz, nx, P, N, cerjan_on;
    long long shot_stride;
};

}  // namespace pam
