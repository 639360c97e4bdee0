// Device code of the receiver-side (adjoint) propagation: receiver injection,
// imaging conditions, anisotropic adjoint operators, the exact discrete
// adjoint, checkpoint compression and the misfit reduction.  Per-cell
// kernels use 2-D blocks of 32 x 8 threads; their neighbour reads are served
// by L1/L2 (these passes are a small share of a migration or gradient run).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "pam_types.h"

namespace pam {

struct GridDims {
    int nz, nx, P, N;          // expanded grid, pitch, absorbing width
    long long stride;          // nz * P
    const float* cerjan;       // [N] or nullptr (CPML)
};

// Cerjan factor of a cell in the order x then z (cpp/Modeling.cu:535-550);
// 1 outside the border, for CPML runs and outside the update region.
__device__ __forceinline__ float damp_factor(const GridDims& g, int z, int x) {
    if (!g.cerjan || z < 4 || z >= g.nz - 4 || x < 4 || x >= g.nx - 4) return 1.0f;
    float f = 1.0f;
    if (x < g.N) f = f * g.cerjan[x];
    if (x >= g.nx - g.N) f = f * g.cerjan[g.nx - 1 - x];
    float h = 1.0f;
    if (z < g.N) h = g.cerjan[z];
    if (z >= g.nz - g.N) h = h * g.cerjan[g.nz - 1 - z];
    return f * h;
}

// Multi-step damping applied value by value exactly like cpp/Modeling.cu:535-550.
__device__ __forceinline__ float damp_apply(const GridDims& g, int z, int x, float v) {
    if (!g.cerjan || z < 4 || z >= g.nz - 4 || x < 4 || x >= g.nx - 4) return v;
    if (x < g.N) v = v * g.cerjan[x];
    if (x >= g.nx - g.N) v = v * g.cerjan[g.nx - 1 - x];
    if (z < g.N) v = v * g.cerjan[z];
    if (z >= g.nz - g.N) v = v * g.cerjan[g.nz - 1 - z];
    return v;
}

// ---------------------------------------------------------------- receivers

// field[b][rz][rx] += scale * D * data[b][it][r]  (cpp/Migration.cu:493-502);
// atomics keep coincident receivers correct.  D is the Cerjan factor of the
// receiver cell when g.cerjan is set (the transpose of the damped recording),
// 1 otherwise.
__global__ void inject_receivers_kernel(float* __restrict__ field, const float* __restrict__ data,
                                        const int* __restrict__ rz, const int* __restrict__ rx, int nrec, int B,
                                        int it, int nt_data, int per_shot, float scale, GridDims g)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nrec * B) return;
    const int r = (int)(i % nrec);
    const int b = (int)(i / nrec);
    const long long ri = per_shot ? (long long)b * nrec + r : r;
    const int z = rz[ri], x = rx[ri];
    const float v = damp_apply(g, z, x, data[((long long)b * nt_data + it) * nrec + r] * scale);
    atomicAdd(field + (long long)b * g.stride + (long long)z * g.P + x, v);
}

// Residual of the L2 misfit: res = dcal - dobs (or dobs - dcal with sign = -1),
// and per-block partial sums of 0.5 res^2 in double for a deterministic total.
__global__ void residual_kernel(const float* __restrict__ dcal, const float* __restrict__ dobs,
                                float* __restrict__ res, long long n, float sign, double* __restrict__ partial)
{
    __shared__ double red[256];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (i < n) {
        const float r = sign * (dcal[i] - dobs[i]);
        res[i] = r;
        acc = 0.5 * (double)r * (double)r;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// ---------------------------------------------------------------- imaging conditions
// Interior cells (z, x) in [N, nz-N) x [N, nx-N); per-shot accumulators [B][nzi][nxi].

// Zero-lag cross-correlation and source illumination (cpp/Migration.cu:541-552):
// img += Ub * P, ilum += P * P.
__global__ void imaging_kernel(const float* __restrict__ ub, const float* __restrict__ P_, float* __restrict__ img,
                               float* __restrict__ ilum, GridDims g, int nzi, int nxi, long long pstride, int B)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (xi >= nxi || zi >= nzi || b >= B) return;
    const long long c = (long long)(zi + g.N) * g.P + xi + g.N;
    const float p = P_[(long long)b * pstride + c];
    const long long o = ((long long)b * nzi + zi) * nxi + xi;
    ilum[o] += p * p;
    img[o] += ub[(long long)b * g.stride + c] * p;
}

// Reference FWI gradient (cpp/inversion.cu:184-194 per cell):
// g += Ub(t) * (P(t+1) - 2 P(t) + P(t-1)) / dt^2.
__global__ void fwi_ref_grad_kernel(const float* __restrict__ ub, const float* __restrict__ pp,
                                    const float* __restrict__ pc, const float* __restrict__ pf,
                                    float* __restrict__ grad, GridDims g, int nzi, int nxi, long long pstride, int B,
                                    float inv_dt2)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (xi >= nxi || zi >= nzi || b >= B) return;
    const long long c = (long long)(zi + g.N) * g.P + xi + g.N;
    const long long pc_ = (long long)b * pstride + c;
    const float d2 = (pf[pc_] - 2.0f * pc[pc_] + pp[pc_]) * inv_dt2;
    grad[((long long)b * nzi + zi) * nxi + xi] += ub[(long long)b * g.stride + c] * d2;
}

// Illumination only: ilum += P * P (the FWI preconditioner, src/Migration.py:1034).
__global__ void ilum_kernel(const float* __restrict__ P_, float* __restrict__ ilum, GridDims g, int nzi, int nxi,
                            long long pstride, int B)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (xi >= nxi || zi >= nzi || b >= B) return;
    const float p = P_[(long long)b * pstride + (long long)(zi + g.N) * g.P + xi + g.N];
    ilum[((long long)b * nzi + zi) * nxi + xi] += p * p;
}

// Sum per-shot accumulators into the running total: out[i] += sum_b part[b][i]
// (fixed order over b, so the total is deterministic).
__global__ void reduce_shots_kernel(const float* __restrict__ part, float* __restrict__ out, long long n, int B)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = out[i];
    for (int b = 0; b < B; b++) s += part[(long long)b * n + i];
    out[i] = s;
}

// ---------------------------------------------------------------- anisotropic adjoint (RTM)

struct AnisoArgs {
    const float* ub;      // receiver field U(t) [B][nz][P] (after injection)
    const float* pf;      // source field at t (stored U(t)), [B][...] with pstride
    long long pstride;
    const float *eps, *del, *cth, *sth;   // [nz][P]
    float* prod;          // 5 fields [5][B][nz][P]: AU, BU, HU, QCxU, QCzU
    GridDims g;
    int B, tti;
    float inv_dx, inv_dz, inv_dx2, inv_dz2;
};

#define PAM_C0 (-1435.0f / 504.0f)
#define PAM_C1 (8.0f / 5.0f)
#define PAM_C2 (-1.0f / 5.0f)
#define PAM_C3 (8.0f / 315.0f)
#define PAM_C4 (-1.0f / 560.0f)
#define PAM_A1 (4.0f / 5.0f)
#define PAM_A2 (-1.0f / 5.0f)
#define PAM_A3 (4.0f / 105.0f)
#define PAM_A4 (-1.0f / 280.0f)

// Products of cpp/Migration.cu:573-666 (VTI) and :757-861 (TTI), computed from
// the source field P (the reference's saved `current`, i.e. damped U(t)).
__global__ void aniso_products_kernel(const AnisoArgs a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const GridDims& g = a.g;
    if (x >= g.nx || z >= g.nz || b >= a.B) return;
    const long long c = (long long)z * g.P + x;
    const long long fs = (long long)a.B * g.stride;
    float* AU = a.prod + (long long)b * g.stride + c;
    float av = 0.f, bv = 0.f, hv = 0.f, qx = 0.f, qz = 0.f;
    if (x >= 4 && x < g.nx - 4 && z >= 4 && z < g.nz - 4) {
        const float* Pb = a.pf + (long long)b * a.pstride;
        auto P = [&](int dz, int dx) { return damp_apply(g, z + dz, x + dx, Pb[c + (long long)dz * g.P + dx]); };
        const float pxx = (PAM_C0 * P(0, 0) + PAM_C1 * (P(0, 1) + P(0, -1)) + PAM_C2 * (P(0, 2) + P(0, -2)) +
                           PAM_C3 * (P(0, 3) + P(0, -3)) + PAM_C4 * (P(0, 4) + P(0, -4))) * a.inv_dx2;
        const float pzz = (PAM_C0 * P(0, 0) + PAM_C1 * (P(1, 0) + P(-1, 0)) + PAM_C2 * (P(2, 0) + P(-2, 0)) +
                           PAM_C3 * (P(3, 0) + P(-3, 0)) + PAM_C4 * (P(4, 0) + P(-4, 0))) * a.inv_dz2;
        const float px = (PAM_A1 * (P(0, 1) - P(0, -1)) + PAM_A2 * (P(0, 2) - P(0, -2)) +
                          PAM_A3 * (P(0, 3) - P(0, -3)) + PAM_A4 * (P(0, 4) - P(0, -4))) * a.inv_dx;
        const float pz = (PAM_A1 * (P(1, 0) - P(-1, 0)) + PAM_A2 * (P(2, 0) - P(-2, 0)) +
                          PAM_A3 * (P(3, 0) - P(-3, 0)) + PAM_A4 * (P(4, 0) - P(-4, 0))) * a.inv_dz;
        const float e = a.eps[c], d = a.del[c];
        float sd = 0.f, Cx = 0.f, Cz = 0.f;
        float A_, B_;
        if (!a.tti) {
            const float px2 = px * px, pz2 = pz * pz, px4 = px2 * px2, pz4 = pz2 * pz2;
            const float num = -2.0f * (e - d) * px2 * pz2;
            const float den = (1.0f + 2.0f * e) * px4 + pz4 + 2.0f * (1.0f + d) * px2 * pz2;
            if (fabsf(den) > 1.0e-12f) {
                sd = num / den;
                const float inv_den2 = 1.0f / (den * den);
                const float factor = 4.0f * (e - d) * ((1.0f + 2.0f * e) * px4 - pz4) * inv_den2;
                Cx = factor * px * pz2;
                Cz = -factor * px2 * pz;
            }
            A_ = 1.0f + 2.0f * e + sd;
            B_ = 1.0f + sd;
        } else {
            const float cs = a.cth[c], sn = a.sth[c];
            const float xi = px * cs - pz * sn, eta = px * sn + pz * cs;
            const float xi2 = xi * xi, eta2 = eta * eta, xi4 = xi2 * xi2, eta4 = eta2 * eta2;
            const float num = -2.0f * (e - d) * xi2 * eta2;
            const float den = (1.0f + 2.0f * e) * xi4 + eta4 + 2.0f * (1.0f + d) * xi2 * eta2;
            if (fabsf(den) > 1.0e-12f) {
                sd = num / den;
                const float K = (1.0f + 2.0f * e) * xi4 - eta4;
                const float factor = 4.0f * (e - d) * xi * eta * K / (den * den);
                Cx = factor * pz;
                Cz = -factor * px;
            }
            const float cos2 = cs * cs, sin2 = sn * sn;
            A_ = (1.0f + 2.0f * e) * cos2 + sin2 + sd;
            B_ = (1.0f + 2.0f * e) * sin2 + cos2 + sd;
            hv = 2.0f * e * (2.0f * sn * cs);   // 2 eps sin(2 theta)
        }
        const float u = a.ub[(long long)b * g.stride + c];
        const float Q = pxx + pzz;
        av = A_ * u;
        bv = B_ * u;
        hv = hv * u;
        qx = Q * Cx * u;
        qz = Q * Cz * u;
    }
    AU[0] = av;
    AU[fs] = bv;
    AU[2 * fs] = hv;
    AU[3 * fs] = qx;
    AU[4 * fs] = qz;
}

// Update of cpp/Migration.cu:668-755 / :863-973:
// new = D (2 Ub - D Ub_prev + kappa (dxx AU + dzz BU - dxz HU - dx QCxU - dz QCzU)).
// The previous field is stored undamped and damped on read, like the stepping kernel.
__global__ void aniso_adjoint_update_kernel(const AnisoArgs a, float* __restrict__ nxt, const float* __restrict__ kap)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const GridDims& g = a.g;
    if (x < 4 || x >= g.nx - 4 || z < 4 || z >= g.nz - 4 || b >= a.B) return;
    const long long c = (long long)z * g.P + x;
    const long long fs = (long long)a.B * g.stride;
    const float* AU = a.prod + (long long)b * g.stride + c;
    const float* BU = AU + fs;
    const float* HU = AU + 2 * fs;
    const float* QX = AU + 3 * fs;
    const float* QZ = AU + 4 * fs;
    const long long s = g.P;
    float op = (PAM_C0 * AU[0] + PAM_C1 * (AU[1] + AU[-1]) + PAM_C2 * (AU[2] + AU[-2]) +
                PAM_C3 * (AU[3] + AU[-3]) + PAM_C4 * (AU[4] + AU[-4])) * a.inv_dx2 +
               (PAM_C0 * BU[0] + PAM_C1 * (BU[s] + BU[-s]) + PAM_C2 * (BU[2 * s] + BU[-2 * s]) +
                PAM_C3 * (BU[3 * s] + BU[-3 * s]) + PAM_C4 * (BU[4 * s] + BU[-4 * s])) * a.inv_dz2;
    if (a.tti) {
        const float aa[5] = {0.f, PAM_A1, PAM_A2, PAM_A3, PAM_A4};
        float dxz = 0.f;
#pragma unroll
        for (int ax = 1; ax <= 4; ax++) {
            float t = 0.f;
#pragma unroll
            for (int az = 1; az <= 4; az++)
                t += aa[az] * (HU[az * s + ax] - HU[-az * s + ax] + HU[-az * s - ax] - HU[az * s - ax]);
            dxz += aa[ax] * t;
        }
        op -= dxz * (a.inv_dx * a.inv_dz);
    }
    op -= (PAM_A1 * (QX[1] - QX[-1]) + PAM_A2 * (QX[2] - QX[-2]) + PAM_A3 * (QX[3] - QX[-3]) +
           PAM_A4 * (QX[4] - QX[-4])) * a.inv_dx;
    op -= (PAM_A1 * (QZ[s] - QZ[-s]) + PAM_A2 * (QZ[2 * s] - QZ[-2 * s]) + PAM_A3 * (QZ[3 * s] - QZ[-3 * s]) +
           PAM_A4 * (QZ[4 * s] - QZ[-4 * s])) * a.inv_dz;
    const long long o = (long long)b * g.stride + c;
    const float uc = a.ub[o];
    const float prev = damp_apply(g, z, x, nxt[o]);
    nxt[o] = damp_apply(g, z, x, 2.0f * uc - prev + kap[c] * op);
}

// ---------------------------------------------------------------- exact discrete adjoint (acoustic)

// 8th-order Laplacian in the stepping kernel's form: literal coefficients,
// sum, then 1/dx^2 and 1/dz^2 (so that its transpose is exact).
__device__ __forceinline__ float laplacian8(const float* W, long long s, float inv_dx2, float inv_dz2) {
    const float pxx = (PAM_C0 * W[0] + PAM_C1 * (W[1] + W[-1]) + PAM_C2 * (W[2] + W[-2]) +
                       PAM_C3 * (W[3] + W[-3]) + PAM_C4 * (W[4] + W[-4])) * inv_dx2;
    const float pzz = (PAM_C0 * W[0] + PAM_C1 * (W[s] + W[-s]) + PAM_C2 * (W[2 * s] + W[-2 * s]) +
                       PAM_C3 * (W[3 * s] + W[-3 * s]) + PAM_C4 * (W[4 * s] + W[-4 * s])) * inv_dz2;
    return pxx + pzz;
}

// work = kappa * D * l(t+1) on the update region (zero elsewhere).
__global__ void exact_adj_scale_kernel(const float* __restrict__ l1, const float* __restrict__ kap,
                                       float* __restrict__ work, GridDims g, int B)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (x >= g.P || z >= g.nz || b >= B) return;
    const long long c = (long long)z * g.P + x;
    float v = 0.f;
    if (x >= 4 && x < g.nx - 4 && z >= 4 && z < g.nz - 4)
        v = kap[c] * damp_apply(g, z, x, l1[(long long)b * g.stride + c]);
    work[(long long)b * g.stride + c] = v;
}

// l(t) = 2 D l(t+1) + L(work) - D^2 l(t+2): l2 holds l(t+2) on entry, l(t) on exit.
__global__ void exact_adj_update_kernel(const float* __restrict__ l1, float* __restrict__ l2,
                                        const float* __restrict__ work, GridDims g, int B, float inv_dx2,
                                        float inv_dz2)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (x < 4 || x >= g.nx - 4 || z < 4 || z >= g.nz - 4 || b >= B) return;
    const long long o = (long long)b * g.stride + (long long)z * g.P + x;
    const float* W = work + o;
    const long long s = g.P;
    const float lap = laplacian8(W, s, inv_dx2, inv_dz2);
    const float dc = damp_apply(g, z, x, l1[o]);
    const float dp = damp_apply(g, z, x, damp_apply(g, z, x, l2[o]));
    l2[o] = 2.0f * dc + lap - dp;
}

// Exact gradient with respect to kappa on the expanded grid:
// gk += l(t+1) * D * (L U(t)), U(t) the stored field (source included).
__global__ void exact_grad_kernel(const float* __restrict__ l1, const float* __restrict__ U, long long ustride,
                                  float* __restrict__ gk, GridDims g, int B, float inv_dx2, float inv_dz2)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (x < 4 || x >= g.nx - 4 || z < 4 || z >= g.nz - 4 || b >= B) return;
    const long long c = (long long)z * g.P + x;
    const float* W = U + (long long)b * ustride + c;
    const long long s = g.P;
    const float lap = laplacian8(W, s, inv_dx2, inv_dz2);
    const float d = damp_factor(g, z, x);
    gk[(long long)b * g.stride + c] += l1[(long long)b * g.stride + c] * d * lap;
}

// ---------------------------------------------------------------- checkpoints

// Largest |value| of each of `nf` fields of length n: out[f] (as ordered float bits).
__global__ void absmax_kernel(const float* __restrict__ src, long long n, int nf, long long fstride,
                              unsigned* __restrict__ out)
{
    const int f = blockIdx.y;
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(src[(long long)f * fstride + i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out + f, __float_as_uint(m));
}

// dst = src * (1/scale) converted to the storage type (FP32 copies verbatim).
template <typename T>
__global__ void pack_kernel(const float* __restrict__ src, T* __restrict__ dst, long long n, int nf,
                            long long fstride, const unsigned* __restrict__ amax, float target)
{
    const int f = blockIdx.y;
    float inv = 1.0f;
    if (amax) {
        const float m = __uint_as_float(amax[f]);
        inv = m > 0.f ? target / m : 1.0f;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = src[(long long)f * fstride + i] * inv;
        if constexpr (sizeof(T) == 4) dst[(long long)f * n + i] = v;
        else if constexpr (std::is_same<T, __nv_bfloat16>::value) dst[(long long)f * n + i] = __float2bfloat16_rn(v);
        else dst[(long long)f * n + i] = __float2half_rn(v);
    }
}

template <typename T>
__global__ void unpack_kernel(const T* __restrict__ src, float* __restrict__ dst, long long n, int nf,
                              long long fstride, const unsigned* __restrict__ amax, float target)
{
    const int f = blockIdx.y;
    float sc = 1.0f;
    if (amax) {
        const float m = __uint_as_float(amax[f]);
        sc = m > 0.f ? m / target : 1.0f;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float v;
        if constexpr (sizeof(T) == 4) v = src[(long long)f * n + i];
        else if constexpr (std::is_same<T, __nv_bfloat16>::value) v = __bfloat162float(src[(long long)f * n + i]);
        else v = __half2float(src[(long long)f * n + i]);
        dst[(long long)f * fstride + i] = v * sc;
    }
}

}  // namespace pam
