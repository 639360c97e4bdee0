// Device code of the receiver-side (adjoint) propagation: receiver injection,
// imaging conditions, anisotropic adjoint operators, the exact discrete
// adjoint, checkpoint compression and the misfit reduction.  Per-cell
// kernels use 2-D blocks of 32 x 8 threads; their neighbour reads are served
// by L1/L2 (these passes are a small share of a migration or gradient run).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "pam_check.cuh"
#include "pam_kernels.cuh"
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
// res may be dobs (the residual overwrites the observed data in place): each
// thread reads and writes only its own sample, so those two are not restrict
__global__ void residual_kernel(const float* __restrict__ dcal, const float* dobs, float* res, long long n,
                                float sign, double* __restrict__ partial)
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
// Interior cells (z, x) in [N, nz-N) x [N, nx-N), totals [nzi][nxi]:
// - imaging: zero-lag cross-correlation img += Ub(t) P(t) and source
//   illumination ilum += P(t)^2 (cpp/Migration.cu:541-552);
// - reference FWI gradient g += Ub(t) (P(t+1) - 2 P(t) + P(t-1)) / dt^2
//   (cpp/inversion.cu:184-194 per cell);
// - illumination only, the FWI preconditioner (src/Migration.py:1034).
// Each sums the batch in registers (shots in order b = 0 .. B-1) and adds to
// the running totals once per step: one thread per interior cell, 8 B read
// per cell and shot (16 B for the gradient), where per-shot accumulators would
// also read and write 8 B per cell and shot.  The reference sums each shot's
// image over time first (src/Migration.py:553); summing the shots of a step
// first changes only the rounding order.
// One thread per 16-byte quad of field columns [4 q, 4 q + 4), counted from
// column 0 of the pitched row, so each warp reads whole aligned 128-byte lines
// (the interior starts N columns in); cells outside the interior are skipped
// when the sums are added.  Pairs of cells use the packed FP32 instructions.
__global__ void imaging_sum_kernel(const float* __restrict__ ub, const float* __restrict__ P_, float* __restrict__ img,
                                   float* __restrict__ ilum, GridDims g, int nzi, int nxi, long long pstride, int B)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    const int xf0 = 4 * q;                                   // first field column of the quad
    if (zi >= nzi || xf0 >= g.N + nxi || xf0 + 4 <= g.N) return;
    const long long c = (long long)(zi + g.N) * g.P + xf0;   // 16-byte aligned: P and the strides are multiples of 32
    float2 si0 = make_float2(0.f, 0.f), si1 = si0, sg0 = si0, sg1 = si0;
#pragma unroll 4
    for (int b = 0; b < B; b++) {
        const float4 p = *reinterpret_cast<const float4*>(
            PAM_CHK(P_ + (long long)b * pstride + c, P_, (long long)B * pstride * 4, 16, 60));
        const float4 u = *reinterpret_cast<const float4*>(
            PAM_CHK(ub + (long long)b * g.stride + c, ub, (long long)B * g.stride * 4, 16, 61));
        const float2 p0 = make_float2(p.x, p.y), p1 = make_float2(p.z, p.w);
        si0 = __ffma2_rn(p0, p0, si0);
        si1 = __ffma2_rn(p1, p1, si1);
        sg0 = __ffma2_rn(make_float2(u.x, u.y), p0, sg0);
        sg1 = __ffma2_rn(make_float2(u.z, u.w), p1, sg1);
    }
    const float si[4] = {si0.x, si0.y, si1.x, si1.y}, sg[4] = {sg0.x, sg0.y, sg1.x, sg1.y};
    const long long row = (long long)zi * nxi;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int xi = xf0 + j - g.N;
        if (xi >= 0 && xi < nxi) {
            *PAM_CHK(&ilum[row + xi], ilum, (long long)nzi * nxi * 4, 4, 62) += si[j];
            *PAM_CHK(&img[row + xi], img, (long long)nzi * nxi * 4, 4, 62) += sg[j];
        }
    }
}

__global__ void fwi_ref_grad_sum_kernel(const float* __restrict__ ub, const float* __restrict__ pp,
                                        const float* __restrict__ pc, const float* __restrict__ pf,
                                        float* __restrict__ grad, GridDims g, int nzi, int nxi, long long pstride,
                                        int B, float inv_dt2)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= nxi || zi >= nzi) return;
    const long long c = (long long)(zi + g.N) * g.P + xi + g.N;
    float sg = 0.0f;
#pragma unroll 4
    for (int b = 0; b < B; b++) {
        const long long pc_ = (long long)b * pstride + c;
        const float d2 = (pf[pc_] - 2.0f * pc[pc_] + pp[pc_]) * inv_dt2;
        sg += ub[(long long)b * g.stride + c] * d2;
    }
    grad[(long long)zi * nxi + xi] += sg;
}

__global__ void ilum_sum_kernel(const float* __restrict__ P_, float* __restrict__ ilum, GridDims g, int nzi, int nxi,
                                long long pstride, int B)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= nxi || zi >= nzi) return;
    const long long c = (long long)(zi + g.N) * g.P + xi + g.N;
    float si = 0.0f;
#pragma unroll 4
    for (int b = 0; b < B; b++) {
        const float p = P_[(long long)b * pstride + c];
        si += p * p;
    }
    ilum[(long long)zi * nxi + xi] += si;
}

// Sum per-shot accumulators into the running total: out[i] += sum_b part[b][i]
// (fixed order over b, so the total is deterministic).
// Migration::Mute (cpp/Migration.cu:86-115) of observed data [B][nt][nrec] in
// place: zero before t1 = sqrt(dz dz + dx dx) / v0 + shift, scale by
// (t - t1) / (t2 - t1) up to t2 = t1 + window, with t = it * dt.  Each float
// operation rounds separately (no contraction), as the host code does.  One
// thread per (receiver, shot, chunk of `rows` time samples); rows at or after
// t2 are not touched, so a thread stops at the first of them.
__global__ void mute_kernel(float* __restrict__ d, const float* __restrict__ coords, int B, int nt, int nrec,
                            int per_shot, float dt, float v0, float shift, float window, int rows)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.z;
    if (r >= nrec) return;
    const long long R = per_shot ? (long long)B * nrec : nrec;
    const long long ri = (per_shot ? (long long)b * nrec : 0) + r;
    const float ddz = __fsub_rn(coords[2 * B + R + ri], coords[B + b]);
    const float ddx = __fsub_rn(coords[2 * B + ri], coords[b]);
    const float t1 = __fadd_rn(__fdiv_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(ddz, ddz), __fmul_rn(ddx, ddx))), v0), shift);
    const float t2 = __fadd_rn(t1, window);
    const float span = __fsub_rn(t2, t1);
    const int it0 = blockIdx.y * rows, it1 = min(it0 + rows, nt);
    float* col = d + (long long)b * nt * nrec + r;
    for (int it = it0; it < it1; it++) {
        const float t = __fmul_rn((float)it, dt);
        if (t >= t2) break;          // t grows with it: no later sample of this chunk changes
        float* p = col + (long long)it * nrec;
        if (t < t1) *p = 0.0f;
        else if (t < t2) *p = __fmul_rn(*p, __fdiv_rn(__fsub_rn(t, t1), span));
    }
}

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

// One backward step of the reference's anisotropic adjoint in a single pass.
//
// The reference (cpp/Migration.cu:573-973) runs it in two kernels: the first
// writes five products of the receiver field U with coefficients taken from
// the source field P (cpp/Migration.cu:573-666 VTI, :757-861 TTI)
//   AU = A U, BU = B U, HU = 2 eps sin(2 theta) U (TTI), QCxU, QCzU,
// the second applies their derivatives (cpp/Migration.cu:668-755, :863-973)
//   new = D (2 U - D U_prev + kappa (dxx AU + dzz BU - dxz HU - dx QCxU - dz QCzU)).
// Here a block owns a 32 x 32 output tile of one shot.  It loads the damped
// source field of the tile with an 8-cell halo into shared memory, forms the
// products of the tile with a 4-cell halo (the update's stencil reach) in
// shared memory, and applies the update from there: no product ever goes to
// HBM.  Per cell and shot the step reads P, U, U_prev and writes the new
// field (16 B) instead of also writing and re-reading five product fields;
// the products of the halo cells are computed again by the neighbouring
// tiles (1.56x the product arithmetic).  The per-cell expressions are the
// reference's, in its order, with its correctly rounded divisions (the
// hardware reciprocal in their place measured no faster).  (Keeping four rows of the z-differentiated products per thread in
// registers raised the registers from 41 to 57, cut the resident blocks from
// six to four per SM and made the kernel 15% slower.)
// Packed second and first derivatives of a cell pair for the anisotropic
// adjoint: (C0 c + C1 (p1 + m1) + ... + C4 (p4 + m4)) * inv and
// (A1 (p1 - m1) + ... + A4 (p4 - m4)) * inv, the coefficients of the
// reference's adjoint kernels (cpp/Migration.cu:600-640).
__device__ __forceinline__ float2 an_d2(float2 c, float2 p1, float2 m1, float2 p2, float2 m2, float2 p3, float2 m3,
                                       float2 p4, float2 m4, float inv) {
    float2 t = pmul2(bc2(PAM_C0), c);
    t = pfma2(bc2(PAM_C1), padd2(p1, m1), t);
    t = pfma2(bc2(PAM_C2), padd2(p2, m2), t);
    t = pfma2(bc2(PAM_C3), padd2(p3, m3), t);
    t = pfma2(bc2(PAM_C4), padd2(p4, m4), t);
    return pmul2(t, bc2(inv));
}
__device__ __forceinline__ float2 an_d1(float2 p1, float2 m1, float2 p2, float2 m2, float2 p3, float2 m3, float2 p4,
                                       float2 m4, float inv) {
    float2 t = pmul2(bc2(PAM_A1), fsub2(p1, m1));
    t = pfma2(bc2(PAM_A2), fsub2(p2, m2), t);
    t = pfma2(bc2(PAM_A3), fsub2(p3, m3), t);
    t = pfma2(bc2(PAM_A4), fsub2(p4, m4), t);
    return pmul2(t, bc2(inv));
}

constexpr int kAnTX = 32, kAnTZ = 32;                 // output tile
constexpr int kAnQX = kAnTX + 8, kAnQZ = kAnTZ + 8;   // products: tile + 4-cell halo
constexpr int kAnSX = kAnTX + 16, kAnSZ = kAnTZ + 16; // source field: tile + 8-cell halo
constexpr int kAnThreads = 256;                       // launched as (32, 8) threads

__host__ __device__ constexpr int aniso_tile_smem_bytes(int tti) {
    return (kAnSZ * kAnSX + kAnQZ * kAnQX * (tti ? 5 : 4)) * 4;
}

template <bool TTI>
__global__ void __launch_bounds__(kAnThreads, TTI ? 4 : 5) aniso_adjoint_tile_kernel(const AnisoArgs a, float* __restrict__ nxt,
                                                                 const float* __restrict__ kap)
{
    extern __shared__ float an_sm[];
    float* Ps = an_sm;                                  // [kAnSZ][kAnSX] damped P
    float* AUs = Ps + kAnSZ * kAnSX;                    // [kAnQZ][kAnQX] each
    float* BUs = AUs + kAnQZ * kAnQX;
    float* QXs = BUs + kAnQZ * kAnQX;
    float* QZs = QXs + kAnQZ * kAnQX;
    float* HUs = QZs + kAnQZ * kAnQX;                   // TTI only
    const GridDims& g = a.g;
    const int x0 = blockIdx.x * kAnTX, z0 = blockIdx.y * kAnTZ, b = blockIdx.z;
    // launched as (32, 8) threads: in the update threadIdx.x runs along x, a warp per row
    [[maybe_unused]] const long long pbytes = (long long)a.B * a.pstride * 4;
    [[maybe_unused]] const long long fbytes = (long long)a.B * g.stride * 4;
    [[maybe_unused]] const long long mbytes = (long long)g.nz * g.P * 4;
    const float* Pb = a.pf + (long long)b * a.pstride;
    const float* Ub = a.ub + (long long)b * g.stride;

    // 1. the damped source field of the tile and its 8-cell halo (zero off
    //    the grid, where only products outside the update region would read)
    // block-uniform: does the source-field region / the output tile reach
    // into the damped border (damp_apply leaves every other cell as it is)?
    const bool src_damped = g.cerjan && !(x0 - 8 >= g.N && x0 + kAnTX + 8 <= g.nx - g.N && z0 - 8 >= g.N &&
                                          z0 + kAnTZ + 8 <= g.nz - g.N);
    const bool out_damped = g.cerjan && !(x0 >= g.N && x0 + kAnTX <= g.nx - g.N && z0 >= g.N &&
                                          z0 + kAnTZ <= g.nz - g.N);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    // every global operand of the products arrives in one batch of 16-byte
    // cp.async (x0 is a multiple of 32, so every quad below starts on a
    // 16-byte boundary of its row: the launcher checks the bases and pitches):
    // the source field of the tile and its 8-cell halo into Ps (zero off the
    // grid, where only products outside the update region would read), and
    // the products' per-cell operands - eps, delta, U (and cos, sin for TTI) -
    // into the product arrays AU, BU, QX (QZ, HU), each at the cell whose
    // product later overwrites it, for quads that reach into the update region
    constexpr int SQX = kAnSX / 4;                       // quads per source row
    for (int i = tid; i < kAnSZ * SQX; i += kAnThreads) {
        const int r = i / SQX, cq = (i % SQX) * 4;
        const int z = z0 - 8 + r, x = x0 - 8 + cq;
        float* dst = Ps + r * kAnSX + cq;
        const bool zon = z >= 0 && z < g.nz;
        if (zon && x >= 0 && x + 3 < g.nx) {
            cp_async16(dst, PAM_CHK(Pb + (long long)z * g.P + x, a.pf, pbytes, 16, 92));
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                dst[k] = (zon && x + k >= 0 && x + k < g.nx)
                             ? *PAM_CHK(Pb + (long long)z * g.P + x + k, a.pf, pbytes, 4, 92) : 0.0f;
        }
    }
    constexpr int QQX = kAnQX / 4;                       // quads per product row
    constexpr int NSTAGE = TTI ? 5 : 3;
    for (int i = tid; i < NSTAGE * kAnQZ * QQX; i += kAnThreads) {
        const int arr = i / (kAnQZ * QQX), j = i % (kAnQZ * QQX);
        const int r = j / QQX, cq = (j % QQX) * 4;
        const int z = z0 - 4 + r, x = x0 - 4 + cq;
        if (z >= 4 && z < g.nz - 4 && x >= 4 && x < g.nx - 4) {
            const long long m = (long long)z * g.P + x;
            const float* src;
            switch (arr) {
                case 0: src = PAM_CHK(a.eps + m, a.eps, mbytes, 16, 93); break;
                case 1: src = PAM_CHK(a.del + m, a.del, mbytes, 16, 93); break;
                case 2: src = PAM_CHK(Ub + m, a.ub, fbytes, 16, 94); break;
                case 3: src = PAM_CHK(a.cth + m, a.cth, mbytes, 16, 93); break;
                default: src = PAM_CHK(a.sth + m, a.sth, mbytes, 16, 93); break;
            }
            cp_async16(AUs + arr * (kAnQZ * kAnQX) + r * kAnQX + cq, src);
        }
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    if (src_damped) {
        for (int i = tid; i < kAnSZ * kAnSX; i += kAnThreads) {
            const int z = z0 - 8 + i / kAnSX, x = x0 - 8 + i % kAnSX;
            if (z >= 0 && z < g.nz && x >= 0 && x < g.nx) Ps[i] = damp_apply(g, z, x, Ps[i]);
        }
        __syncthreads();
    }

    // 2. the products of the tile and its 4-cell halo (zero outside the
    //    update region, as the reference's products kernel leaves them), for
    //    pairs of x-adjacent cells: 8-byte shared loads and the packed FP32x2
    //    instructions for the derivatives, the Sd ratio per cell
    constexpr int QXP = kAnQX / 2;
    for (int i = tid; i < kAnQZ * QXP; i += kAnThreads) {   // whole warps on consecutive pairs
        const int qz = i / QXP, qx = (i % QXP) * 2;
        const int z = z0 - 4 + qz, x = x0 - 4 + qx;
        const bool zin = z >= 4 && z < g.nz - 4;
        const bool in0 = zin && x >= 4 && x < g.nx - 4, in1 = zin && x + 1 >= 4 && x + 1 < g.nx - 4;
        float2 av = make_float2(0.f, 0.f), bv = av, hv = av, qxv = av, qzv = av;
        if (in0 || in1) {
            const float* c = Ps + (qz + 4) * kAnSX + (qx + 4);
            auto L = [&](int off) { return *reinterpret_cast<const float2*>(c + off); };   // even offsets
            const float2 A0 = L(-4), A1 = L(-2), A2 = L(0), A3 = L(2), A4 = L(4);
            const float2 Om3 = make_float2(A0.y, A1.x), Om1 = make_float2(A1.y, A2.x);
            const float2 Op1 = make_float2(A2.y, A3.x), Op3 = make_float2(A3.y, A4.x);
            const float2 Z1 = L(kAnSX), Zm1 = L(-kAnSX), Z2 = L(2 * kAnSX), Zm2 = L(-2 * kAnSX);
            const float2 Z3 = L(3 * kAnSX), Zm3 = L(-3 * kAnSX), Z4 = L(4 * kAnSX), Zm4 = L(-4 * kAnSX);
            const float2 pxx = an_d2(A2, Op1, Om1, A3, A1, Op3, Om3, A4, A0, a.inv_dx2);
            const float2 pzz = an_d2(A2, Z1, Zm1, Z2, Zm2, Z3, Zm3, Z4, Zm4, a.inv_dz2);
            const float2 px = an_d1(Op1, Om1, A3, A1, Op3, Om3, A4, A0, a.inv_dx);
            const float2 pz = an_d1(Z1, Zm1, Z2, Zm2, Z3, Zm3, Z4, Zm4, a.inv_dz);
            // the staged operands of this pair (overwritten by its products below)
            const int qs = qz * kAnQX + qx;
            const float2 e2v = *reinterpret_cast<const float2*>(AUs + qs);
            const float2 d2v = *reinterpret_cast<const float2*>(BUs + qs);
            const float2 u2 = *reinterpret_cast<const float2*>(QXs + qs);
            float2 cs2 = make_float2(0.f, 0.f), sn2 = cs2;
            if (TTI) {
                cs2 = *reinterpret_cast<const float2*>(QZs + qs);
                sn2 = *reinterpret_cast<const float2*>(HUs + qs);
            }
            // the reference's per-cell products (cpp/Migration.cu:573-666, 757-861)
            auto cell = [&](float pxs, float pzs, float pxxs, float pzzs, float e, float d, float u, float cs, float sn,
                            float& A_u, float& B_u, float& H_u, float& QX_u, float& QZ_u) {
                float sd = 0.f, Cx = 0.f, Cz = 0.f, A_, B_, hs = 0.f;
                if (!TTI) {
                    const float px2 = pxs * pxs, pz2 = pzs * pzs, px4 = px2 * px2, pz4 = pz2 * pz2;
                    const float num = -2.0f * (e - d) * px2 * pz2;
                    const float den = (1.0f + 2.0f * e) * px4 + pz4 + 2.0f * (1.0f + d) * px2 * pz2;
                    if (fabsf(den) > 1.0e-12f) {
                        sd = num / den;
                        const float inv_den2 = 1.0f / (den * den);
                        const float factor = 4.0f * (e - d) * ((1.0f + 2.0f * e) * px4 - pz4) * inv_den2;
                        Cx = factor * pxs * pz2;
                        Cz = -factor * px2 * pzs;
                    }
                    A_ = 1.0f + 2.0f * e + sd;
                    B_ = 1.0f + sd;
                } else {
                    const float xi = pxs * cs - pzs * sn, eta = pxs * sn + pzs * cs;
                    const float xi2 = xi * xi, eta2 = eta * eta, xi4 = xi2 * xi2, eta4 = eta2 * eta2;
                    const float num = -2.0f * (e - d) * xi2 * eta2;
                    const float den = (1.0f + 2.0f * e) * xi4 + eta4 + 2.0f * (1.0f + d) * xi2 * eta2;
                    if (fabsf(den) > 1.0e-12f) {
                        sd = num / den;
                        const float K = (1.0f + 2.0f * e) * xi4 - eta4;
                        const float factor = 4.0f * (e - d) * xi * eta * K / (den * den);
                        Cx = factor * pzs;
                        Cz = -factor * pxs;
                    }
                    const float cos2 = cs * cs, sin2 = sn * sn;
                    A_ = (1.0f + 2.0f * e) * cos2 + sin2 + sd;
                    B_ = (1.0f + 2.0f * e) * sin2 + cos2 + sd;
                    hs = 2.0f * e * (2.0f * sn * cs);   // 2 eps sin(2 theta)
                }
                const float Q = pxxs + pzzs;
                A_u = A_ * u;
                B_u = B_ * u;
                H_u = hs * u;
                QX_u = Q * Cx * u;
                QZ_u = Q * Cz * u;
            };
            if (in0) cell(px.x, pz.x, pxx.x, pzz.x, e2v.x, d2v.x, u2.x, cs2.x, sn2.x, av.x, bv.x, hv.x, qxv.x, qzv.x);
            if (in1) cell(px.y, pz.y, pxx.y, pzz.y, e2v.y, d2v.y, u2.y, cs2.y, sn2.y, av.y, bv.y, hv.y, qxv.y, qzv.y);
        }
        const int q = qz * kAnQX + qx;
        *reinterpret_cast<float2*>(AUs + q) = av;
        *reinterpret_cast<float2*>(BUs + q) = bv;
        *reinterpret_cast<float2*>(QXs + q) = qxv;
        *reinterpret_cast<float2*>(QZs + q) = qzv;
        if (TTI) *reinterpret_cast<float2*>(HUs + q) = hv;
    }
    __syncthreads();

    // 3. the update of the tile's cells, by pairs of x-adjacent cells:
    //    new = D (2 U - D U_prev + kappa (dxx AU + dzz BU - dxz HU - dx QCxU - dz QCzU))
    //    (each thread's U, kappa and U_prev loaded before any of its arithmetic)
    constexpr int TXP = kAnTX / 2;
    constexpr int NUPD = kAnTZ * TXP / kAnThreads;      // pairs per thread
    static_assert(kAnTZ * TXP % kAnThreads == 0, "whole pairs per thread");
    float2 ucv[NUPD], kvv[NUPD], pvv[NUPD];
#pragma unroll
    for (int it = 0; it < NUPD; it++) {
        const int i = tid + it * kAnThreads;
        const int z = z0 + i / TXP, x = x0 + (i % TXP) * 2;
        const bool zin = z >= 4 && z < g.nz - 4;
        ucv[it] = kvv[it] = pvv[it] = make_float2(0.f, 0.f);
        if (zin && x + 1 >= 4 && x < g.nx - 4) {
            const long long m = (long long)z * g.P + x;
            const long long o = (long long)b * g.stride + m;
            ucv[it] = *reinterpret_cast<const float2*>(PAM_CHK(a.ub + o, a.ub, fbytes, 8, 95));
            kvv[it] = *reinterpret_cast<const float2*>(PAM_CHK(kap + m, kap, mbytes, 8, 93));
            pvv[it] = *reinterpret_cast<const float2*>(PAM_CHK(nxt + o, nxt, fbytes, 8, 96));
        }
    }
#pragma unroll
    for (int it = 0; it < NUPD; it++) {
        const int i = tid + it * kAnThreads;
        const int tz = i / TXP, tx = (i % TXP) * 2;
        const int z = z0 + tz, x = x0 + tx;
        const bool zin = z >= 4 && z < g.nz - 4;
        const bool in0 = zin && x >= 4 && x < g.nx - 4, in1 = zin && x + 1 >= 4 && x + 1 < g.nx - 4;
        if (!in0 && !in1) continue;
        const int q = (tz + 4) * kAnQX + (tx + 4);
        constexpr int s = kAnQX;
        auto L = [&](const float* f, int off) { return *reinterpret_cast<const float2*>(f + q + off); };
        float2 op;
        {
            const float2 A0 = L(AUs, -4), A1 = L(AUs, -2), A2 = L(AUs, 0), A3 = L(AUs, 2), A4 = L(AUs, 4);
            const float2 dxx = an_d2(A2, make_float2(A2.y, A3.x), make_float2(A1.y, A2.x), A3, A1,
                                     make_float2(A3.y, A4.x), make_float2(A0.y, A1.x), A4, A0, a.inv_dx2);
            const float2 dzz = an_d2(L(BUs, 0), L(BUs, s), L(BUs, -s), L(BUs, 2 * s), L(BUs, -2 * s), L(BUs, 3 * s),
                                     L(BUs, -3 * s), L(BUs, 4 * s), L(BUs, -4 * s), a.inv_dz2);
            op = padd2(dxx, dzz);
        }
        if (TTI) {
            // the factorised cross derivative (cpp/Migration.cu:906-928) of HU, per
            // pair: for each az the rows +az and -az (columns -4 .. +5 around the
            // pair, five aligned 8-byte loads each) feed the sums of all four ax,
            // in the order of sum_ax a_ax sum_az a_az (...)
            const float aa[5] = {0.f, PAM_A1, PAM_A2, PAM_A3, PAM_A4};
            float2 tax[5] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                             make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int az = 1; az <= 4; az++) {
                float vp[10], vm[10];
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    const float2 hp = L(HUs, az * s - 4 + 2 * k), hm = L(HUs, -az * s - 4 + 2 * k);
                    vp[2 * k] = hp.x; vp[2 * k + 1] = hp.y;
                    vm[2 * k] = hm.x; vm[2 * k + 1] = hm.y;
                }
#pragma unroll
                for (int ax = 1; ax <= 4; ax++) {
                    // H(dz, dx) of the pair = (v[4 + dx], v[5 + dx]) of row dz
                    const float2 hpa = make_float2(vp[4 + ax], vp[5 + ax]), hma = make_float2(vm[4 + ax], vm[5 + ax]);
                    const float2 hpb = make_float2(vp[4 - ax], vp[5 - ax]), hmb = make_float2(vm[4 - ax], vm[5 - ax]);
                    const float2 comb = padd2(fsub2(hpa, hma), fsub2(hmb, hpb));
                    tax[ax] = pfma2(bc2(aa[az]), comb, tax[ax]);
                }
            }
            float2 dxz = make_float2(0.f, 0.f);
#pragma unroll
            for (int ax = 1; ax <= 4; ax++) dxz = pfma2(bc2(aa[ax]), tax[ax], dxz);
            op = fsub2(op, pmul2(dxz, bc2(a.inv_dx * a.inv_dz)));
        }
        {
            const float2 X0 = L(QXs, -4), X1 = L(QXs, -2), X2 = L(QXs, 0), X3 = L(QXs, 2), X4 = L(QXs, 4);
            op = fsub2(op, an_d1(make_float2(X2.y, X3.x), make_float2(X1.y, X2.x), X3, X1, make_float2(X3.y, X4.x),
                                 make_float2(X0.y, X1.x), X4, X0, a.inv_dx));
            op = fsub2(op, an_d1(L(QZs, s), L(QZs, -s), L(QZs, 2 * s), L(QZs, -2 * s), L(QZs, 3 * s),
                                 L(QZs, -3 * s), L(QZs, 4 * s), L(QZs, -4 * s), a.inv_dz));
        }
        const long long o = (long long)b * g.stride + (long long)z * g.P + x;
        const float2 uc = ucv[it], kv = kvv[it];
        float2 prev = pvv[it];
        if (out_damped) prev = make_float2(damp_apply(g, z, x, prev.x), damp_apply(g, z, x + 1, prev.y));
        float2 out = pfma2(kv, op, fsub2(padd2(uc, uc), prev));
        if (out_damped) out = make_float2(damp_apply(g, z, x, out.x), damp_apply(g, z, x + 1, out.y));
        if (in0 && in1) {
            *reinterpret_cast<float2*>(PAM_CHK(nxt + o, nxt, fbytes, 8, 96)) = out;
        } else {
            if (in0) *PAM_CHK(nxt + o, nxt, fbytes, 4, 96) = out.x;
            if (in1) *PAM_CHK(nxt + o + 1, nxt, fbytes, 4, 96) = out.y;
        }
    }
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

// The exact adjoint runs on the scaled variable w = kappa D lambda.  With the
// forward recursion U(t+1) = D (2 U(t) - D U(t-1) + kappa L U(t)) + f(t+1),
// the adjoint lambda(t) = 2 D lambda(t+1) + L(kappa D lambda(t+1))
// - D^2 lambda(t+2) + D R^T r(t) becomes
//   w(t) = D (2 w(t+1) - D w(t+2) + kappa L w(t+1)) + kappa D^2 R^T r(t),
// the forward recursion itself (the stepping kernel, no source) plus this
// receiver injection.  data holds the residual r = dcal - dobs.
__global__ void inject_adjoint_kernel(float* __restrict__ w, const float* __restrict__ data,
                                      const int* __restrict__ rz, const int* __restrict__ rx, int nrec, int B, int it,
                                      int nt_data, int per_shot, const float* __restrict__ kap, GridDims g)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nrec * B) return;
    const int r = (int)(i % nrec);
    const int b = (int)(i / nrec);
    const long long ri = per_shot ? (long long)b * nrec + r : r;
    const int z = rz[ri], x = rx[ri];
    const long long c = (long long)z * g.P + x;
    const float v = damp_apply(g, z, x, damp_apply(g, z, x, data[((long long)b * nt_data + it) * nrec + r]));
    atomicAdd(w + (long long)b * g.stride + c, kap[c] * v);
}

// ---------------------------------------------------------------- multiparameter gradients

// Per-cell epsilon, delta (and theta) gradient increments of the reference's
// calculateGradientVTI / calculateGradientTTI (src/utils.py:1309-1463):
//   g_eps   += adj ((-2 cos^2 - dSd/deps) pxx - (2 sin^2 + dSd/deps) pzz + 2 sin 2th pxz)
//   g_delta += adj (-dSd/ddelta (pxx + pzz))
//   g_theta += adj ((2 eps sin 2th - dSd/dth) pxx + (-2 eps sin 2th - dSd/dth) pzz + 4 eps cos 2th pxz)
// (theta = 0 for VTI), Sd = num/den of the rotated gradient (h, q).  The
// reference evaluates in float64; here in float32 with (h, q) divided by
// max(|h|, |q|) first - every ratio is homogeneous of degree 0 in (h, q), so
// this is exact in exact arithmetic and keeps den = O(1) instead of |grad U|^4
// (which underflows float32).  Cells within 4 of the physical region's edge
// are skipped, as the reference's interior arrays do.  One thread per
// interior cell sums the batch's shots in registers (shots in order) and adds
// the sums to the running totals [nz][nx] once per step, like the imaging
// condition; the reference sums each shot over time first.  grid (nx, nz)
// blocks of 32 x 8.
__global__ void mp_grad_kernel(const float* __restrict__ P_, const float* __restrict__ ub, long long pstride,
                               const float* __restrict__ eps, const float* __restrict__ del,
                               const float* __restrict__ cth, const float* __restrict__ sth,
                               float* __restrict__ geps, float* __restrict__ gdel, float* __restrict__ gth,
                               GridDims g, int nzi, int nxi, int B, float inv_dx, float inv_dz, float inv_dx2,
                               float inv_dz2)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int zi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi < 4 || xi >= nxi - 4 || zi < 4 || zi >= nzi - 4) return;
    const long long c = (long long)(zi + g.N) * g.P + xi + g.N;
    const long long s = g.P;
    const bool tti = gth != nullptr;
    const float ct = tti ? cth[c] : 1.0f, st = tti ? sth[c] : 0.0f;
    const float e = eps[c], d = del[c];
    const float s2 = 2.0f * st * ct, c2 = ct * ct, sn2 = st * st;
    float sum_e = 0.0f, sum_d = 0.0f, sum_t = 0.0f;
    for (int b = 0; b < B; b++) {
        const float* U = P_ + (long long)b * pstride + c;
        const float pxx = (PAM_C0 * U[0] + PAM_C1 * (U[1] + U[-1]) + PAM_C2 * (U[2] + U[-2]) +
                           PAM_C3 * (U[3] + U[-3]) + PAM_C4 * (U[4] + U[-4])) * inv_dx2;
        const float pzz = (PAM_C0 * U[0] + PAM_C1 * (U[s] + U[-s]) + PAM_C2 * (U[2 * s] + U[-2 * s]) +
                           PAM_C3 * (U[3 * s] + U[-3 * s]) + PAM_C4 * (U[4 * s] + U[-4 * s])) * inv_dz2;
        const float px = (PAM_A1 * (U[1] - U[-1]) + PAM_A2 * (U[2] - U[-2]) + PAM_A3 * (U[3] - U[-3]) +
                          PAM_A4 * (U[4] - U[-4])) * inv_dx;
        const float pz = (PAM_A1 * (U[s] - U[-s]) + PAM_A2 * (U[2 * s] - U[-2 * s]) +
                          PAM_A3 * (U[3 * s] - U[-3 * s]) + PAM_A4 * (U[4 * s] - U[-4 * s])) * inv_dz;
        float pxz = 0.0f;
        if (tti) {
            const float a[4] = {PAM_A1, PAM_A2, PAM_A3, PAM_A4};
#pragma unroll
            for (int m = 1; m <= 4; m++) {
                float t = 0.0f;
#pragma unroll
                for (int n = 1; n <= 4; n++)
                    t += a[n - 1] * (U[n * s + m] - U[-n * s + m] + U[-n * s - m] - U[n * s - m]);
                pxz += a[m - 1] * t;
            }
            pxz *= inv_dx * inv_dz;
        }
        float h = px * ct - pz * st, q = px * st + pz * ct;
        const float mh = fmaxf(fabsf(h), fabsf(q));
        float dSe = 0.0f, dSdl = 0.0f, dSt = 0.0f;
        if (mh > 0.0f) {
            h /= mh;
            q /= mh;
            const float h2 = h * h, q2 = q * q, t = h2 * q2, h4 = h2 * h2, q4 = q2 * q2;
            const float num = -2.0f * (e - d) * t;
            const float den = (1.0f + 2.0f * e) * h4 + q4 + 2.0f * (1.0f + d) * t;
            const float r = 1.0f / (den * den);
            dSe = (-2.0f * t * den - num * 2.0f * h4) * r;
            dSdl = (2.0f * t * den - num * 2.0f * t) * r;
            if (tti) {
                const float w = -2.0f * h * q * q2 + 2.0f * h * h2 * q;
                const float dnum = -2.0f * (e - d) * w;
                const float dden =
                    -4.0f * (1.0f + 2.0f * e) * h * h2 * q + 4.0f * h * q * q2 + 2.0f * (1.0f + d) * w;
                dSt = (dnum * den - num * dden) * r;
            }
        }
        const float a = ub[(long long)b * g.stride + c];
        sum_e += a * (-(2.0f * c2 + dSe) * pxx - (2.0f * sn2 + dSe) * pzz + 2.0f * s2 * pxz);
        sum_d += a * (-dSdl * (pxx + pzz));
        if (tti) {
            const float cos2 = c2 - sn2;
            sum_t += a * ((2.0f * e * s2 - dSt) * pxx + (-2.0f * e * s2 - dSt) * pzz + 4.0f * e * cos2 * pxz);
        }
    }
    const long long o = (long long)zi * nxi + xi;
    geps[o] += sum_e;
    gdel[o] += sum_d;
    if (tti) gth[o] += sum_t;
}

// ---------------------------------------------------------------- boundary saving

// The saved band: the outer four rows and columns of the physical region
// (src/Migration.py:288-298), as a flat list - rows [N, N+4) and
// [N+nz-4, N+nz) over the nx physical columns, then columns [N, N+4) and
// [N+nx-4, N+nx) over the nz-8 rows in between.  Four cells is the stencil
// half-width, so the reverse steps of the cells inside the band read only the
// band and themselves.
__host__ __device__ inline long long band_cells(int nzi, int nxi) { return 8LL * nxi + 8LL * (nzi - 8); }

__device__ __forceinline__ void band_cell(long long i, int N, int nzi, int nxi, int& z, int& x) {
    const long long rows = 4LL * nxi;
    if (i < rows) { z = N + (int)(i / nxi); x = N + (int)(i % nxi); return; }
    i -= rows;
    if (i < rows) { z = N + nzi - 4 + (int)(i / nxi); x = N + (int)(i % nxi); return; }
    i -= rows;
    const long long side = 4LL * (nzi - 8);
    if (i < side) { z = N + 4 + (int)(i / 4); x = N + (int)(i % 4); return; }
    i -= side;
    z = N + 4 + (int)(i / 4);
    x = N + nxi - 4 + (int)(i % 4);
}

constexpr int kBandChunk = 256;   // cells per scale (one block)

template <typename T>
__device__ __forceinline__ T band_pack(float v);
template <>
__device__ __forceinline__ float band_pack<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 band_pack<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ __half band_pack<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float band_unpack(float v) { return v; }
__device__ __forceinline__ float band_unpack(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float band_unpack(__half v) { return __half2float(v); }

// Save the band of every shot of `field` into dst[b][nband]; the compressed
// formats keep one scale per chunk of kBandChunk cells (|max| of the chunk
// mapped to `target`), stored as its inverse in inv_scale[b][nchunk].
// grid (nchunk, B), block kBandChunk.
template <typename T>
__global__ void __launch_bounds__(kBandChunk)
band_save_kernel(const float* __restrict__ field, T* __restrict__ dst, float* __restrict__ inv_scale, GridDims g,
                 int nzi, int nxi, float target)
{
    __shared__ float red[kBandChunk / 32];
    const long long nb = band_cells(nzi, nxi);
    const int nchunk = (int)((nb + kBandChunk - 1) / kBandChunk);
    const int b = blockIdx.y;
    const long long i = (long long)blockIdx.x * kBandChunk + threadIdx.x;
    float v = 0.0f;
    if (i < nb) {
        int z, x;
        band_cell(i, g.N, nzi, nxi, z, x);
        v = field[(long long)b * g.stride + (long long)z * g.P + x];
    }
    float s = 1.0f;
    if (target > 0.0f) {
        float m = fabsf(v);
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
        __syncthreads();
        m = red[0];
        for (int w = 1; w < kBandChunk / 32; w++) m = fmaxf(m, red[w]);
        // a chunk of values below 1e-30 is stored unscaled (and flushes to
        // zero in FP16): scaling it up could overflow target / m
        s = m > 1e-30f ? target / m : 1.0f;
        if (threadIdx.x == 0) inv_scale[(long long)b * nchunk + blockIdx.x] = 1.0f / s;
    }
    if (i < nb) dst[(long long)b * nb + i] = band_pack<T>(v * s);
}

// Write a saved band back into `field` (grid and block as band_save_kernel).
template <typename T>
__global__ void __launch_bounds__(kBandChunk)
band_restore_kernel(const T* __restrict__ src, const float* __restrict__ inv_scale, float* __restrict__ field,
                    GridDims g, int nzi, int nxi, int scaled)
{
    const long long nb = band_cells(nzi, nxi);
    const int nchunk = (int)((nb + kBandChunk - 1) / kBandChunk);
    const int b = blockIdx.y;
    const long long i = (long long)blockIdx.x * kBandChunk + threadIdx.x;
    if (i >= nb) return;
    int z, x;
    band_cell(i, g.N, nzi, nxi, z, x);
    float v = band_unpack(src[(long long)b * nb + i]);
    if (scaled) v *= inv_scale[(long long)b * nchunk + blockIdx.x];
    field[(long long)b * g.stride + (long long)z * g.P + x] = v;
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
        inv = m > 1e-30f ? target / m : 1.0f;   // below 1e-30 unscaled: target / m could overflow
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
        sc = m > 1e-30f ? m / target : 1.0f;
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
