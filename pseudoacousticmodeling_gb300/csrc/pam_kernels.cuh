// Device code of the finite-difference hot path, written for sm_103a (GB300).
//
// Layout in HBM (one shot batch):
//   wavefields   float [B][nz][P]   nz = nz_abc, P = row pitch (multiple of 32
//                                   floats, >= the last tile's reach); cells
//                                   outside [4,nz-4) x [4,nx-4) stay zero
//   models       float [nz][P]      kappa = vp^2 dt^2 (+ eps, delta, cos/sin
//                                   theta), shared by every shot of the batch
//   CPML x strip float2 [B][nz][2N] (d psi_x, d psi_x + zeta_x) per step
//   CPML z strip float2 [B][2N][P]  (d psi_z, d psi_z + zeta_z) per step
//
// Stepping kernel ("warp march"): one warp owns one shot, one 128-column tile
// (32 lanes x float4) and one z segment.  It walks down its segment keeping
// the nine rows z-4..z+4 of U(t) (plus one prefetched row) in a rotating
// register queue; x neighbours come from the adjacent lanes through shuffles.
// Lanes 0 and 31 only feed neighbours (their quads are the tile's x halo), so
// a tile writes 120 columns.  No shared memory and no block barriers: every
// warp is independent, and the grid is ordered shot-fastest so that the
// model rows a tile needs are read from HBM once and from L2 by the other
// shots.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pam_types.h"

namespace pam {


// 8th-order coefficients.  Literal values of the reference kernels
// (cpp/Modeling.cu:500-504, 560-563); as floats they equal the exact
// fractions -1435/504, 8/5, -1/5, 8/315, -1/560 and 4/5, -1/5, 4/105, -1/280.
__device__ __constant__ static const float kC0 = -2.847222222222f;
__device__ __constant__ static const float kC1 = 1.6f;
__device__ __constant__ static const float kC2 = -0.2f;
__device__ __constant__ static const float kC3 = 0.02539682539f;
__device__ __constant__ static const float kC4 = -0.00178571428f;
__device__ __constant__ static const float kA1 = 0.8f;
__device__ __constant__ static const float kA2 = -0.2f;
__device__ __constant__ static const float kA3 = 0.03809523809f;
__device__ __constant__ static const float kA4 = -0.00357142857f;



__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ float4 shfl_up4(float4 v) {
    float4 r;
    r.x = __shfl_up_sync(0xffffffffu, v.x, 1);
    r.y = __shfl_up_sync(0xffffffffu, v.y, 1);
    r.z = __shfl_up_sync(0xffffffffu, v.z, 1);
    r.w = __shfl_up_sync(0xffffffffu, v.w, 1);
    return r;
}
__device__ __forceinline__ float4 shfl_dn4(float4 v) {
    float4 r;
    r.x = __shfl_down_sync(0xffffffffu, v.x, 1);
    r.y = __shfl_down_sync(0xffffffffu, v.y, 1);
    r.z = __shfl_down_sync(0xffffffffu, v.z, 1);
    r.w = __shfl_down_sync(0xffffffffu, v.w, 1);
    return r;
}
__device__ __forceinline__ float get(const float4& v, int j) {
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set(float4& v, int j, float s) {
    if (j == 0) v.x = s; else if (j == 1) v.y = s; else if (j == 2) v.z = s; else v.w = s;
}

// Second derivative along z of element j from the nine queued rows.
#define PAM_D2Z(j, Q)                                                                              \
    (kC0 * get(Q##4, j) + kC1 * (get(Q##5, j) + get(Q##3, j)) + kC2 * (get(Q##6, j) + get(Q##2, j)) + \
     kC3 * (get(Q##7, j) + get(Q##1, j)) + kC4 * (get(Q##8, j) + get(Q##0, j)))
#define PAM_D1Z(j, Q)                                                                     \
    (kA1 * (get(Q##5, j) - get(Q##3, j)) + kA2 * (get(Q##6, j) - get(Q##2, j)) +          \
     kA3 * (get(Q##7, j) - get(Q##1, j)) + kA4 * (get(Q##8, j) - get(Q##0, j)))

// Pseudo-acoustic Sd term (cpp/Modeling.cu:605-611): on only when |den| > 1e-12.
__device__ __forceinline__ float sd_term(float e, float d, float px, float pz) {
    const float px2 = px * px, pz2 = pz * pz;
    const float num = -2.0f * (e - d) * px2 * pz2;
    const float den = (1.0f + 2.0f * e) * (px2 * px2) + pz2 * pz2 + 2.0f * (1.0f + d) * px2 * pz2;
    return fabsf(den) > 1e-12f ? __fdiv_rn(num, den) : 0.0f;
}

// ---------------------------------------------------------------------------
// One forward time step for a shot batch (see the file header).
template <int APPROX, int BC>
__global__ void __launch_bounds__(128) step_kernel(const StepArgs a)
{
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int shot = warp % a.B;
    const int rest = warp / a.B;
    const int tile = rest % a.ntiles;
    const int seg = rest / a.ntiles;
    if (seg >= a.nseg) return;   // uniform per warp

    const int x0 = tile * kTileOut + lane * 4;          // first column of this lane's quad
    const int z0 = 4 + seg * a.H;
    const int z1 = min(z0 + a.H, a.nz - 4);
    const int P = a.P;
    const float* __restrict__ cur = a.cur + (long long)shot * a.shot_stride + x0;
    float* __restrict__ nxt = a.nxt + (long long)shot * a.shot_stride + x0;
    const bool writer = (lane >= 1 && lane <= 30);
    const int zmax = a.nz - 1;

    // source position of this shot, folded into the new field
    const int sz = a.src_z[shot];
    const int sx = a.src_x[shot];

    // Cerjan factors along x for the four columns of this quad (x first, then z,
    // the order of cpp/Modeling.cu:535-550).
    float4 cx = make_float4(1.f, 1.f, 1.f, 1.f);
    if (BC == kCerjan) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int x = x0 + j;
            float f = 1.0f;
            if (x < a.N) f = a.cerjan[x];
            if (x >= a.nx - a.N && x < a.nx) f = f * a.cerjan[a.nx - 1 - x];
            set(cx, j, f);
        }
    }

    // register queue: rows r-4 .. r+5 of U(t) at the start of iteration r
    float4 q0 = ldg4(cur + (long long)(z0 - 4) * P);
    float4 q1 = ldg4(cur + (long long)(z0 - 3) * P);
    float4 q2 = ldg4(cur + (long long)(z0 - 2) * P);
    float4 q3 = ldg4(cur + (long long)(z0 - 1) * P);
    float4 q4 = ldg4(cur + (long long)(z0) * P);
    float4 q5 = ldg4(cur + (long long)min(z0 + 1, zmax) * P);
    float4 q6 = ldg4(cur + (long long)min(z0 + 2, zmax) * P);
    float4 q7 = ldg4(cur + (long long)min(z0 + 3, zmax) * P);
    float4 q8 = ldg4(cur + (long long)min(z0 + 4, zmax) * P);
    float4 q9 = ldg4(cur + (long long)min(z0 + 5, zmax) * P);

    auto row = [&](int r, float4& Q0, float4& Q1, float4& Q2, float4& Q3, float4& Q4, float4& Q5,
                   float4& Q6, float4& Q7, float4& Q8, float4& Q9) {
        // prefetch row r+6 of U(t) into the slot of row r-4 after this row is done
        const float4 center = Q4;
        const float4 left = shfl_up4(center);
        const float4 right = shfl_dn4(center);
        float w[12] = {left.x, left.y, left.z, left.w, center.x, center.y, center.z, center.w,
                       right.x, right.y, right.z, right.w};

        float4 pz4, pzz4;
        pz4.x = PAM_D1Z(0, Q); pz4.y = PAM_D1Z(1, Q); pz4.z = PAM_D1Z(2, Q); pz4.w = PAM_D1Z(3, Q);
        pzz4.x = PAM_D2Z(0, Q); pzz4.y = PAM_D2Z(1, Q); pzz4.z = PAM_D2Z(2, Q); pzz4.w = PAM_D2Z(3, Q);

        float pxz[4] = {0.f, 0.f, 0.f, 0.f};
        if (APPROX == kTTI) {
            const float4 pzl = shfl_up4(pz4);
            const float4 pzr = shfl_dn4(pz4);
            float v[12] = {pzl.x, pzl.y, pzl.z, pzl.w, pz4.x, pz4.y, pz4.z, pz4.w,
                           pzr.x, pzr.y, pzr.z, pzr.w};
#pragma unroll
            for (int j = 0; j < 4; j++)
                pxz[j] = (kA1 * (v[j + 5] - v[j + 3]) + kA2 * (v[j + 6] - v[j + 2]) +
                          kA3 * (v[j + 7] - v[j + 1]) + kA4 * (v[j + 8] - v[j])) *
                         (a.inv_dx * a.inv_dz);
        }

        // slot of row r-4 now free: fetch row r+6
        Q0 = ldg4(cur + (long long)min(r + 6, zmax) * P);

        if (writer) {
            const long long ro = (long long)r * P;
            float4 prev = *reinterpret_cast<const float4*>(nxt + ro);
            const float4 kap = ldg4(a.kap + x0 + ro);
            float4 e4, d4, c4, s4;
            if (APPROX != kAcoustic) { e4 = ldg4(a.eps + x0 + ro); d4 = ldg4(a.del + x0 + ro); }
            if (APPROX == kTTI) { c4 = ldg4(a.cth + x0 + ro); s4 = ldg4(a.sth + x0 + ro); }
            float cz = 1.0f;
            if (BC == kCerjan) {
                if (r < a.N) cz = a.cerjan[r];
                if (r >= a.nz - a.N) cz = cz * a.cerjan[a.nz - 1 - r];
            }
            const bool zstrip = (BC == kCPML) && (r < a.N || r >= a.nz - a.N);
            float4 out;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int x = x0 + j;
                const float pxx = (kC0 * w[j + 4] + kC1 * (w[j + 5] + w[j + 3]) + kC2 * (w[j + 6] + w[j + 2]) +
                                   kC3 * (w[j + 7] + w[j + 1]) + kC4 * (w[j + 8] + w[j])) * a.inv_dx2;
                const float pzz = get(pzz4, j) * a.inv_dz2;
                float p = get(prev, j);
                if (BC == kCerjan) p = (p * get(cx, j)) * cz;   // damping of U(t-1) deferred to here
                float gx = 0.f, hx = 0.f, gz = 0.f, hz = 0.f;
                if (BC == kCPML) {
                    if (x < a.N || (x >= a.nx - a.N && x < a.nx - 4)) {
                        const int c = x < a.N ? x : x - (a.nx - 2 * a.N);
                        const float2 t = a.xaux[(long long)shot * a.xaux_stride + (long long)r * (2 * a.N) + c];
                        gx = t.x; hx = t.y;
                    }
                    if (zstrip) {
                        const int rr = r < a.N ? r : r - (a.nz - 2 * a.N);
                        const float2 t = a.zaux[(long long)shot * a.zaux_stride + (long long)rr * P + x];
                        gz = t.x; hz = t.y;
                    }
                }
                const float uc = get(center, j);
                const float k = get(kap, j);
                float o;
                if (APPROX == kAcoustic) {
                    o = k * (pxx + pzz + hx + hz) + 2.0f * uc - p;
                } else {
                    float px = (kA1 * (w[j + 5] - w[j + 3]) + kA2 * (w[j + 6] - w[j + 2]) +
                                kA3 * (w[j + 7] - w[j + 1]) + kA4 * (w[j + 8] - w[j])) * a.inv_dx;
                    float pz = get(pz4, j) * a.inv_dz;
                    px += gx;
                    pz += gz;
                    const float pxxe = pxx + hx, pzze = pzz + hz;
                    const float e = get(e4, j), d = get(d4, j);
                    const float e2 = 1.0f + 2.0f * e;
                    if (APPROX == kVTI) {
                        const float sd = sd_term(e, d, px, pz);
                        o = 2.0f * uc - p + k * (e2 + sd) * pxxe + k * (1.0f + sd) * pzze;
                    } else {
                        const float c = get(c4, j), s = get(s4, j);
                        const float pxr = px * c - pz * s;
                        const float pzr = px * s + pz * c;
                        const float sd = sd_term(e, d, pxr, pzr);
                        const float c2 = c * c, s2 = s * s;
                        o = 2.0f * uc - p + k * (e2 * c2 + s2 + sd) * pxxe + k * (e2 * s2 + c2 + sd) * pzze -
                            2.0f * e * k * (2.0f * s * c) * pxz[j];
                    }
                }
                if (BC == kCerjan) o = (o * get(cx, j)) * cz;
                if (r == sz && x == sx) o += a.src_amp;
                set(out, j, o);
            }
            // store the columns inside the update region [4, nx-4)
            if (x0 + 3 < a.nx - 4) {
                *reinterpret_cast<float4*>(nxt + ro) = out;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j < a.nx - 4) nxt[ro + j] = get(out, j);
            }
        }
    };

    // Rotate the queue by renaming: ten calls per pass, each with the slots
    // shifted by one, so no register is moved.
    int r = z0;
    while (true) {
        row(r, q0, q1, q2, q3, q4, q5, q6, q7, q8, q9); if (++r >= z1) break;
        row(r, q1, q2, q3, q4, q5, q6, q7, q8, q9, q0); if (++r >= z1) break;
        row(r, q2, q3, q4, q5, q6, q7, q8, q9, q0, q1); if (++r >= z1) break;
        row(r, q3, q4, q5, q6, q7, q8, q9, q0, q1, q2); if (++r >= z1) break;
        row(r, q4, q5, q6, q7, q8, q9, q0, q1, q2, q3); if (++r >= z1) break;
        row(r, q5, q6, q7, q8, q9, q0, q1, q2, q3, q4); if (++r >= z1) break;
        row(r, q6, q7, q8, q9, q0, q1, q2, q3, q4, q5); if (++r >= z1) break;
        row(r, q7, q8, q9, q0, q1, q2, q3, q4, q5, q6); if (++r >= z1) break;
        row(r, q8, q9, q0, q1, q2, q3, q4, q5, q6, q7); if (++r >= z1) break;
        row(r, q9, q0, q1, q2, q3, q4, q5, q6, q7, q8); if (++r >= z1) break;
    }
}

// ---------------------------------------------------------------------------
// CPML memory variables (src/utils.py:242-377): psi = a psi + b dU, then
// zeta = a zeta + b (d2U + d psi_new), for every strip cell, and the terms the
// stepping kernel adds: (d psi_new, d psi_new + zeta_new).  psi and zeta are
// zero outside their strip, so each strip row (x) or strip column (z) is
// self-contained.

// x strips: one warp per (shot, row, side); z strips: one 128-thread block
// per (shot, side, 32-column slab).  Shared memory holds psi_new with four
// zero cells on each side.

__global__ void __launch_bounds__(128) cpml_x_kernel(const CpmlArgs a)
{
    __shared__ float sm[kCpmlMaxStrip + 8][kWarpsPerBlock];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const long long item = (long long)blockIdx.x * kWarpsPerBlock + wib;
    const int rows = a.nz - 8;
    const long long total = (long long)a.B * rows * 2;
    if (item >= total) return;
    const int side = (int)(item % 2);
    const int z = 4 + (int)((item / 2) % rows);
    const int shot = (int)(item / (2LL * rows));
    const int W = a.N - 4;                          // strip width
    const int xbeg = side == 0 ? 4 : a.nx - a.N;    // first strip column
    const int cbeg = side == 0 ? 4 : a.N;           // its index in the [2N] strip row
    const float* U = a.cur + (long long)shot * a.shot_stride + (long long)z * a.P;
    const long long so = (long long)shot * a.xs_stride + (long long)z * (2 * a.N);
    for (int i = lane; i < W + 8; i += 32) sm[i][wib] = 0.0f;
    __syncwarp();
    for (int i = lane; i < W; i += 32) {
        const int x = xbeg + i;
        const float px = (kA1 * (U[x + 1] - U[x - 1]) + kA2 * (U[x + 2] - U[x - 2]) +
                          kA3 * (U[x + 3] - U[x - 3]) + kA4 * (U[x + 4] - U[x - 4])) * a.inv_dx;
        const float2 ab = a.cxab[(long long)z * (2 * a.N) + cbeg + i];
        const long long o = so + cbeg + i;
        const float ps = ab.x * a.psix[o] + ab.y * px;
        a.psix[o] = ps;
        sm[i + 4][wib] = ps;
    }
    __syncwarp();
    for (int i = lane; i < W; i += 32) {
        const int x = xbeg + i;
        const float pxx = (kC0 * U[x] + kC1 * (U[x + 1] + U[x - 1]) + kC2 * (U[x + 2] + U[x - 2]) +
                           kC3 * (U[x + 3] + U[x - 3]) + kC4 * (U[x + 4] + U[x - 4])) * a.inv_dx2;
        const int k = i + 4;
        const float dps = (kA1 * (sm[k + 1][wib] - sm[k - 1][wib]) + kA2 * (sm[k + 2][wib] - sm[k - 2][wib]) +
                           kA3 * (sm[k + 3][wib] - sm[k - 3][wib]) + kA4 * (sm[k + 4][wib] - sm[k - 4][wib])) *
                          a.inv_dx;
        const float2 ab = a.cxab[(long long)z * (2 * a.N) + cbeg + i];
        const long long o = so + cbeg + i;
        const float ze = ab.x * a.zetax[o] + ab.y * (pxx + dps);
        a.zetax[o] = ze;
        a.xaux[o] = make_float2(dps, dps + ze);
    }
}

__global__ void __launch_bounds__(128) cpml_z_kernel(const CpmlArgs a)
{
    // block: 32 columns x 4 row groups; shared psi_new[W + 8][32]
    extern __shared__ float smz[];
    const int tx = threadIdx.x & 31;
    const int ty = threadIdx.x >> 5;
    const int nslab = (a.nx - 8 + 31) / 32;
    const long long item = blockIdx.x;
    const int slab = (int)(item % nslab);
    const int side = (int)((item / nslab) % 2);
    const int shot = (int)(item / (2LL * nslab));
    const int W = a.N - 4;
    const int x = 4 + slab * 32 + tx;
    const bool active = x < a.nx - 4;
    const int zbeg = side == 0 ? 4 : a.nz - a.N;
    const int rbeg = side == 0 ? 4 : a.N;
    const long long P = a.P;
    const float* U = a.cur + (long long)shot * a.shot_stride;
    const long long so = (long long)shot * a.zs_stride;
    for (int i = ty; i < W + 8; i += 4) smz[i * 32 + tx] = 0.0f;
    __syncthreads();
    if (active) {
        for (int i = ty; i < W; i += 4) {
            const int z = zbeg + i;
            const float* u = U + (long long)z * P + x;
            const float pz = (kA1 * (u[P] - u[-P]) + kA2 * (u[2 * P] - u[-2 * P]) + kA3 * (u[3 * P] - u[-3 * P]) +
                              kA4 * (u[4 * P] - u[-4 * P])) * a.inv_dz;
            const long long o = so + (long long)(rbeg + i) * P + x;
            const float2 ab = a.czab[(long long)(rbeg + i) * P + x];
            const float ps = ab.x * a.psiz[o] + ab.y * pz;
            a.psiz[o] = ps;
            smz[(i + 4) * 32 + tx] = ps;
        }
    }
    __syncthreads();
    if (active) {
        for (int i = ty; i < W; i += 4) {
            const int z = zbeg + i;
            const float* u = U + (long long)z * P + x;
            const float pzz = (kC0 * u[0] + kC1 * (u[P] + u[-P]) + kC2 * (u[2 * P] + u[-2 * P]) +
                               kC3 * (u[3 * P] + u[-3 * P]) + kC4 * (u[4 * P] + u[-4 * P])) * a.inv_dz2;
            const int k = i + 4;
            const float dps = (kA1 * (smz[(k + 1) * 32 + tx] - smz[(k - 1) * 32 + tx]) +
                               kA2 * (smz[(k + 2) * 32 + tx] - smz[(k - 2) * 32 + tx]) +
                               kA3 * (smz[(k + 3) * 32 + tx] - smz[(k - 3) * 32 + tx]) +
                               kA4 * (smz[(k + 4) * 32 + tx] - smz[(k - 4) * 32 + tx])) * a.inv_dz;
            const long long o = so + (long long)(rbeg + i) * P + x;
            const float2 ab = a.czab[(long long)(rbeg + i) * P + x];
            const float ze = ab.x * a.zetaz[o] + ab.y * (pzz + dps);
            a.zetaz[o] = ze;
            a.zaux[o] = make_float2(dps, dps + ze);
        }
    }
}

// ---------------------------------------------------------------------------
// Receiver recording (cpp/Modeling.cu:488-497): seis[b][t][r] = D * U(t) at
// the receiver cell, D the Cerjan factor there (1 for CPML and the interior).

__global__ void record_kernel(const RecordArgs a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)a.nrec * a.B) return;
    const int r = (int)(i % a.nrec);
    const int b = (int)(i / a.nrec);
    const long long ri = a.per_shot ? (long long)b * a.nrec + r : r;
    const int z = a.rz[ri], x = a.rx[ri];
    float v = a.cur[(long long)b * a.shot_stride + (long long)z * a.P + x];
    if (a.cerjan_on && z >= 4 && z < a.nz - 4 && x >= 4 && x < a.nx - 4) {
        if (x < a.N) v = v * a.cerjan[x];
        if (x >= a.nx - a.N) v = v * a.cerjan[a.nx - 1 - x];
        if (z < a.N) v = v * a.cerjan[z];
        if (z >= a.nz - a.N) v = v * a.cerjan[a.nz - 1 - z];
    }
    a.seis[((long long)b * a.nt_data + a.it) * a.nrec + r] = v;
}

// Writes the first wavelet sample at each shot's source cell (the injection
// of step 0, cpp/Modeling.cu:447); fields are zeroed beforehand.
// Source indices of the device entry point are not host-validated, so the
// kernel skips any cell outside the update region instead of writing it.
__global__ void inject_first_kernel(float* __restrict__ cur, const int* __restrict__ sz, const int* __restrict__ sx,
                                    float amp, int B, int P, long long shot_stride, int nz, int nx)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const int z = sz[b], x = sx[b];
    if (z < 4 || z >= nz - 4 || x < 4 || x >= nx - 4) return;
    cur[(long long)b * shot_stride + (long long)z * P + x] += amp;
}

}  // namespace pam
