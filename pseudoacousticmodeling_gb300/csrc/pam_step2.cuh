// Two time steps per launch ("temporal blocking") of the acoustic scheme with
// Cerjan damping, for sm_103a.
//
// One launch reads U(t-1) and U(t) and writes U(t+1) and U(t+2): 16 B of
// field traffic per cell and shot for two steps instead of 24 B for two
// launches of step_kernel.  Each warp marches one z segment of one 128-column
// tile of one shot (as in step_kernel) and runs two stages four rows apart:
//   stage 1 computes U(t+1) at row r from the nine-row register window of
//           U(t) (rows r-4 .. r+4) and feeds it into a second window;
//   stage 2 computes U(t+2) at row r-4 from that window of U(t+1)
//           (rows r-8 .. r), U(t) at row r-4 (the oldest row of the first
//           window) and kappa at row r-4 (still in the ring).
// Stage 2 needs U(t+1) four columns beyond the columns it writes, so tiles
// overlap: a tile covers 128 columns from 120 * tile, lanes 0 and 31 compute
// stage 1 only (the neighbours' halo), and lanes 1..30 write both stages
// (120 columns).  Stage 2 also needs U(t+1) four rows above and below the
// segment, so stage 1 runs over the segment plus four rows on each side
// (computed, not stored).  U(t+1) values outside the update region
// [4, nz-4) x [4, nx-4) are held at zero, as the stored field is.
// The arithmetic of each stage is that of step_kernel<kAcoustic, kCerjan>
// operation for operation (packed FP32 pairs as inline PTX, the reference's
// coefficient order, damping of U(t-1) deferred to its read), so a launch
// gives bitwise the fields of two one-step launches.
#pragma once
#include "pam_kernels.cuh"

namespace pam {

constexpr int kStep2Cols = 120;        // columns a tile writes (lanes 1..30)
constexpr int kStep2RingA = 4;         // ring slots of U(t) leading row + U(t-1) row
constexpr int kStep2RingK = 8;         // ring slots of kappa rows (stage 2 reads them 4 rows late)
constexpr int kStep2SlotA = 32 + 2 + 32;   // U(t) leading row, its two x halo quads, U(t-1)
constexpr int kStep2Ahead = 2;         // rows in flight ahead of stage 1
static_assert(kStep2Ahead + 1 <= kStep2RingA, "ring too small for the prefetch distance");
static_assert(kStep2Ahead + 5 <= kStep2RingK, "kappa ring too small for the stage-2 lag");

__host__ __device__ constexpr int step2_warp_quads() {
    return kStep2RingA * kStep2SlotA + kStep2RingK * 32 + 2 * 34 + 2 * 32;
}
__host__ __device__ constexpr int step2_smem_bytes() { return kWarpsPerBlock * step2_warp_quads() * 16; }

// One acoustic update of a quad (cells 0..3): U_new = D (2 U - D U_prev +
// kappa (pxx + pzz)) with the operand order of step_kernel<kAcoustic, *>.
__device__ __forceinline__ void acoustic_quad(const float4& left, const float4& center, const float4& right,
                                              const float4& q0, const float4& q1, const float4& q2,
                                              const float4& q3, const float4& q5, const float4& q6,
                                              const float4& q7, const float4& q8, const float4& prev,
                                              const float4& kap, const float* cxf, float cz, float inv_dx2,
                                              float inv_dz2, float out[4]) {
    const float2 P0 = make_float2(left.x, left.y), P1 = make_float2(left.z, left.w);
    const float2 P2 = make_float2(center.x, center.y), P3 = make_float2(center.z, center.w);
    const float2 P4 = make_float2(right.x, right.y), P5 = make_float2(right.z, right.w);
    const float2 O0 = make_float2(left.y, left.z), O1 = make_float2(left.w, center.x);
    const float2 O2 = make_float2(center.y, center.z), O3 = make_float2(center.w, right.x);
    const float2 O4 = make_float2(right.y, right.z);
    float2 pxx[2], pzz[2];
    pxx[0] = d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, inv_dx2);
    pxx[1] = d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, inv_dx2);
    pzz[0] = d2_pair(lo2(center), lo2(q5), lo2(q3), lo2(q6), lo2(q2), lo2(q7), lo2(q1), lo2(q8), lo2(q0), inv_dz2);
    pzz[1] = d2_pair(hi2(center), hi2(q5), hi2(q3), hi2(q6), hi2(q2), hi2(q7), hi2(q1), hi2(q8), hi2(q0), inv_dz2);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const float2 uc = q == 0 ? lo2(center) : hi2(center);
        const float2 k = q == 0 ? lo2(kap) : hi2(kap);
        const float2 cxq = make_float2(cxf[2 * q], cxf[2 * q + 1]);
        const float2 czq = make_float2(cz, cz);
        const float2 p = pmul2(pmul2(q == 0 ? lo2(prev) : hi2(prev), cxq), czq);
        const float2 base = fsub2(padd2(uc, uc), p);
        float2 o = pfma2(k, padd2(pxx[q], pzz[q]), base);
        o = pmul2(pmul2(o, cxq), czq);
        out[2 * q] = o.x;
        out[2 * q + 1] = o.y;
    }
}

// Args: cur = U(t), prev = U(t-1) (never aliased with the outputs), nxt =
// U(t+1), nxt2 = U(t+2); src_amp / src_amp2 the wavelet samples t+1 / t+2;
// ntiles / nseg / H describe this kernel's own tiling (120-column tiles).
__global__ void __launch_bounds__(128, 3) step2_kernel(const StepArgs a)
{
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* __restrict__ ringA = smem4 + wib * step2_warp_quads();
    float4* __restrict__ ringK = ringA + kStep2RingA * kStep2SlotA;
    float4* __restrict__ xb1 = ringK + kStep2RingK * 32;   // [2][34]: U(t) centre row with its halo quads
    float4* __restrict__ xb2 = xb1 + 2 * 34;               // [2][32]: U(t+1) centre row

    const int warp = blockIdx.x * kWarpsPerBlock + wib;
    const int shot = warp % a.B;
    const int rest = warp / a.B;
    const int tile = rest % a.ntiles;
    const int seg = rest / a.ntiles;
    if (seg >= a.nseg) return;   // uniform per warp

    const int x0 = tile * kStep2Cols + lane * 4;
    const int z0 = 4 + seg * a.H;
    const int z1 = min(z0 + a.H, a.nz - 4);
    const int rs = z0 - 4, re = z1 + 4;        // stage-1 rows
    const int P = a.P;
    const int zmax = a.nz - 1;
    const long long so = (long long)shot * a.shot_stride + x0;
    const float* __restrict__ cur = a.cur + so;
    const float* __restrict__ prv = a.prev + so;
    float* __restrict__ out1 = a.nxt + so;
    float* __restrict__ out2 = a.nxt2 + so;
    const bool owner = lane >= 1 && lane <= 30;
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long mbytes = (long long)a.nz * a.P * 4;
    const int sz = *PAM_CHK(&a.src_z[shot], a.src_z, a.B * 4, 4, 70);
    const int sx = *PAM_CHK(&a.src_x[shot], a.src_x, a.B * 4, 4, 70);

    // columns of this quad inside the update region, and their Cerjan factors
    bool colin[4];
    float cxf[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + j;
        colin[j] = x >= 4 && x < a.nx - 4;
        float f = 1.0f;
        if (x < a.N) f = *PAM_CHK(&a.cerjan[x], a.cerjan, a.N * 4, 4, 71);
        if (x >= a.nx - a.N && x < a.nx) f = f * *PAM_CHK(&a.cerjan[a.nx - 1 - x], a.cerjan, a.N * 4, 4, 71);
        cxf[j] = f;
    }
    const bool allin = colin[0] && colin[1] && colin[2] && colin[3];
    auto czf = [&](int r) {
        float c = 1.0f;
        if (r < a.N) c = *PAM_CHK(&a.cerjan[r], a.cerjan, a.N * 4, 4, 72);
        if (r >= a.nz - a.N) c = c * *PAM_CHK(&a.cerjan[a.nz - 1 - r], a.cerjan, a.N * 4, 4, 72);
        return c;
    };

    // ring loads for stage-1 row rr: U(t) row rr+4 (every lane) with the x
    // halo quads of U(t) row rr (lane 0: columns x0-4, lane 31: x0+4; tile 0
    // has no left halo, its columns 0..3 are held at zero), U(t-1) and kappa
    // at row rr (every lane: the halo lanes compute stage 1 too)
    auto issue = [&](int rr) {
        float4* sa = ringA + (rr & (kStep2RingA - 1)) * kStep2SlotA;
        const long long rl = (long long)min(rr, zmax) * P;
        cp_async16(sa + lane, PAM_CHK(cur + (long long)min(rr + 4, zmax) * P, a.cur, fbytes, 16, 73));
        if ((lane == 0 && tile > 0) || lane == 31)
            cp_async16(sa + 32 + (lane == 0 ? 0 : 1), PAM_CHK(cur + rl + (lane == 0 ? -4 : 4), a.cur, fbytes, 16, 74));
        cp_async16(sa + 34 + lane, PAM_CHK(prv + rl, a.prev, fbytes, 16, 75));
        cp_async16(ringK + (rr & (kStep2RingK - 1)) * 32 + lane, PAM_CHK(a.kap + x0 + rl, a.kap, mbytes, 16, 76));
        cp_async_commit();
    };

    float4 w[9], v[9];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        w[i] = ldg4(PAM_CHK(cur + (long long)max(min(rs - 4 + i, zmax), 0) * P, a.cur, fbytes, 16, 77));
        v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < kStep2Ahead; i++) issue(rs + i);

    for (int r = rs; r < re; r++) {
        issue(r + kStep2Ahead);
        cp_async_wait<kStep2Ahead>();
        const float4* sa = ringA + (r & (kStep2RingA - 1)) * kStep2SlotA;
        w[8] = sa[lane];

        // ---- stage 1: U(t+1) at row r (zero outside the update region)
        {
            float4* xb = xb1 + (r & 1) * 34;
            xb[lane + 1] = w[4];
            if (lane == 0) xb[0] = sa[32];
            if (lane == 31) xb[33] = sa[33];
            __syncwarp();
            const float4 left = xb[lane], right = xb[lane + 2];
            const float4 prev = sa[34 + lane];
            const float4 kap = ringK[(r & (kStep2RingK - 1)) * 32 + lane];
            float o[4];
            acoustic_quad(left, w[4], right, w[0], w[1], w[2], w[3], w[5], w[6], w[7], w[8], prev, kap, cxf, czf(r),
                          a.inv_dx2, a.inv_dz2, o);
            if (r == sz) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j == sx) o[j] += a.src_amp;
            }
            const bool rowin = r >= 4 && r < a.nz - 4;
#pragma unroll
            for (int j = 0; j < 4; j++) o[j] = (rowin && colin[j]) ? o[j] : 0.0f;
            v[8] = make_float4(o[0], o[1], o[2], o[3]);
            if (owner && r >= z0 && r < z1) {
                const long long ro = (long long)r * P;
                if (allin) {
                    *reinterpret_cast<float4*>(PAM_CHK(out1 + ro, a.nxt, fbytes, 16, 78)) = v[8];
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (colin[j]) *PAM_CHK(&out1[ro + j], a.nxt, fbytes, 4, 78) = o[j];
                }
            }
        }

        // ---- stage 2: U(t+2) at row r - 4, once the window holds U(t+1) rows r-8 .. r
        if (r >= z0 + 4) {
            const int r2 = r - 4;
            float4* xb = xb2 + (r & 1) * 32;
            xb[lane] = v[4];
            __syncwarp();
            const float4 left = xb[(lane + 31) & 31], right = xb[(lane + 1) & 31];
            const float4 kap = ringK[(r2 & (kStep2RingK - 1)) * 32 + lane];
            float o[4];
            acoustic_quad(left, v[4], right, v[0], v[1], v[2], v[3], v[5], v[6], v[7], v[8], w[0], kap, cxf,
                          czf(r2), a.inv_dx2, a.inv_dz2, o);
            if (r2 == sz) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j == sx) o[j] += a.src_amp2;
            }
            if (owner) {
                const long long ro = (long long)r2 * P;
                if (allin) {
                    *reinterpret_cast<float4*>(PAM_CHK(out2 + ro, a.nxt2, fbytes, 16, 79)) =
                        make_float4(o[0], o[1], o[2], o[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (colin[j]) *PAM_CHK(&out2[ro + j], a.nxt2, fbytes, 4, 79) = o[j];
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            w[i] = w[i + 1];
            v[i] = v[i + 1];
        }
    }
    cp_async_wait<0>();
}

}  // namespace pam
