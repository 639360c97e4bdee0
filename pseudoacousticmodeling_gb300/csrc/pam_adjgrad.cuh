// The exact adjoint step of the acoustic Cerjan scheme fused with the
// gradient and illumination sums of the same backward step (sm_103a).
//
// The backward sweep of the exact gradient advances the scaled adjoint
//   w(t) = D (2 w(t+1) - D w(t+2) + kappa L w(t+1))
// (the forward recursion, see inject_adjoint_kernel) and accumulates
//   G    += w(t+1) L U(t)    (kappa dJ/dkappa on the expanded grid)
//   ilum += U(t)^2           (source illumination)
// summed over the shots of the batch.  This kernel does both in one pass:
// each warp marches one z segment of one 128-column tile of one shot like
// step_kernel, with a second nine-row register window holding U(t), so
// w(t+1) and L U(t) meet in registers and U(t) is read once per step
// instead of once by the stepping kernel and again (with its halo) by a
// separate gradient kernel.
//
// The sum over shots: a block is four warps of the same tile and segment
// and four consecutive shots (shots are the fastest grid dimension).  Each
// row, the four warps put their products in shared memory (double-buffered
// by row parity, one block barrier per row), and warps 0 and 1 add the four
// values in a fixed order to the block's own row of a per-group partial sum
// ([shots / 4][nz][P]: every (group, cell) belongs to exactly one block, so
// there is no atomic and the result does not depend on scheduling).  The
// groups are added after the sweep (adjgrad_fold_kernel).  Batches whose
// size is not a multiple of four are padded with ghost shots that read shot
// B-1, contribute zero and store nothing.
#pragma once
#include "pam_kernels.cuh"

namespace pam {

constexpr int kAgRing = 4;                        // ring slots
constexpr int kAgAhead = 2;                       // rows in flight
constexpr int kAgSlot = 34 + 34 + 32 + 32;        // w lead + halo, U lead + halo, w(t+2), kappa
static_assert(kAgAhead + 1 <= kAgRing, "ring too small for the prefetch distance");

__host__ __device__ constexpr int adjgrad_warp_quads() { return kAgRing * kAgSlot + 2 * 34 + 2 * 34; }
__host__ __device__ constexpr int adjgrad_smem_bytes() {
    return (kWarpsPerBlock * adjgrad_warp_quads() + 2 * 2 * kWarpsPerBlock * 32) * 16;
}

struct AdjGradArgs {
    StepArgs s;            // the adjoint step: cur = w(t+1), nxt = w(t+2) in / w(t) out (in place)
    const float* U;        // U(t), [B][nz][P] with the stride of s
    float* gp;             // [Bp / 4][nz][P] partial sums of w(t+1) L U(t)
    float* ip;             // [Bp / 4][nz][P] partial sums of U(t)^2
    int Bp;                // batch padded to a multiple of four
    int grad;              // 0: illumination only (the last step)
};

__global__ void __launch_bounds__(128, 3) adjgrad_kernel(const AdjGradArgs ag)
{
    const StepArgs& a = ag.s;
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* __restrict__ ring = smem4 + wib * adjgrad_warp_quads();
    float4* __restrict__ xbw = ring + kAgRing * kAgSlot;     // [2][34] w(t+1) centre row with halo quads
    float4* __restrict__ xbu = xbw + 2 * 34;                   // [2][34] U(t) centre row with halo quads
    float4* __restrict__ red = smem4 + kWarpsPerBlock * adjgrad_warp_quads();   // [2 parity][2 field][4 warps][32]

    const int warp = blockIdx.x * kWarpsPerBlock + wib;
    const int slot_shot = warp % ag.Bp;
    const int rest = warp / ag.Bp;
    const int tile = rest % a.ntiles;
    const int seg = rest / a.ntiles;
    if (seg >= a.nseg) return;   // uniform per block (Bp is a multiple of the block's warps)
    const bool ghost = slot_shot >= a.B;
    const int shot = ghost ? a.B - 1 : slot_shot;
    const int grp = slot_shot / kWarpsPerBlock;

    const int x0 = tile * kTileWide + lane * 4;
    const int z0 = 4 + seg * a.H;
    const int z1 = min(z0 + a.H, a.nz - 4);
    const int P = a.P;
    const int zmax = a.nz - 1;
    const long long so = (long long)shot * a.shot_stride + x0;
    const float* __restrict__ wc = a.cur + so;      // w(t+1)
    float* __restrict__ wn = a.nxt + so;            // w(t+2) in, w(t) out
    const float* __restrict__ uc = ag.U + so;       // U(t)
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long mbytes = (long long)a.nz * a.P * 4;
    [[maybe_unused]] const long long pbytes = (long long)(ag.Bp / kWarpsPerBlock) * a.shot_stride * 4;

    bool colin[4];
    float cxf[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + j;
        colin[j] = x >= 4 && x < a.nx - 4;
        float f = 1.0f;
        if (x < a.N) f = *PAM_CHK(&a.cerjan[x], a.cerjan, a.N * 4, 4, 80);
        if (x >= a.nx - a.N && x < a.nx) f = f * *PAM_CHK(&a.cerjan[a.nx - 1 - x], a.cerjan, a.N * 4, 4, 80);
        cxf[j] = f;
    }
    const bool allin = colin[0] && colin[1] && colin[2] && colin[3];

    // ring loads for row rr: leading rows rr+4 of w(t+1) and U(t) (every
    // lane), the x halo quads of their row rr (lane 0: x0-4, tile 0 has none
    // and only its unwritten columns 0..3 would use it; lane 31: x0+4), and
    // w(t+2), kappa at row rr
    auto issue = [&](int rr) {
        float4* sa = ring + (rr & (kAgRing - 1)) * kAgSlot;
        const long long rl = (long long)min(rr, zmax) * P;
        const long long ra = (long long)min(rr + 4, zmax) * P;
        cp_async16(sa + lane, PAM_CHK(wc + ra, a.cur, fbytes, 16, 81));
        cp_async16(sa + 34 + lane, PAM_CHK(uc + ra, ag.U, fbytes, 16, 82));
        if ((lane == 0 && tile > 0) || lane == 31) {
            const int h = lane == 0 ? 0 : 1;
            const int off = lane == 0 ? -4 : 4;
            cp_async16(sa + 32 + h, PAM_CHK(wc + rl + off, a.cur, fbytes, 16, 83));
            cp_async16(sa + 66 + h, PAM_CHK(uc + rl + off, ag.U, fbytes, 16, 84));
        }
        cp_async16(sa + 68 + lane, PAM_CHK(wn + rl, a.nxt, fbytes, 16, 85));
        cp_async16(sa + 100 + lane, PAM_CHK(a.kap + x0 + rl, a.kap, mbytes, 16, 86));
        cp_async_commit();
    };

    float4 ww[9], uu[9];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const long long ro = (long long)min(z0 - 4 + i, zmax) * P;
        ww[i] = ldg4(PAM_CHK(wc + ro, a.cur, fbytes, 16, 87));
        uu[i] = ldg4(PAM_CHK(uc + ro, ag.U, fbytes, 16, 87));
    }
#pragma unroll
    for (int i = 0; i < kAgAhead; i++) issue(z0 + i);

    for (int r = z0; r < z1; r++) {
        issue(r + kAgAhead);
        cp_async_wait<kAgAhead>();
        const float4* sa = ring + (r & (kAgRing - 1)) * kAgSlot;
        ww[8] = sa[lane];
        uu[8] = sa[34 + lane];
        {
            float4* xw = xbw + (r & 1) * 34;
            float4* xu = xbu + (r & 1) * 34;
            xw[lane + 1] = ww[4];
            xu[lane + 1] = uu[4];
            if (lane == 0) { xw[0] = sa[32]; xu[0] = sa[66]; }
            if (lane == 31) { xw[33] = sa[33]; xu[33] = sa[67]; }
        }
        __syncwarp();
        const float4* xw = xbw + (r & 1) * 34;
        const float4* xu = xbu + (r & 1) * 34;
        const float4 wl = xw[lane], wr = xw[lane + 2], ul = xu[lane], ur = xu[lane + 2];
        const float4 w2 = sa[68 + lane], kap = sa[100 + lane];

        float cz = 1.0f;
        if (r < a.N) cz = *PAM_CHK(&a.cerjan[r], a.cerjan, a.N * 4, 4, 88);
        if (r >= a.nz - a.N) cz = cz * *PAM_CHK(&a.cerjan[a.nz - 1 - r], a.cerjan, a.N * 4, 4, 88);

        float4 gq = make_float4(0.f, 0.f, 0.f, 0.f), iq = make_float4(0.f, 0.f, 0.f, 0.f);
        {
            // w(t): the operand order of step_kernel<kAcoustic, kCerjan>
            const float4& c = ww[4];
            const float2 P0 = lo2(wl), P1 = hi2(wl), P2 = lo2(c), P3 = hi2(c), P4 = lo2(wr), P5 = hi2(wr);
            const float2 O0 = make_float2(wl.y, wl.z), O1 = make_float2(wl.w, c.x), O2 = make_float2(c.y, c.z);
            const float2 O3 = make_float2(c.w, wr.x), O4 = make_float2(wr.y, wr.z);
            float2 pxx[2], pzz[2];
            pxx[0] = d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx2);
            pxx[1] = d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx2);
            pzz[0] = d2_pair(lo2(c), lo2(ww[5]), lo2(ww[3]), lo2(ww[6]), lo2(ww[2]), lo2(ww[7]), lo2(ww[1]),
                             lo2(ww[8]), lo2(ww[0]), a.inv_dz2);
            pzz[1] = d2_pair(hi2(c), hi2(ww[5]), hi2(ww[3]), hi2(ww[6]), hi2(ww[2]), hi2(ww[7]), hi2(ww[1]),
                             hi2(ww[8]), hi2(ww[0]), a.inv_dz2);
            float o[4];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const float2 uq = q == 0 ? lo2(c) : hi2(c);
                const float2 k = q == 0 ? lo2(kap) : hi2(kap);
                const float2 cxq = make_float2(cxf[2 * q], cxf[2 * q + 1]);
                const float2 czq = make_float2(cz, cz);
                const float2 p = pmul2(pmul2(q == 0 ? lo2(w2) : hi2(w2), cxq), czq);
                const float2 base = fsub2(padd2(uq, uq), p);
                float2 v = pfma2(k, padd2(pxx[q], pzz[q]), base);
                v = pmul2(pmul2(v, cxq), czq);
                o[2 * q] = v.x;
                o[2 * q + 1] = v.y;
            }
            if (!ghost) {
                const long long ro = (long long)r * P;
                if (allin) {
                    *reinterpret_cast<float4*>(PAM_CHK(wn + ro, a.nxt, fbytes, 16, 89)) =
                        make_float4(o[0], o[1], o[2], o[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (colin[j]) *PAM_CHK(&wn[ro + j], a.nxt, fbytes, 4, 89) = o[j];
                }
            }
        }
        if (!ghost) {
            // L U(t) and the products with w(t+1), U(t)
            const float4& c = uu[4];
            const float2 P0 = lo2(ul), P1 = hi2(ul), P2 = lo2(c), P3 = hi2(c), P4 = lo2(ur), P5 = hi2(ur);
            const float2 O0 = make_float2(ul.y, ul.z), O1 = make_float2(ul.w, c.x), O2 = make_float2(c.y, c.z);
            const float2 O3 = make_float2(c.w, ur.x), O4 = make_float2(ur.y, ur.z);
            float2 lap[2];
            lap[0] = padd2(d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx2),
                           d2_pair(lo2(c), lo2(uu[5]), lo2(uu[3]), lo2(uu[6]), lo2(uu[2]), lo2(uu[7]), lo2(uu[1]),
                                   lo2(uu[8]), lo2(uu[0]), a.inv_dz2));
            lap[1] = padd2(d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx2),
                           d2_pair(hi2(c), hi2(uu[5]), hi2(uu[3]), hi2(uu[6]), hi2(uu[2]), hi2(uu[7]), hi2(uu[1]),
                                   hi2(uu[8]), hi2(uu[0]), a.inv_dz2));
            if (ag.grad) {
                const float2 g0 = pmul2(lo2(ww[4]), lap[0]), g1 = pmul2(hi2(ww[4]), lap[1]);
                gq = make_float4(g0.x, g0.y, g1.x, g1.y);
            }
            const float2 i0 = pmul2(lo2(c), lo2(c)), i1 = pmul2(hi2(c), hi2(c));
            iq = make_float4(i0.x, i0.y, i1.x, i1.y);
        }
        // the block's sum over its four shots, into the group's partial sums
        float4* rb = red + (r & 1) * (2 * kWarpsPerBlock * 32);
        rb[wib * 32 + lane] = gq;
        rb[(kWarpsPerBlock + wib) * 32 + lane] = iq;
        __syncthreads();
        if (wib < 2) {
            const float4* src = rb + wib * kWarpsPerBlock * 32 + lane;
            float4 s = src[0];
#pragma unroll
            for (int k = 1; k < kWarpsPerBlock; k++) {
                const float4 v = src[k * 32];
                const float2 lo = padd2(lo2(s), lo2(v)), hi = padd2(hi2(s), hi2(v));
                s = make_float4(lo.x, lo.y, hi.x, hi.y);
            }
            float* dst = (wib == 0 ? ag.gp : ag.ip) + (long long)grp * a.shot_stride + (long long)r * P + x0;
            float* base = wib == 0 ? ag.gp : ag.ip;
            if (allin) {
                float4* d4 = reinterpret_cast<float4*>(PAM_CHK(dst, base, pbytes, 16, 90));
                const float4 old = *d4;
                const float2 lo = padd2(lo2(old), lo2(s)), hi = padd2(hi2(old), hi2(s));
                *d4 = make_float4(lo.x, lo.y, hi.x, hi.y);
            } else {
                const float sv[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (colin[j]) *PAM_CHK(&dst[j], base, pbytes, 4, 90) += sv[j];
            }
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            ww[i] = ww[i + 1];
            uu[i] = uu[i + 1];
        }
    }
    cp_async_wait<0>();
}

// G = sum of the group partials (expanded grid, the update region); ilum on
// the interior grid [nzi][nxi] from the illumination partials.
__global__ void adjgrad_fold_kernel(const float* __restrict__ gp, const float* __restrict__ ip, int ngroups,
                                    long long stride, int nz, int nx, int P, int N, int nzi, int nxi,
                                    float* __restrict__ G, float* __restrict__ ilum)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x >= nx || z >= nz) return;
    const long long c = (long long)z * P + x;
    float g = 0.0f, i = 0.0f;
    for (int k = 0; k < ngroups; k++) {
        g += gp[(long long)k * stride + c];
        i += ip[(long long)k * stride + c];
    }
    G[c] = g;
    const int zi = z - N, xi = x - N;
    if (zi >= 0 && zi < nzi && xi >= 0 && xi < nxi) ilum[(long long)zi * nxi + xi] = i;
}

}  // namespace pam
