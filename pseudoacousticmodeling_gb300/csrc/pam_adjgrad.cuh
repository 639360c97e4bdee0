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
// and four consecutive shots (shots are the fastest grid dimension).  The
// warps march two rows per trip; per trip they put their products in shared
// memory (double-buffered by trip parity, one block barrier per trip), and
// each warp then adds the four shots' values of one (row, field) pair in a
// fixed order to the block's own row of a per-group partial sum
// ([shots / 4][nz][P]: every (group, cell) belongs to exactly one block, so
// there is no atomic and the result does not depend on scheduling).  The
// groups are added after the sweep (adjgrad_fold_kernel).  The partial rows
// are fetched with cp.async a few rows ahead, so the read-modify-write does
// not wait on a DRAM round trip.  Batches whose size is not a multiple of
// four are padded with ghost shots that load nothing, contribute zero and
// store nothing.
#pragma once
#include "pam_kernels.cuh"

namespace pam {

constexpr int kAgRing = 4;                        // field ring slots
constexpr int kAgAhead = 3;                       // rows in flight
constexpr int kAgSlot = 34 + 34 + 32 + 32;        // w lead + halo, U lead + halo, w(t+2), kappa
constexpr int kAgPart = 4;                        // partial-row slots (one per trip, trip index mod 4)
static_assert(kAgAhead + 1 <= kAgRing, "ring too small for the prefetch distance");
// the partial row of trip T is fetched during trip T - 2 or T - 1, into the
// slot trip T - 4 used, whose sum was stored at the end of trip T - 4
static_assert(kAgPart >= 3 && (kAgAhead + 1) / 2 + 1 < kAgPart, "too few partial slots for the prefetch distance");

__host__ __device__ constexpr int adjgrad_warp_quads() { return kAgRing * kAgSlot + 2 * 34 + 2 * 34 + kAgPart * 32; }
// per warp: ring, x exchange rows, partial rows; per block: the products of
// [2 trip parity][2 rows][2 fields][4 warps][32 lanes]
__host__ __device__ constexpr int adjgrad_smem_bytes() {
    return (kWarpsPerBlock * adjgrad_warp_quads() + 2 * 2 * 2 * kWarpsPerBlock * 32) * 16;
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
    float4* __restrict__ pbuf = xbu + 2 * 34;                  // [kAgPart][32] partial rows
    float4* __restrict__ red = smem4 + kWarpsPerBlock * adjgrad_warp_quads();

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

    // this warp's share of the per-trip sums: row (wib >> 1) of the trip,
    // field (wib & 1): 0 gradient, 1 illumination
    const int myj = wib >> 1;
    float* const pbase = (wib & 1) ? ag.ip : ag.gp;
    float* const prow = pbase + (long long)grp * a.shot_stride + x0;

    // warp-uniform: does the tile reach into an x border?
    const int tx0 = tile * kTileWide - 4, tx1 = tx0 + kTileWide + 8;
    const bool xborder = (tx0 < a.N) || (tx1 > a.nx - a.N);
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

    // loads for row rr: leading rows rr+4 of w(t+1) and U(t) (every lane),
    // the x halo quads of their row rr (lane 0: x0-4, tile 0 has none and only
    // its unwritten columns 0..3 would use it; lane 31: x0+4), w(t+2) and
    // kappa at row rr, and the partial row rr if this warp sums that row.
    // Rows past the segment are clamped to the grid and never used.
    auto issue = [&](int rr) {
        float4* sa = ring + (rr & (kAgRing - 1)) * kAgSlot;
        const long long rl = (long long)min(rr, zmax) * P;
        if (!ghost) {
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
        }
        if (((rr - z0) & 1) == myj)
            cp_async16(pbuf + (((rr - z0) >> 1) & (kAgPart - 1)) * 32 + lane, PAM_CHK(prow + rl, pbase, pbytes, 16, 91));
        cp_async_commit();
    };

    // One row: w(t) from the w(t+1) window, stored; the products of this
    // shot into red.  w[0..8], u[0..8] are rows rr-4 .. rr+4 (the last one
    // taken from the ring here).
    auto row = [&](auto edge_tag, int rr, int j, float4* __restrict__ rb, float4& w8, float4& u8,
                   const float4& w0, const float4& w1, const float4& w2r, const float4& w3, const float4& c,
                   const float4& w5, const float4& w6, const float4& w7,
                   const float4& u0, const float4& u1, const float4& u2, const float4& u3, const float4& uc4,
                   const float4& u5, const float4& u6, const float4& u7) {
        constexpr bool EDGE = decltype(edge_tag)::value;
        issue(rr + kAgAhead);
        cp_async_wait<kAgAhead>();
        float4 gq = make_float4(0.f, 0.f, 0.f, 0.f), iq = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!ghost) {
            const float4* sa = ring + (rr & (kAgRing - 1)) * kAgSlot;
            w8 = sa[lane];
            u8 = sa[34 + lane];
            {
                float4* xw = xbw + (rr & 1) * 34;
                float4* xu = xbu + (rr & 1) * 34;
                xw[lane + 1] = c;
                xu[lane + 1] = uc4;
                if (lane == 0) { xw[0] = sa[32]; xu[0] = sa[66]; }
                if (lane == 31) { xw[33] = sa[33]; xu[33] = sa[67]; }
            }
            __syncwarp();
            const float4* xw = xbw + (rr & 1) * 34;
            const float4* xu = xbu + (rr & 1) * 34;
            const float4 wl = xw[lane], wr = xw[lane + 2], ul = xu[lane], ur = xu[lane + 2];
            const float4 wp = sa[68 + lane], kap = sa[100 + lane];

            const bool zborder = EDGE && ((rr < a.N) || (rr >= a.nz - a.N));
            const bool damp = EDGE && (xborder || zborder);
            float cz = 1.0f;
            if (EDGE && zborder) {
                if (rr < a.N) cz = *PAM_CHK(&a.cerjan[rr], a.cerjan, a.N * 4, 4, 88);
                if (rr >= a.nz - a.N) cz = cz * *PAM_CHK(&a.cerjan[a.nz - 1 - rr], a.cerjan, a.N * 4, 4, 88);
            }
            {
                // w(t): the operand order of step_kernel<kAcoustic, kCerjan>;
                // undamped cells skip the factors, which are exactly 1 there
                const float2 P0 = lo2(wl), P1 = hi2(wl), P2 = lo2(c), P3 = hi2(c), P4 = lo2(wr), P5 = hi2(wr);
                const float2 O0 = make_float2(wl.y, wl.z), O1 = make_float2(wl.w, c.x), O2 = make_float2(c.y, c.z);
                const float2 O3 = make_float2(c.w, wr.x), O4 = make_float2(wr.y, wr.z);
                float2 pxx[2], pzz[2];
                pxx[0] = d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx2);
                pxx[1] = d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx2);
                pzz[0] = d2_pair(lo2(c), lo2(w5), lo2(w3), lo2(w6), lo2(w2r), lo2(w7), lo2(w1), lo2(w8), lo2(w0),
                                 a.inv_dz2);
                pzz[1] = d2_pair(hi2(c), hi2(w5), hi2(w3), hi2(w6), hi2(w2r), hi2(w7), hi2(w1), hi2(w8), hi2(w0),
                                 a.inv_dz2);
                float o[4];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const float2 uq = q == 0 ? lo2(c) : hi2(c);
                    const float2 k = q == 0 ? lo2(kap) : hi2(kap);
                    const float2 cxq = make_float2(cxf[2 * q], cxf[2 * q + 1]);
                    const float2 czq = make_float2(cz, cz);
                    float2 p = q == 0 ? lo2(wp) : hi2(wp);
                    if (damp) p = pmul2(pmul2(p, cxq), czq);
                    const float2 base = fsub2(padd2(uq, uq), p);
                    float2 v = pfma2(k, padd2(pxx[q], pzz[q]), base);
                    if (damp) v = pmul2(pmul2(v, cxq), czq);
                    o[2 * q] = v.x;
                    o[2 * q + 1] = v.y;
                }
                const long long ro = (long long)rr * P;
                if (!EDGE || allin) {
                    *reinterpret_cast<float4*>(PAM_CHK(wn + ro, a.nxt, fbytes, 16, 89)) =
                        make_float4(o[0], o[1], o[2], o[3]);
                } else {
#pragma unroll
                    for (int jj = 0; jj < 4; jj++)
                        if (colin[jj]) *PAM_CHK(&wn[ro + jj], a.nxt, fbytes, 4, 89) = o[jj];
                }
            }
            {
                // L U(t) and the products with w(t+1), U(t)
                const float2 P0 = lo2(ul), P1 = hi2(ul), P2 = lo2(uc4), P3 = hi2(uc4), P4 = lo2(ur), P5 = hi2(ur);
                const float2 O0 = make_float2(ul.y, ul.z), O1 = make_float2(ul.w, uc4.x);
                const float2 O2 = make_float2(uc4.y, uc4.z), O3 = make_float2(uc4.w, ur.x);
                const float2 O4 = make_float2(ur.y, ur.z);
                float2 lap[2];
                lap[0] = padd2(d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx2),
                               d2_pair(lo2(uc4), lo2(u5), lo2(u3), lo2(u6), lo2(u2), lo2(u7), lo2(u1), lo2(u8),
                                       lo2(u0), a.inv_dz2));
                lap[1] = padd2(d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx2),
                               d2_pair(hi2(uc4), hi2(u5), hi2(u3), hi2(u6), hi2(u2), hi2(u7), hi2(u1), hi2(u8),
                                       hi2(u0), a.inv_dz2));
                if (ag.grad) {
                    const float2 g0 = pmul2(lo2(c), lap[0]), g1 = pmul2(hi2(c), lap[1]);
                    gq = make_float4(g0.x, g0.y, g1.x, g1.y);
                }
                const float2 i0 = pmul2(lo2(uc4), lo2(uc4)), i1 = pmul2(hi2(uc4), hi2(uc4));
                iq = make_float4(i0.x, i0.y, i1.x, i1.y);
            }
        }
        rb[((j * 2 + 0) * kWarpsPerBlock + wib) * 32 + lane] = gq;
        rb[((j * 2 + 1) * kWarpsPerBlock + wib) * 32 + lane] = iq;
    };

    // the four shots' sum of this warp's (row, field) of the trip, added to
    // the group's partial row
    auto reduce = [&](auto edge_tag, int r, int trip, const float4* __restrict__ rb) {
        constexpr bool EDGE = decltype(edge_tag)::value;
        const int rr = r + myj;
        if (rr >= z1) return;
        const float4* src = rb + ((myj * 2 + (wib & 1)) * kWarpsPerBlock) * 32 + lane;
        float4 s = src[0];
#pragma unroll
        for (int k = 1; k < kWarpsPerBlock; k++) {
            const float4 v = src[k * 32];
            const float2 lo = padd2(lo2(s), lo2(v)), hi = padd2(hi2(s), hi2(v));
            s = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
        const float4 old = pbuf[(trip & (kAgPart - 1)) * 32 + lane];
        const float2 lo = padd2(lo2(old), lo2(s)), hi = padd2(hi2(old), hi2(s));
        float* dst = prow + (long long)rr * P;
        if (!EDGE || allin) {
            *reinterpret_cast<float4*>(PAM_CHK(dst, pbase, pbytes, 16, 90)) = make_float4(lo.x, lo.y, hi.x, hi.y);
        } else {
            const float sv[4] = {lo.x, lo.y, hi.x, hi.y};
#pragma unroll
            for (int jj = 0; jj < 4; jj++)
                if (colin[jj]) *PAM_CHK(&dst[jj], pbase, pbytes, 4, 90) = sv[jj];
        }
    };

    // The march: register windows w[0..9], u[0..9] = rows r-4 .. r+5 of a
    // trip of two rows (r, r+1); a trip's second row past z1 (odd segment
    // height) is skipped by the whole block.
    auto march = [&](auto edge_tag) {
        float4 w[10], u[10];
        if (!ghost) {
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const long long ro = (long long)min(z0 - 4 + i, zmax) * P;
                w[i] = ldg4(PAM_CHK(wc + ro, a.cur, fbytes, 16, 87));
                u[i] = ldg4(PAM_CHK(uc + ro, ag.U, fbytes, 16, 87));
            }
        }
#pragma unroll
        for (int i = 0; i < kAgAhead; i++) issue(z0 + i);
        int trip = 0;
        for (int r = z0; r < z1; r += 2, trip++) {
            float4* rb = red + (trip & 1) * (2 * 2 * kWarpsPerBlock * 32);
            row(edge_tag, r, 0, rb, w[8], u[8], w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7],
                u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7]);
            if (r + 1 < z1)
                row(edge_tag, r + 1, 1, rb, w[9], u[9], w[1], w[2], w[3], w[4], w[5], w[6], w[7], w[8],
                    u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8]);
            __syncthreads();
            reduce(edge_tag, r, trip, rb);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                w[i] = w[i + 2];
                u[i] = u[i + 2];
            }
        }
    };
    const bool edge = xborder || z0 < a.N || z1 > a.nz - a.N;
    if (edge) march(IntTag<1>{});
    else march(IntTag<0>{});
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
