// Device code of the finite-difference hot path, written for sm_103a (GB300).
//
// Layout in HBM (one shot batch):
//   wavefields   float [B][nz][P]   nz = nz_abc, P = row pitch (multiple of 32
//                                   floats, >= the last tile's reach); cells
//                                   outside [4,nz-4) x [4,nx-4) stay zero
//   models       float [nz][P]      kappa = vp^2 dt^2; for VTI/TTI the update
//                                   coefficients 1+2eps, -2(eps-delta),
//                                   2(1+delta) (and cos/sin theta), shared by
//                                   every shot of the batch
//   CPML x strip float2 [B][nz][2N] (d psi_x, d psi_x + zeta_x) per step
//   CPML z strip float2 [B][2N][P]  (d psi_z, d psi_z + zeta_z) per step
//
// Stepping kernel ("warp march"): one warp owns one shot, one tile of 32
// lanes x float4 and one z segment whose height the engine tunes per batch
// size.  It walks down its segment keeping the nine rows z-4..z+4 of U(t) in
// a register window; the leading row, U(t-1) and the model rows arrive two
// (acoustic: three) rows ahead through a per-warp cp.async ring in shared
// memory, and x neighbours are exchanged through a shared row.  Acoustic and
// VTI tiles are 128 aligned columns with the 4-column halo on each side
// fetched as two extra quads; TTI tiles keep lanes 0 and 31 as halo lanes
// (its cross derivative needs the z derivative at the halo columns) and write
// 120 columns.  Warps whose tile or segment reaches into the absorbing border
// march one row per loop trip with the Cerjan damping or CPML strip terms;
// all others march several rows per trip with no border code.  No block
// barriers: every warp is independent, and the grid is ordered shot-fastest
// so that the model rows a tile needs are read from HBM once and from L2 by
// the other shots.  The arithmetic runs on packed two-wide FP32 instructions
// (FFMA2 / FADD2 / FMUL2).
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pam_check.cuh"
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

// ---------------------------------------------------------------------------
// One forward time step for a shot batch (see the file header).
//
// Per row r a warp needs U(t) rows r-4..r+4 (a nine-row register window) and,
// for its writer lanes, U(t-1) and the model at row r.  The window's leading
// row r+4, U(t-1) and the model rows arrive through a per-warp ring of kRing
// shared-memory slots filled by cp.async ring_ahead() rows ahead, so their HBM
// latency overlaps the arithmetic of earlier rows without costing registers.
// x neighbours are exchanged through a double-buffered shared row (one
// 16-byte store and two loads per row).

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int kRing = 4;    // ring slots per warp

// Rows in flight ahead of the one being computed (at most kRing - 1: the slot
// refilled at row r is the one read at row r + ahead - kRing).  The acoustic
// kernel, with the least arithmetic to hide the latency behind, gains from
// three; the anisotropic ones run best with two.
template <int APPROX>
__host__ __device__ constexpr int ring_ahead() { return APPROX == kAcoustic ? 3 : 2; }
static_assert(3 <= kRing - 1, "ring too small for the prefetch distance");

// ring arrays per slot: U(t) leading row (all lanes), then U(t-1), kappa,
// 1 + 2 eps, -2 (eps - delta), 2 (1 + delta), cos, sin (writer lanes)
template <int APPROX>
__host__ __device__ constexpr int ring_arrays() { return APPROX == kAcoustic ? 3 : (APPROX == kVTI ? 6 : 8); }

// Acoustic and VTI tiles write all 128 columns and fetch the 4-column x halo
// on each side (two extra quads per row in the ring); TTI keeps lanes 0 and
// 31 as halo lanes, because its cross derivative needs the z derivative at
// the halo columns, i.e. their whole z window.
template <int APPROX>
__host__ __device__ constexpr bool fetched_halo() { return APPROX != kTTI; }

// float4 entries per ring slot: the arrays, plus the two halo quads
template <int APPROX>
__host__ __device__ constexpr int slot_quads() { return ring_arrays<APPROX>() * 32 + (fetched_halo<APPROX>() ? 2 : 0); }

// shared exchange entries per warp: U(t) double-buffered (34 quads with the
// fetched halo), plus the z derivative for the TTI cross term
template <int APPROX>
__host__ __device__ constexpr int xchg_quads() { return APPROX == kTTI ? 4 * 32 : 2 * 34; }

template <int APPROX>
__host__ __device__ constexpr int step_smem_bytes() {
    return kWarpsPerBlock * (kRing * slot_quads<APPROX>() + xchg_quads<APPROX>()) * 16;
}

// Packed two-wide FP32 arithmetic (sm_100+ FFMA2 / FADD2 / FMUL2), written
// as inline PTX: every operation rounds exactly as written, whichever kernel
// and code path it is inlined into, so that kernels evaluating the same
// update (one step per launch, two steps per launch) agree bit for bit.
__device__ __forceinline__ unsigned long long f2bits(float2 v) { return *reinterpret_cast<unsigned long long*>(&v); }
__device__ __forceinline__ float2 bits2f(unsigned long long b) { return *reinterpret_cast<float2*>(&b); }
__device__ __forceinline__ float2 padd2(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}
__device__ __forceinline__ float2 pmul2(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}
__device__ __forceinline__ float2 pfma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)), "l"(f2bits(c)));
    return bits2f(d);
}
__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ float2 bc2(float c) { return make_float2(c, c); }

// Second derivative of a cell pair: (C0 c + C1 (p1 + m1) + ... + C4 (p4 + m4)) * inv,
// the reference's literal coefficients and term order (cpp/Modeling.cu:521-525).
__device__ __forceinline__ float2 d2_pair(float2 c, float2 p1, float2 m1, float2 p2, float2 m2, float2 p3, float2 m3,
                                          float2 p4, float2 m4, float inv) {
    float2 t = pmul2(bc2(kC0), c);
    t = pfma2(bc2(kC1), padd2(p1, m1), t);
    t = pfma2(bc2(kC2), padd2(p2, m2), t);
    t = pfma2(bc2(kC3), padd2(p3, m3), t);
    t = pfma2(bc2(kC4), padd2(p4, m4), t);
    return pmul2(t, bc2(inv));
}

// Two-wide subtraction a - b (PTX sub.f32x2, sm_100+), the same rounding as
// a + (-b) in each half.
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(d);
}

// First derivative of a cell pair with coefficients A_k / d already scaled.
__device__ __forceinline__ float2 d1_pair(float2 p1, float2 m1, float2 p2, float2 m2, float2 p3, float2 m3, float2 p4,
                                          float2 m4, const float* a1) {
    float2 t = pmul2(bc2(a1[0]), fsub2(p1, m1));
    t = pfma2(bc2(a1[1]), fsub2(p2, m2), t);
    t = pfma2(bc2(a1[2]), fsub2(p3, m3), t);
    t = pfma2(bc2(a1[3]), fsub2(p4, m4), t);
    return t;
}

// First derivative of a cell pair in the reference's written form
// (cpp/Modeling.cu:595-603): (a1 (p1 - m1) + a2 (p2 - m2) + a3 (p3 - m3) +
// a4 (p4 - m4)) * inv with the literal coefficients, the sum contracted as
// the compiler contracts the reference's expression (the first product
// fused into the second, then one fused multiply-add per term).  The Sd
// switch |den| > 1e-12 makes the anisotropic update sensitive to how px and
// pz round near the threshold; pre-scaling the coefficients by inv biases
// every derivative by their rounding errors and switched Sd in enough cells
// to move the seismograms 1.4-1.8e-5 from the reference's own kernels.
__device__ __forceinline__ float2 d1_pair_ref(float2 p1, float2 m1, float2 p2, float2 m2, float2 p3, float2 m3,
                                              float2 p4, float2 m4, float inv) {
    float2 t = pfma2(bc2(kA1), fsub2(p1, m1), pmul2(bc2(kA2), fsub2(p2, m2)));
    t = pfma2(bc2(kA3), fsub2(p3, m3), t);
    t = pfma2(bc2(kA4), fsub2(p4, m4), t);
    return pmul2(t, bc2(inv));
}

// Sd = num / den where |den| > 1e-12, else 0 (cpp/Modeling.cu:605-611), with
// the hardware reciprocal (rcp.approx, about 1 ulp) in place of the
// correctly rounded division; den > 1e-12 keeps its input normal.  A build
// with -DPAM_SD_DIV divides with correct rounding instead, as the reference
// does (the measurement build of the parity tests).
__device__ __forceinline__ float sd_ratio(float num, float den) {
#ifdef PAM_SD_DIV
    return fabsf(den) > 1e-12f ? __fdiv_rn(num, den) : 0.0f;
#else
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(den));
    return fabsf(den) > 1e-12f ? num * r : 0.0f;
#endif
}

template <int APPROX>
__host__ __device__ constexpr int step_min_blocks() { return APPROX == kTTI ? 3 : 4; }

// Rows per trip of the interior march loop.  The nine-row register window
// shifts by register moves once per trip (eight quads), so unrolling divides
// those moves by this factor, as far as the registers allow.
template <int APPROX>
__host__ __device__ constexpr int interior_unroll() { return APPROX == kAcoustic ? 2 : 4; }

template <int V>
struct IntTag { static constexpr int value = V; };

// One time step of this thread's warp (its shot, tile and segment): the
// body of step_kernel, also run once per step by step_persistent_kernel.
template <int APPROX, int BC>
__device__ __forceinline__ void step_body(const StepArgs& a)
{
    constexpr int NA = ring_arrays<APPROX>();
    constexpr bool XH = fetched_halo<APPROX>();
    constexpr int SQ = slot_quads<APPROX>();
    constexpr int kAhead = ring_ahead<APPROX>();
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* __restrict__ ring = smem4 + wib * (kRing * SQ);
    float4* __restrict__ xbuf = smem4 + kWarpsPerBlock * kRing * SQ + wib * xchg_quads<APPROX>();

    const int warp = blockIdx.x * kWarpsPerBlock + wib;
    const int shot = warp % a.B;
    const int rest = warp / a.B;
    const int tile = rest % a.ntiles;
    const int seg = rest / a.ntiles;
    if (seg >= a.nseg) return;   // uniform per warp

    // first column of this lane's quad: with fetched halos tile t covers the
    // 128-aligned columns [128 t, 128 t + 128) (so every row access is four
    // whole 128-byte lines) and writes those inside [4, nx - 4); with halo
    // lanes lane 0 holds the tile's left halo (columns 120 tile + 4 lane ..)
    const int x0 = XH ? tile * kTileWide + lane * 4 : tile * kTileOut + lane * 4;
    const int z0 = 4 + seg * a.H;
    const int z1 = min(z0 + a.H, a.nz - 4);
    const int P = a.P;
    const long long so = (long long)shot * a.shot_stride + x0;
    const float* __restrict__ cur = a.cur + so;
    float* __restrict__ nxt = a.nxt + so;
    const float* prv = (a.prev ? a.prev : a.nxt) + so;   // U(t-1); may alias nxt
    const bool writer = XH || (lane >= 1 && lane <= 30);
    const int zmax = a.nz - 1;
    // buffer extents for the check build's guards (PAM_CHK; unused otherwise)
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;   // a field of the batch
    [[maybe_unused]] const long long mbytes = (long long)a.nz * a.P * 4;            // a model array
    const int sz = *PAM_CHK(&a.src_z[shot], a.src_z, a.B * 4, 4, 15);
    const int sx = *PAM_CHK(&a.src_x[shot], a.src_x, a.B * 4, 4, 15);

    // warp-uniform: does this tile reach into an x border / strip?
    const int tx0 = XH ? tile * kTileWide - 4 : tile * kTileOut, tx1 = tx0 + kTileLoad + (XH ? 8 : 0);
    const bool xborder = (tx0 < a.N) || (tx1 > a.nx - a.N);

    // Cerjan factors along x for this quad (x first, then z: cpp/Modeling.cu:535-550)
    float cxf[4] = {1.f, 1.f, 1.f, 1.f};
    if (BC == kCerjan && xborder) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int x = x0 + j;
            float f = 1.0f;
            if (x < a.N) f = *PAM_CHK(&a.cerjan[x], a.cerjan, a.N * 4, 4, 13);
            if (x >= a.nx - a.N && x < a.nx) f = f * *PAM_CHK(&a.cerjan[a.nx - 1 - x], a.cerjan, a.N * 4, 4, 13);
            cxf[j] = f;
        }
    }

    // prefetch ring, kAhead rows ahead: U(t) row r+4 (the queue's leading row)
    // for every lane; U(t-1) and the model arrays at row r for writer lanes.
    auto issue = [&](int rr) {
        float4* slot = ring + ((rr - z0) & (kRing - 1)) * SQ + lane;
        cp_async16(slot, PAM_CHK(cur + (long long)min(rr + 4, zmax) * P, a.cur, fbytes, 16, 1));
        if (XH && ((lane == 0 && tile > 0) || lane == 31)) {
            // the x halo quads of row rr: columns x0 - 4 (lane 0; tile 0 has no
            // left halo, and only its unwritten columns 0..3 would use it) and
            // x0 + 4 (lane 31)
            const long long ro = (long long)min(rr, zmax) * P;
            cp_async16(ring + ((rr - z0) & (kRing - 1)) * SQ + NA * 32 + (lane == 0 ? 0 : 1),
                       PAM_CHK(cur + ro + (lane == 0 ? -4 : 4), a.cur, fbytes, 16, 2));
        }
        if (writer) {
            const long long ro = (long long)min(rr, zmax) * P;
            cp_async16(slot + 32, PAM_CHK(prv + ro, a.prev ? a.prev : a.nxt, fbytes, 16, 3));
            cp_async16(slot + 64, PAM_CHK(a.kap + x0 + ro, a.kap, mbytes, 16, 4));
            if (NA > 3) {
                cp_async16(slot + 96, PAM_CHK(a.e2 + x0 + ro, a.e2, mbytes, 16, 5));
                cp_async16(slot + 128, PAM_CHK(a.m1 + x0 + ro, a.m1, mbytes, 16, 6));
                cp_async16(slot + 160, PAM_CHK(a.m2 + x0 + ro, a.m2, mbytes, 16, 7));
            }
            if (NA > 6) {
                cp_async16(slot + 192, PAM_CHK(a.cth + x0 + ro, a.cth, mbytes, 16, 8));
                cp_async16(slot + 224, PAM_CHK(a.sth + x0 + ro, a.sth, mbytes, 16, 9));
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int i = 0; i < kAhead; i++) issue(z0 + i);

    // One row of the march.  EDGE rows may lie in the absorbing border (Cerjan
    // damping, CPML strip terms, partial stores); interior rows are free of
    // all of it.  A row past the segment end (live false: the tail of an
    // unrolled trip) is computed from in-bounds reads but not stored.
    auto row = [&](auto edge_tag, int r, bool live, float4& Q0, float4& Q1, float4& Q2, float4& Q3, float4& Q4,
                   float4& Q5, float4& Q6, float4& Q7, float4& Q8) {
        constexpr bool EDGE = decltype(edge_tag)::value != 0;
        issue(r + kAhead);
        cp_async_wait<kAhead>();
        const float4* slot0 = ring + ((r - z0) & (kRing - 1)) * SQ;
        const float4* slot = slot0 + lane;
        Q8 = slot[0];
        // CPML strip terms of this row, loaded before its arithmetic so that
        // their latency overlaps it (zero outside the strips)
        float2 xst[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        float4 zst[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
        if (EDGE && BC == kCPML && xborder) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int x = x0 + j;
                if (x < a.N || (x >= a.nx - a.N && x < a.nx - 4)) {
                    const int c = x < a.N ? x : x - (a.nx - 2 * a.N);
                    xst[j] = *PAM_CHK(&a.xaux[(long long)shot * a.xaux_stride + (long long)r * (2 * a.N) + c], a.xaux,
                                      (long long)a.B * a.xaux_stride * 8, 8, 11);
                }
            }
        }
        if (EDGE && BC == kCPML && ((r < a.N) || (r >= a.nz - a.N))) {
            const int rr = r < a.N ? r : r - (a.nz - 2 * a.N);
            const float4* zt = PAM_CHK(reinterpret_cast<const float4*>(
                                           a.zaux + (long long)shot * a.zaux_stride + (long long)rr * P + x0),
                                       a.zaux, (long long)a.B * a.zaux_stride * 8, 32, 12);
            zst[0] = zt[0];
            zst[1] = zt[1];
        }

        // x neighbours through the shared exchange row
        const float4 center = Q4;
        float4 left, right;
        if (XH) {
            float4* xb = xbuf + (r & 1) * 34;
            xb[lane + 1] = center;
            if (lane == 0) xb[0] = slot0[NA * 32];
            if (lane == 31) xb[33] = slot0[NA * 32 + 1];
            __syncwarp();
            left = xb[lane];
            right = xb[lane + 2];
        } else {
            float4* xb = xbuf + (r & 1) * 32;
            xb[lane] = center;
            __syncwarp();
            left = xb[(lane + 31) & 31];
            right = xb[(lane + 1) & 31];
        }

        // The arithmetic runs on packed pairs (cells 0,1 and cells 2,3 of the quad)
        // with the sm_100+ two-wide FP32 instructions.  Window w[0..11] = left,
        // center, right; aligned pairs Pm = (w[2m], w[2m+1]) and odd pairs
        // Om = (w[2m+1], w[2m+2]) give every stencil operand of both cell pairs.
        float2 pxx2[2], px2v[2], pzz2[2], pz2v[2];
        {
            const float2 P0 = make_float2(left.x, left.y), P1 = make_float2(left.z, left.w);
            const float2 P2 = make_float2(center.x, center.y), P3 = make_float2(center.z, center.w);
            const float2 P4 = make_float2(right.x, right.y), P5 = make_float2(right.z, right.w);
            const float2 O0 = make_float2(left.y, left.z), O1 = make_float2(left.w, center.x);
            const float2 O2 = make_float2(center.y, center.z), O3 = make_float2(center.w, right.x);
            const float2 O4 = make_float2(right.y, right.z);
            // pair 0: centre P2; pair 1: centre P3
            pxx2[0] = d2_pair(P2, O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx2);
            pxx2[1] = d2_pair(P3, O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx2);
            px2v[0] = d1_pair_ref(O2, O1, P3, P1, O3, O0, P4, P0, a.inv_dx);
            px2v[1] = d1_pair_ref(O3, O2, P4, P2, O4, O1, P5, P1, a.inv_dx);
            const float2 z0 = lo2(Q0), z1 = lo2(Q1), z2 = lo2(Q2), z3 = lo2(Q3), z4 = lo2(Q4), z5 = lo2(Q5),
                         z6 = lo2(Q6), z7 = lo2(Q7), z8 = lo2(Q8);
            pzz2[0] = d2_pair(z4, z5, z3, z6, z2, z7, z1, z8, z0, a.inv_dz2);
            pz2v[0] = d1_pair_ref(z5, z3, z6, z2, z7, z1, z8, z0, a.inv_dz);
            const float2 y0 = hi2(Q0), y1 = hi2(Q1), y2 = hi2(Q2), y3 = hi2(Q3), y4 = hi2(Q4), y5 = hi2(Q5),
                         y6 = hi2(Q6), y7 = hi2(Q7), y8 = hi2(Q8);
            pzz2[1] = d2_pair(y4, y5, y3, y6, y2, y7, y1, y8, y0, a.inv_dz2);
            pz2v[1] = d1_pair_ref(y5, y3, y6, y2, y7, y1, y8, y0, a.inv_dz);
        }
        float2 pxz2[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (APPROX == kTTI) {
            // cross derivative: x derivative of the z derivative (cpp/Modeling.cu:674-693
            // factorised), from the neighbours' pz through the second exchange row
            float4* zb = xbuf + (2 + (r & 1)) * 32;
            zb[lane] = make_float4(pz2v[0].x, pz2v[0].y, pz2v[1].x, pz2v[1].y);
            __syncwarp();
            const float4 pl = zb[(lane + 31) & 31];
            const float4 pr = zb[(lane + 1) & 31];
            const float2 V0 = make_float2(pl.x, pl.y), V1 = make_float2(pl.z, pl.w);
            const float2 V2 = pz2v[0], V3 = pz2v[1];
            const float2 V4 = make_float2(pr.x, pr.y), V5 = make_float2(pr.z, pr.w);
            const float2 W0 = make_float2(pl.y, pl.z), W1 = make_float2(pl.w, V2.x);
            const float2 W2 = make_float2(V2.y, V3.x), W3 = make_float2(V3.y, pr.x);
            const float2 W4 = make_float2(pr.y, pr.z);
            pxz2[0] = d1_pair(W2, W1, V3, V1, W3, W0, V4, V0, a.cx1);
            pxz2[1] = d1_pair(W3, W2, V4, V2, W4, W1, V5, V1, a.cx1);
        }

        if (writer) {
            const float4 prev = slot[32];
            const float4 kap = slot[64];
            float4 e4, n4, b4, c4, s4;
            if (NA > 3) { e4 = slot[96]; n4 = slot[128]; b4 = slot[160]; }
            if (NA > 6) { c4 = slot[192]; s4 = slot[224]; }
            const bool zborder = EDGE && ((r < a.N) || (r >= a.nz - a.N));
            float cz = 1.0f;
            if (EDGE && BC == kCerjan && zborder) {
                if (r < a.N) cz = *PAM_CHK(&a.cerjan[r], a.cerjan, a.N * 4, 4, 14);
                if (r >= a.nz - a.N) cz = cz * *PAM_CHK(&a.cerjan[a.nz - 1 - r], a.cerjan, a.N * 4, 4, 14);
            }
            const bool damp = EDGE && (BC == kCerjan) && (xborder || zborder);
            const long long ro = (long long)r * P;

            // CPML strip terms (loaded at the top of the row), added to the
            // derivatives by strip warps only (a warp-uniform branch; interior
            // warps neither load nor add them).
            // Acoustic: pxx <- pxx + pzz and pzz <- hx + hz, so the common
            // lap = pxx + pzz below is (pxx + pzz) + (hx + hz).
            if (EDGE && BC == kCPML && (xborder || zborder)) {
                float gx[4] = {0.f, 0.f, 0.f, 0.f}, hx[4] = {0.f, 0.f, 0.f, 0.f};
                float gz[4] = {0.f, 0.f, 0.f, 0.f}, hz[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    gx[j] = xst[j].x;
                    hx[j] = xst[j].y;
                }
                gz[0] = zst[0].x; hz[0] = zst[0].y; gz[1] = zst[0].z; hz[1] = zst[0].w;
                gz[2] = zst[1].x; hz[2] = zst[1].y; gz[3] = zst[1].z; hz[3] = zst[1].w;
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const float2 hxq = make_float2(hx[2 * q], hx[2 * q + 1]);
                    const float2 hzq = make_float2(hz[2 * q], hz[2 * q + 1]);
                    if (APPROX == kAcoustic) {
                        pxx2[q] = padd2(pxx2[q], pzz2[q]);
                        pzz2[q] = padd2(hxq, hzq);
                    } else {
                        px2v[q] = padd2(px2v[q], make_float2(gx[2 * q], gx[2 * q + 1]));
                        pz2v[q] = padd2(pz2v[q], make_float2(gz[2 * q], gz[2 * q + 1]));
                        pxx2[q] = padd2(pxx2[q], hxq);
                        pzz2[q] = padd2(pzz2[q], hzq);
                    }
                }
            }

            float2 outp[2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const float2 uc = q == 0 ? lo2(center) : hi2(center);
                float2 p = q == 0 ? lo2(prev) : hi2(prev);
                const float2 k = q == 0 ? lo2(kap) : hi2(kap);
                const float2 cxq = make_float2(cxf[2 * q], cxf[2 * q + 1]);
                const float2 czq = make_float2(cz, cz);
                if (damp) p = pmul2(pmul2(p, cxq), czq);   // damping of U(t-1) deferred to this read
                const float2 base = fsub2(padd2(uc, uc), p);   // 2 U(t) - U(t-1)
                float2 o;
                if (APPROX == kAcoustic) {
                    o = pfma2(k, padd2(pxx2[q], pzz2[q]), base);
                } else {
                    const float2 px = px2v[q], pz = pz2v[q];
                    const float2 pxxe = pxx2[q], pzze = pzz2[q];
                    const float2 e2 = q == 0 ? lo2(e4) : hi2(e4);   // 1 + 2 eps
                    const float2 m1 = q == 0 ? lo2(n4) : hi2(n4);   // -2 (eps - delta)
                    const float2 m2 = q == 0 ? lo2(b4) : hi2(b4);   // 2 (1 + delta)
                    float2 sx_ = px, sz_ = pz, ca, sa;
                    if (APPROX == kTTI) {
                        ca = q == 0 ? lo2(c4) : hi2(c4);
                        sa = q == 0 ? lo2(s4) : hi2(s4);
                        sx_ = pfma2(px, ca, neg2(pmul2(pz, sa)));
                        sz_ = pfma2(px, sa, pmul2(pz, ca));
                    }
                    // Sd of cpp/Modeling.cu:605-611 (VTI) and :719-727 (TTI), switched
                    // on where |den| > 1e-12: the reference's products in its
                    // written order, its sums contracted as the compiler does
                    const float2 px2 = pmul2(sx_, sx_), pz2 = pmul2(sz_, sz_);
                    const float2 num = pmul2(pmul2(m1, px2), pz2);
                    float2 den;
                    if (APPROX == kVTI) {
                        // (1 + 2 eps) (px px px px) + (pz pz pz pz) + 2 (1 + delta) (px px) (pz pz)
                        const float2 p4x = pmul2(pmul2(px2, sx_), sx_), p4z = pmul2(pmul2(pz2, sz_), sz_);
                        den = pfma2(pmul2(m2, px2), pz2, pfma2(e2, p4x, p4z));
                    } else {
                        // (1 + 2 eps) xr2 xr2 + zr2 zr2 + 2 (1 + delta) xr2 zr2
                        den = pfma2(pmul2(m2, px2), pz2, pfma2(pmul2(e2, px2), px2, pmul2(pz2, pz2)));
                    }
                    const float2 sd = make_float2(sd_ratio(num.x, den.x), sd_ratio(num.y, den.y));
                    if (APPROX == kVTI) {
                        const float2 ax = pmul2(k, padd2(e2, sd));
                        const float2 az = pmul2(k, padd2(make_float2(1.f, 1.f), sd));
                        o = pfma2(az, pzze, pfma2(ax, pxxe, base));   // the pxx term first, as written
                    } else {
                        const float2 c2 = pmul2(ca, ca), s2 = pmul2(sa, sa);
                        const float2 ax = pmul2(k, padd2(pfma2(e2, c2, s2), sd));
                        const float2 az = pmul2(k, padd2(pfma2(e2, s2, c2), sd));
                        // -2 eps kappa sin(2 theta) pxz = (1 - e2) kappa 2 s c pxz
                        const float2 hs = pmul2(fsub2(make_float2(1.f, 1.f), e2),
                                                     pmul2(k, pmul2(padd2(sa, sa), ca)));
                        o = pfma2(hs, pxz2[q], pfma2(az, pzze, pfma2(ax, pxxe, base)));   // in written order
                    }
                }
                if (damp) o = pmul2(pmul2(o, cxq), czq);
                outp[q] = o;
            }
            float out[4] = {outp[0].x, outp[0].y, outp[1].x, outp[1].y};
            if (r == sz) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j == sx) out[j] += a.src_amp;
            }
            if (!live) {
            } else if (!EDGE || (x0 >= 4 && x0 + 3 < a.nx - 4)) {
                *reinterpret_cast<float4*>(PAM_CHK(nxt + ro, a.nxt, fbytes, 16, 16)) =
                    make_float4(out[0], out[1], out[2], out[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j >= 4 && x0 + j < a.nx - 4) *PAM_CHK(&nxt[ro + j], a.nxt, fbytes, 4, 17) = out[j];
            }
        }
    };

    // The march down the segment: register window w[0..7] = rows r-4 .. r+3,
    // row r+4 arriving through the ring; U rows per trip, then the window
    // shifts by U rows.  The rows past z1 in the last trip (at most U - 1;
    // interior marches only, so no damping or strip reads) read only the ring,
    // whose addresses are clamped to the field, and are not stored.
    auto march = [&](auto edge_tag, auto unroll_tag) {
        constexpr int U = decltype(unroll_tag)::value;
        static_assert(U >= 1 && U <= 8, "rows per trip");
        float4 w[8 + U];
#pragma unroll
        for (int i = 0; i < 8; i++)
            w[i] = ldg4(PAM_CHK(cur + (long long)min(z0 - 4 + i, zmax) * P, a.cur, fbytes, 16, 10));
        for (int r = z0; r < z1; r += U) {
#pragma unroll
            for (int j = 0; j < U; j++)
                row(edge_tag, r + j, j == 0 || r + j < z1, w[j], w[j + 1], w[j + 2], w[j + 3], w[j + 4], w[j + 5],
                    w[j + 6], w[j + 7], w[j + 8]);
#pragma unroll
            for (int i = 0; i < 8; i++) w[i] = w[i + U];
        }
    };
    // Edge warps: the tile reaches into an x border or the segment into a z
    // border (only those rows carry damping or strip terms, and only x-border
    // tiles have columns outside [4, nx - 4)).
    const bool edge = xborder || z0 < a.N || z1 > a.nz - a.N;
    if (edge) march(IntTag<1>{}, IntTag<1>{});
    else march(IntTag<0>{}, IntTag<interior_unroll<APPROX>()>{});
    cp_async_wait<0>();
}

template <int APPROX, int BC>
__global__ void __launch_bounds__(128, step_min_blocks<APPROX>()) step_kernel(const StepArgs a)
{
    step_body<APPROX, BC>(a);
}

// ---------------------------------------------------------------------------
// CPML memory variables (src/utils.py:242-377): psi = a psi + b dU, then
// zeta = a zeta + b (d2U + d psi_new), for every strip cell, and the terms the
// stepping kernel adds: (d psi_new, d psi_new + zeta_new).  psi and zeta are
// zero outside their strip, so each strip row (x) or strip column (z) is
// self-contained.

// x strips: one thread per strip cell.  A block covers `rows` whole strip
// rows of one (shot, side) - blockDim.x = the strip width rounded up to 8,
// blockDim.y = rows - so every thread issues its loads at once, and psi_new
// goes through shared memory (four zero cells on each side of a row, psi
// being zero outside the strip) for its x derivative.
struct CpmlXShape {
    int bx, rows;
};
__host__ __device__ inline CpmlXShape cpml_x_shape(int N) {
    const int W = N - 4;
    const int bx = (W + 7) / 8 * 8;
    int rows = 256 / bx;
    if (rows < 1) rows = 1;
    return CpmlXShape{bx, rows};
}

static __global__ void __launch_bounds__(256) cpml_x_kernel(const CpmlArgs a)
{
    extern __shared__ float xsm[];                  // [rows][bx + 8]
    // grid: (side, row block, shot)
    const CpmlXShape sh = cpml_x_shape(a.N);
    const int W = a.N - 4;
    const int side = blockIdx.x, rb = blockIdx.y, shot = blockIdx.z;
    const int i = threadIdx.x, ty = threadIdx.y;
    const int z = 4 + rb * sh.rows + ty;
    const bool valid = i < W && z < a.nz - 4;
    float* srow = xsm + ty * (sh.bx + 8);
    const int xbeg = side == 0 ? 4 : a.nx - a.N;    // first strip column
    const int cbeg = side == 0 ? 4 : a.N;           // its index in the [2N] strip row
    float pxx = 0.0f, zeta_old = 0.0f;
    float2 ab = make_float2(0.0f, 0.0f);
    long long so = 0;
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long sbytes = (long long)a.B * a.xs_stride * 4;   // psi_x, zeta_x (xaux: twice)
    if (valid) {
        // U[-4 .. 4] of the strip cell
        const float* U = PAM_CHK(a.cur + (long long)shot * a.shot_stride + (long long)z * a.P + xbeg + i - 4, a.cur,
                                 fbytes, 36, 20) + 4;
        so = (long long)shot * a.xs_stride + (long long)z * (2 * a.N) + cbeg + i;
        const float u0 = U[0], up1 = U[1], um1 = U[-1], up2 = U[2], um2 = U[-2];
        const float up3 = U[3], um3 = U[-3], up4 = U[4], um4 = U[-4];
        ab = *PAM_CHK(&a.cxab[(long long)z * (2 * a.N) + cbeg + i], a.cxab, a.xs_stride * 8, 8, 21);
        const float ps_old = *PAM_CHK(&a.psix[so], a.psix, sbytes, 4, 22);
        zeta_old = *PAM_CHK(&a.zetax[so], a.zetax, sbytes, 4, 22);
        const float px =
            (kA1 * (up1 - um1) + kA2 * (up2 - um2) + kA3 * (up3 - um3) + kA4 * (up4 - um4)) * a.inv_dx;
        pxx = (kC0 * u0 + kC1 * (up1 + um1) + kC2 * (up2 + um2) + kC3 * (up3 + um3) + kC4 * (up4 + um4)) *
              a.inv_dx2;
        const float ps = ab.x * ps_old + ab.y * px;
        *PAM_CHK(&a.psix[so], a.psix, sbytes, 4, 22) = ps;
        srow[i + 4] = ps;
    } else if (i < sh.bx) {
        srow[i + 4] = 0.0f;
    }
    if (i < 4) { srow[i] = 0.0f; srow[sh.bx + 4 + i] = 0.0f; }
    __syncthreads();
    if (!valid) return;
    const float* sr = srow + i + 4;
    const float dps = (kA1 * (sr[1] - sr[-1]) + kA2 * (sr[2] - sr[-2]) + kA3 * (sr[3] - sr[-3]) +
                       kA4 * (sr[4] - sr[-4])) * a.inv_dx;
    const float ze = ab.x * zeta_old + ab.y * (pxx + dps);
    *PAM_CHK(&a.zetax[so], a.zetax, sbytes, 4, 23) = ze;
    *PAM_CHK(&a.xaux[so], a.xaux, 2 * sbytes, 8, 23) = make_float2(dps, dps + ze);
}

// x strips of an even border width (N even, hence an even strip width W and
// even strip-row offsets): one thread per pair of x-adjacent strip cells, so
// psi, zeta, the (a, b) pairs and the strip terms move as 8- and 16-byte
// accesses and U's ten taps of the pair are read once; per cell the same
// expressions as cpml_x_kernel.  A block covers `rows` strip rows of one
// (shot, side): blockDim = (pairs per row rounded up to 8, rows).
struct CpmlXPairShape {
    int bx, rows;
};
__host__ __device__ inline CpmlXPairShape cpml_x_pair_shape(int N) {
    const int pairs = (N - 4) / 2;
    const int bx = (pairs + 7) / 8 * 8;
    int rows = 256 / bx;
    if (rows < 1) rows = 1;
    return CpmlXPairShape{bx, rows};
}

static __global__ void __launch_bounds__(256) cpml_x_pair_kernel(const CpmlArgs a)
{
    extern __shared__ float xpsm[];                 // [rows][2 bx + 8]
    // grid: (side, row block, shot)
    const CpmlXPairShape sh = cpml_x_pair_shape(a.N);
    const int pairs = (a.N - 4) / 2;
    const int side = blockIdx.x, rb = blockIdx.y, shot = blockIdx.z;
    const int j = threadIdx.x, ty = threadIdx.y;
    const int i = 2 * j;                            // first strip column of the pair
    const int z = 4 + rb * sh.rows + ty;
    const bool valid = j < pairs && z < a.nz - 4;
    float* srow = xpsm + ty * (2 * sh.bx + 8);
    const int xbeg = side == 0 ? 4 : a.nx - a.N;    // first strip column
    const int cbeg = side == 0 ? 4 : a.N;           // its index in the [2N] strip row
    float pxx0 = 0.0f, pxx1 = 0.0f;
    float2 zeta_old = make_float2(0.0f, 0.0f);
    float4 ab = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    long long so = 0;
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long sbytes = (long long)a.B * a.xs_stride * 4;
    if (valid) {
        // U[-4 .. 5] around the pair (cell 0 at u[4], cell 1 at u[5])
        const float* U = PAM_CHK(a.cur + (long long)shot * a.shot_stride + (long long)z * a.P + xbeg + i - 4, a.cur,
                                 fbytes, 40, 24);
        float u[10];
#pragma unroll
        for (int k = 0; k < 10; k++) u[k] = U[k];
        so = (long long)shot * a.xs_stride + (long long)z * (2 * a.N) + cbeg + i;
        ab = *reinterpret_cast<const float4*>(
            PAM_CHK(&a.cxab[(long long)z * (2 * a.N) + cbeg + i], a.cxab, a.xs_stride * 8, 16, 25));
        const float2 ps_old = *reinterpret_cast<const float2*>(PAM_CHK(&a.psix[so], a.psix, sbytes, 8, 26));
        zeta_old = *reinterpret_cast<const float2*>(PAM_CHK(&a.zetax[so], a.zetax, sbytes, 8, 26));
        const float px0 = (kA1 * (u[5] - u[3]) + kA2 * (u[6] - u[2]) + kA3 * (u[7] - u[1]) + kA4 * (u[8] - u[0])) *
                          a.inv_dx;
        const float px1 = (kA1 * (u[6] - u[4]) + kA2 * (u[7] - u[3]) + kA3 * (u[8] - u[2]) + kA4 * (u[9] - u[1])) *
                          a.inv_dx;
        pxx0 = (kC0 * u[4] + kC1 * (u[5] + u[3]) + kC2 * (u[6] + u[2]) + kC3 * (u[7] + u[1]) + kC4 * (u[8] + u[0])) *
               a.inv_dx2;
        pxx1 = (kC0 * u[5] + kC1 * (u[6] + u[4]) + kC2 * (u[7] + u[3]) + kC3 * (u[8] + u[2]) + kC4 * (u[9] + u[1])) *
               a.inv_dx2;
        const float ps0 = ab.x * ps_old.x + ab.y * px0;
        const float ps1 = ab.z * ps_old.y + ab.w * px1;
        *reinterpret_cast<float2*>(PAM_CHK(&a.psix[so], a.psix, sbytes, 8, 26)) = make_float2(ps0, ps1);
        srow[i + 4] = ps0;
        srow[i + 5] = ps1;
    } else if (j < sh.bx) {
        srow[i + 4] = 0.0f;                         // psi is zero past the strip
        srow[i + 5] = 0.0f;
    }
    if (j < 4) { srow[j] = 0.0f; srow[2 * sh.bx + 4 + j] = 0.0f; }
    __syncthreads();
    if (!valid) return;
    const float* sr = srow + i + 4;                 // cell 0 at sr[0], cell 1 at sr[1]
    const float dps0 = (kA1 * (sr[1] - sr[-1]) + kA2 * (sr[2] - sr[-2]) + kA3 * (sr[3] - sr[-3]) +
                        kA4 * (sr[4] - sr[-4])) * a.inv_dx;
    const float dps1 = (kA1 * (sr[2] - sr[0]) + kA2 * (sr[3] - sr[-1]) + kA3 * (sr[4] - sr[-2]) +
                        kA4 * (sr[5] - sr[-3])) * a.inv_dx;
    const float ze0 = ab.x * zeta_old.x + ab.y * (pxx0 + dps0);
    const float ze1 = ab.z * zeta_old.y + ab.w * (pxx1 + dps1);
    *reinterpret_cast<float2*>(PAM_CHK(&a.zetax[so], a.zetax, sbytes, 8, 27)) = make_float2(ze0, ze1);
    *reinterpret_cast<float4*>(PAM_CHK(&a.xaux[so], a.xaux, 2 * sbytes, 16, 27)) =
        make_float4(dps0, dps0 + ze0, dps1, dps1 + ze1);
}

// z strips: a block covers 32 columns and the whole strip height of one
// (shot, side); each thread owns R consecutive strip rows of one column
// (blockDim = (32, ceil(W / R))), so it reads the R + 8 rows of U its
// stencils need once.  All loads of a thread are issued before its
// arithmetic; psi_new goes through shared memory (four zero rows above and
// below the strip) for its z derivative.
constexpr int kCpmlZCols = 32;

__host__ __device__ inline int cpml_z_rows_per_thread(int N) { return N - 4 <= 6 * 32 ? 6 : 8; }
__host__ __device__ inline int cpml_z_block_rows(int N) {
    const int R = cpml_z_rows_per_thread(N);
    return (N - 4 + R - 1) / R;
}

template <int R>
__global__ void __launch_bounds__(1024) cpml_z_kernel(const CpmlArgs a)
{
    extern __shared__ float zsm[];                  // [by * R + 8][32]
    // grid: (column slab, side, shot)
    const int W = a.N - 4;
    const int slab = blockIdx.x, side = blockIdx.y, shot = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y, by = blockDim.y;
    const int x = 4 + slab * kCpmlZCols + tx;
    const bool xv = x < a.nx - 4;
    const int zbeg = side == 0 ? 4 : a.nz - a.N;    // first strip row
    const int rbeg = side == 0 ? 4 : a.N;           // its index in the [2N] strip rows
    const long long P = a.P;
    const int i0 = ty * R;                          // first strip row of this thread
    const int n = min(R, W - i0);                   // rows it owns (may be <= 0)
    const float* U = a.cur + (long long)shot * a.shot_stride + (long long)(zbeg + i0) * P + x;
    const long long so = (long long)shot * a.zs_stride + (long long)(rbeg + i0) * P + x;
    const float2* abp = a.czab + (long long)(rbeg + i0) * P + x;

    if (ty == 0)
#pragma unroll
        for (int r = 0; r < 4; r++) zsm[r * kCpmlZCols + tx] = 0.0f;
    float u[R + 8], ps_old[R], ze_old[R];
    float2 ab[R];
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long sbytes = (long long)a.B * a.zs_stride * 4;   // psi_z, zeta_z (zaux: twice)
    if (xv && n > 0) {
#pragma unroll
        for (int j = 0; j < R + 8; j++)
            if (j < n + 8) u[j] = *PAM_CHK(&U[(long long)(j - 4) * P], a.cur, fbytes, 4, 30);
#pragma unroll
        for (int k = 0; k < R; k++)
            if (k < n) {
                ps_old[k] = *PAM_CHK(&a.psiz[so + k * P], a.psiz, sbytes, 4, 31);
                ze_old[k] = *PAM_CHK(&a.zetaz[so + k * P], a.zetaz, sbytes, 4, 31);
                ab[k] = *PAM_CHK(&abp[k * P], a.czab, a.zs_stride * 8, 8, 32);
            }
    }
    float pzz[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        if (k >= n) break;
        float psn = 0.0f;
        if (xv) {
            const float* v = u + k;
            const float pz = (kA1 * (v[5] - v[3]) + kA2 * (v[6] - v[2]) + kA3 * (v[7] - v[1]) +
                              kA4 * (v[8] - v[0])) * a.inv_dz;
            pzz[k] = (kC0 * v[4] + kC1 * (v[5] + v[3]) + kC2 * (v[6] + v[2]) + kC3 * (v[7] + v[1]) +
                      kC4 * (v[8] + v[0])) * a.inv_dz2;
            psn = ab[k].x * ps_old[k] + ab[k].y * pz;
            *PAM_CHK(&a.psiz[so + k * P], a.psiz, sbytes, 4, 31) = psn;
        }
        zsm[(i0 + k + 4) * kCpmlZCols + tx] = psn;
    }
    // rows W .. by*R + 7 of the buffer: the zero rows below the strip and the
    // unused tail of the last thread row
    for (int r = W + 4 + ty; r < by * R + 8; r += by) zsm[r * kCpmlZCols + tx] = 0.0f;
    __syncthreads();
    if (!xv) return;
#pragma unroll
    for (int k = 0; k < R; k++) {
        if (k >= n) break;
        const float* c = zsm + (i0 + k + 4) * kCpmlZCols + tx;
        const int s = kCpmlZCols;
        const float dps = (kA1 * (c[s] - c[-s]) + kA2 * (c[2 * s] - c[-2 * s]) + kA3 * (c[3 * s] - c[-3 * s]) +
                           kA4 * (c[4 * s] - c[-4 * s])) * a.inv_dz;
        const float ze = ab[k].x * ze_old[k] + ab[k].y * (pzz[k] + dps);
        *PAM_CHK(&a.zetaz[so + k * P], a.zetaz, sbytes, 4, 33) = ze;
        *PAM_CHK(&a.zaux[so + k * P], a.zaux, 2 * sbytes, 8, 33) = make_float2(dps, dps + ze);
    }
}

// z strips in pairs of columns: a block covers 32 columns (16 pairs) and the
// whole strip height of one (shot, side), each thread 3 consecutive strip
// rows of one pair of columns (blockDim = (16, ceil(W / 3)), at most 64 rows,
// so strips up to 192 cells high), reading the 11 rows of U its stencils need
// as 8-byte pairs; psi, zeta and the strip terms move as 8- and 16-byte
// accesses.  Per cell the same expressions as cpml_z_kernel.
constexpr int kCpmlZPairRows = 3;

__host__ __device__ inline int cpml_z_pair_block_rows(int N) {
    return (N - 4 + kCpmlZPairRows - 1) / kCpmlZPairRows;
}
__host__ __device__ inline bool cpml_z_pairs_usable(int N) { return cpml_z_pair_block_rows(N) <= 64; }

static __global__ void __launch_bounds__(1024) cpml_z_pair_kernel(const CpmlArgs a)
{
    constexpr int R = kCpmlZPairRows;
    extern __shared__ float zpsm[];                 // [by * R + 8][32]
    // grid: (column slab, side, shot)
    const int W = a.N - 4;
    const int slab = blockIdx.x, side = blockIdx.y, shot = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y, by = blockDim.y;
    const int x = 4 + slab * kCpmlZCols + 2 * tx;   // first column of the pair (even)
    const bool xv0 = x < a.nx - 4, xv1 = x + 1 < a.nx - 4;
    const int zbeg = side == 0 ? 4 : a.nz - a.N;    // first strip row
    const int rbeg = side == 0 ? 4 : a.N;           // its index in the [2N] strip rows
    const long long P = a.P;
    const int i0 = ty * R;                          // first strip row of this thread
    const int n = min(R, W - i0);                   // rows it owns (may be <= 0)
    const float* U = a.cur + (long long)shot * a.shot_stride + (long long)(zbeg + i0) * P + x;
    const long long so = (long long)shot * a.zs_stride + (long long)(rbeg + i0) * P + x;
    const float2* abp = a.czab + (long long)(rbeg + i0) * P + x;

    if (ty == 0)
#pragma unroll
        for (int r = 0; r < 4; r++) *reinterpret_cast<float2*>(&zpsm[r * kCpmlZCols + 2 * tx]) = make_float2(0.f, 0.f);
    float2 u[R + 8], ps_old[R], ze_old[R];
    float4 ab[R];
    [[maybe_unused]] const long long fbytes = (long long)a.B * a.shot_stride * 4;
    [[maybe_unused]] const long long sbytes = (long long)a.B * a.zs_stride * 4;
    if (xv0 && n > 0) {
#pragma unroll
        for (int j = 0; j < R + 8; j++)
            if (j < n + 8)
                u[j] = *reinterpret_cast<const float2*>(PAM_CHK(&U[(long long)(j - 4) * P], a.cur, fbytes, 8, 34));
#pragma unroll
        for (int k = 0; k < R; k++)
            if (k < n) {
                ps_old[k] = *reinterpret_cast<const float2*>(PAM_CHK(&a.psiz[so + k * P], a.psiz, sbytes, 8, 35));
                ze_old[k] = *reinterpret_cast<const float2*>(PAM_CHK(&a.zetaz[so + k * P], a.zetaz, sbytes, 8, 35));
                ab[k] = *reinterpret_cast<const float4*>(PAM_CHK(&abp[k * P], a.czab, a.zs_stride * 8, 16, 36));
            }
    }
    float2 pzz[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        if (k >= n) break;
        float2 psn = make_float2(0.f, 0.f);
        if (xv0) {
            const float2* v = u + k;
            const float pz0 = (kA1 * (v[5].x - v[3].x) + kA2 * (v[6].x - v[2].x) + kA3 * (v[7].x - v[1].x) +
                               kA4 * (v[8].x - v[0].x)) * a.inv_dz;
            const float pz1 = (kA1 * (v[5].y - v[3].y) + kA2 * (v[6].y - v[2].y) + kA3 * (v[7].y - v[1].y) +
                               kA4 * (v[8].y - v[0].y)) * a.inv_dz;
            pzz[k].x = (kC0 * v[4].x + kC1 * (v[5].x + v[3].x) + kC2 * (v[6].x + v[2].x) + kC3 * (v[7].x + v[1].x) +
                        kC4 * (v[8].x + v[0].x)) * a.inv_dz2;
            pzz[k].y = (kC0 * v[4].y + kC1 * (v[5].y + v[3].y) + kC2 * (v[6].y + v[2].y) + kC3 * (v[7].y + v[1].y) +
                        kC4 * (v[8].y + v[0].y)) * a.inv_dz2;
            psn.x = ab[k].x * ps_old[k].x + ab[k].y * pz0;
            psn.y = ab[k].z * ps_old[k].y + ab[k].w * pz1;
            if (xv1) *reinterpret_cast<float2*>(PAM_CHK(&a.psiz[so + k * P], a.psiz, sbytes, 8, 35)) = psn;
            else *PAM_CHK(&a.psiz[so + k * P], a.psiz, sbytes, 4, 35) = psn.x;
        }
        *reinterpret_cast<float2*>(&zpsm[(i0 + k + 4) * kCpmlZCols + 2 * tx]) = psn;
    }
    // rows W + 4 .. by * R + 7: the zero rows below the strip and the unused
    // tail of the last thread row
    for (int r = W + 4 + ty; r < by * R + 8; r += by)
        *reinterpret_cast<float2*>(&zpsm[r * kCpmlZCols + 2 * tx]) = make_float2(0.f, 0.f);
    __syncthreads();
    if (!xv0) return;
#pragma unroll
    for (int k = 0; k < R; k++) {
        if (k >= n) break;
        const float* c = zpsm + (i0 + k + 4) * kCpmlZCols + 2 * tx;
        constexpr int s = kCpmlZCols;
        auto L = [&](int off) { return *reinterpret_cast<const float2*>(c + off); };
        const float2 p1 = L(s), m1 = L(-s), p2 = L(2 * s), m2 = L(-2 * s);
        const float2 p3 = L(3 * s), m3 = L(-3 * s), p4 = L(4 * s), m4 = L(-4 * s);
        const float dps0 = (kA1 * (p1.x - m1.x) + kA2 * (p2.x - m2.x) + kA3 * (p3.x - m3.x) + kA4 * (p4.x - m4.x)) *
                           a.inv_dz;
        const float dps1 = (kA1 * (p1.y - m1.y) + kA2 * (p2.y - m2.y) + kA3 * (p3.y - m3.y) + kA4 * (p4.y - m4.y)) *
                           a.inv_dz;
        const float ze0 = ab[k].x * ze_old[k].x + ab[k].y * (pzz[k].x + dps0);
        const float ze1 = ab[k].z * ze_old[k].y + ab[k].w * (pzz[k].y + dps1);
        if (xv1) {
            *reinterpret_cast<float2*>(PAM_CHK(&a.zetaz[so + k * P], a.zetaz, sbytes, 8, 37)) = make_float2(ze0, ze1);
            *reinterpret_cast<float4*>(PAM_CHK(&a.zaux[so + k * P], a.zaux, 2 * sbytes, 16, 37)) =
                make_float4(dps0, dps0 + ze0, dps1, dps1 + ze1);
        } else {
            *PAM_CHK(&a.zetaz[so + k * P], a.zetaz, sbytes, 4, 37) = ze0;
            *PAM_CHK(&a.zaux[so + k * P], a.zaux, 2 * sbytes, 8, 37) = make_float2(dps0, dps0 + ze0);
        }
    }
}

// ---------------------------------------------------------------------------
// Receiver recording (cpp/Modeling.cu:488-497): seis[b][t][r] = D * U(t) at
// the receiver cell, D the Cerjan factor there (1 for CPML and the interior).

__device__ __forceinline__ void record_sample(const RecordArgs& a, long long i)
{
    if (i >= (long long)a.nrec * a.B) return;
    const int r = (int)(i % a.nrec);
    const int b = (int)(i / a.nrec);
    const long long ri = a.per_shot ? (long long)b * a.nrec + r : r;
    [[maybe_unused]] const long long rbytes = (long long)(a.per_shot ? a.B : 1) * a.nrec * 4;
    const int z = *PAM_CHK(&a.rz[ri], a.rz, rbytes, 4, 40), x = *PAM_CHK(&a.rx[ri], a.rx, rbytes, 4, 40);
    float v = *PAM_CHK(&a.cur[(long long)b * a.shot_stride + (long long)z * a.P + x], a.cur,
                       (long long)a.B * a.shot_stride * 4, 4, 41);
    if (a.cerjan_on && z >= 4 && z < a.nz - 4 && x >= 4 && x < a.nx - 4) {
        if (x < a.N) v = v * a.cerjan[x];
        if (x >= a.nx - a.N) v = v * a.cerjan[a.nx - 1 - x];
        if (z < a.N) v = v * a.cerjan[z];
        if (z >= a.nz - a.N) v = v * a.cerjan[a.nz - 1 - z];
    }
    *PAM_CHK(&a.seis[((long long)b * a.nt_data + a.it) * a.nrec + r], a.seis, (long long)a.B * a.nt_data * a.nrec * 4,
             4, 42) = v;
    if (!isfinite(v)) atomicOr(a.status, 1);   // an unstable scheme overflows the fields
}

static __global__ void record_kernel(const RecordArgs a)
{
    record_sample(a, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// The forward time loop of a small batch in one cooperative launch: steps
// k0 .. k1-1, each the warps' step_body, the recording of U(k) by the first
// nrec * B threads of the grid, and a grid-wide barrier (a cooperative launch
// keeps every block resident, so each barrier is reached by all of them).
// For runs whose steps are so short that one CUDA-graph launch per kernel
// and step dominates (the single-shot plain case: about 3 us of a 5.7 us
// step); larger batches keep the graph of one-step launches.
struct PersistArgs {
    StepArgs base;                  // cur / nxt / src_amp set per step
    float* u[2];                    // the two field buffers: U(k) in u[k & 1]
    const float* __restrict__ wavelet;   // [nt]
    RecordArgs rec;                 // it set per step; seis == nullptr: no recording
    int nt, itlag, k0, k1;
};

template <int APPROX, int BC>
__global__ void __launch_bounds__(128, step_min_blocks<APPROX>()) step_persistent_kernel(const PersistArgs p)
{
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (int k = p.k0; k < p.k1; k++) {
        StepArgs a = p.base;
        a.cur = p.u[k & 1];
        a.nxt = p.u[(k + 1) & 1];
        a.prev = nullptr;
        a.src_amp = k + 1 < p.nt ? p.wavelet[k + 1] : 0.0f;
        if (k >= p.itlag && p.rec.seis) {
            RecordArgs r = p.rec;
            r.cur = a.cur;
            r.it = k - p.itlag;
            record_sample(r, gtid);
        }
        step_body<APPROX, BC>(a);
        grid.sync();
    }
}

// Writes the first wavelet sample at each shot's source cell (the injection
// of step 0, cpp/Modeling.cu:447); fields are zeroed beforehand.
// Source indices of the device entry point are not host-validated, so the
// kernel skips any cell outside the update region instead of writing it.
static __global__ void inject_first_kernel(float* __restrict__ cur, const int* __restrict__ sz, const int* __restrict__ sx,
                                    float amp, int B, int P, long long shot_stride, int nz, int nx)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const int z = sz[b], x = sx[b];
    if (z < 4 || z >= nz - 4 || x < 4 || x >= nx - 4) return;
    cur[(long long)b * shot_stride + (long long)z * P + x] += amp;
}

}  // namespace pam
