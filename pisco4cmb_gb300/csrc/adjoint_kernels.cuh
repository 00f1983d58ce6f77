// adjoint_kernels.cuh -- the adjoint's kernels: transpose of the TUNED
// forward, TOD residuals back-projected onto the sky I/Q/U/V maps and
// (optionally) onto the beam maps or the Gaussian beam's parameters.
// Included by adjoint.cu (kernels that build each sample's plan in the warp)
// and adjoint_planned.cu (kernels that read plans built beforehand), so the
// two sets compile in parallel.
////
// The forward is linear in the sky and in the beam:
//   tod_a(s) = sum_p I a0 + Q (a1 c2 - a2 s2) + U (a2 c2 + a1 s2) + V a3
//   tod_b(s) = sum_p I b0 + Q (-b1 c2 + b2 s2) + U (-b2 c2 - b1 s2) + V b3
// (convolver.cpp:195-202 with the GPU's V term, cudaConv2.cu:204,214), so
//   dL/dI(p) += ga a0 + gb b0,  dL/dQ(p) += ga (a1 c2 - a2 s2) + gb (-b1 c2 + b2 s2), ...
//   dL/da0(b) += ga I, dL/da1(b) += ga (Q c2 + U s2), dL/da2(b) += ga (U c2 - Q s2), ...
// for every pair (s, p) with beam pixel b, with the pair set and the beam
// pixel of each pair taken by exactly the TUNED forward's geometry
// (tuned_core.cuh), so the adjoint is the transpose of that operator.  With
// the bilinear lookup the pair's beam value is sum_i w_i beam[b_i], and its
// beam gradient goes to the stencil pixels b_i by the weights w_i.
//
// Accumulation, two variants:
//  * ATOMIC: float atomics (vector float4 adds for the sky) -- fast, but the
//    order of the additions, hence the last bits, varies run to run.
//  * DETERMINISTIC: 64-bit fixed-point integer atomics.  Integer addition is
//    associative, so the sums are bit-identical whatever the order.  The
//    scale 2^S is set from a rigorous bound on any total (computed by fixed-
//    order reductions), leaving 2^-62 of that bound as the resolution; the
//    per-pixel error is at most (#contributions x 2^-S) / 2.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "tuned_core.cuh"

namespace pisco {
namespace {

constexpr int kAW = PISCO_TUNED_WARPS;

// Queued pairs are redone after the sample has moved on, so the weights
// (ga, gb) of their sample travel in its slot (stash / deferred).
template <bool kFixed>
struct Scatter {
    static constexpr bool kSums = false;
    static constexpr bool kStencil = false;  // the sky gradient needs the interpolated value only
    float ga, gb;
    float* gsky;                  // ATOMIC: float4-interleaved [npix][4]
    unsigned long long* gsky_fx;  // DETERMINISTIC: int64 planes [4][npix]
    float* gbeam;                 // ATOMIC: [npixB][8] (a.IQUV, b.IQUV) or null
    unsigned long long* gbeam_fx;
    const float4* sky;            // for the beam gradient
    float ssky, sbeam;            // fixed-point scales 2^S (at most 2^126)
    int want_v;                   // accumulate the V column
    long long plane;              // npix: the stride of the fixed-point planes

    // v 2^S rounded to the nearest integer.  The scale is a power of two, so
    // the FP32 product is exact and the FP32 -> int64 conversion gives what
    // the FP64 route would, without two FP64 instructions per component (the
    // FP64 pipe of this GPU issues a small fraction of the FP32 rate).
    __device__ __forceinline__ static unsigned long long fx(float v, float scale)
    {
        return (unsigned long long)__float2ll_rn(v * scale);
    }

    __device__ __forceinline__ void stash(tuned::Pend& p) const
    {
        p.ga = ga;
        p.gb = gb;
    }
    __device__ __forceinline__ void deferred(const tuned::Pend& p, int pix, const F8& B, int,
                                            float c2, float s2, float&, float&) const
    {
        scatter(p.ga, p.gb, pix, B, c2, s2);
    }
    __device__ __forceinline__ int fetch(int) const { return 0; }
    __device__ __forceinline__ void pair(int pix, int, const F8& B, int, float c2, float s2) const
    {
        scatter(ga, gb, pix, B, c2, s2);
    }

    __device__ __forceinline__ void scatter(float wa, float wb, int pix, const F8& B, float c2,
                                           float s2) const
    {
        const float gI = wa * B.a.x + wb * B.b.x;
        const float gQ = wa * (B.a.y * c2 - B.a.z * s2) + wb * (-B.b.y * c2 + B.b.z * s2);
        const float gU = wa * (B.a.z * c2 + B.a.y * s2) + wb * (-B.b.z * c2 - B.b.y * s2);
        const float gV = want_v ? wa * B.a.w + wb * B.b.w : 0.0f;
        if (kFixed) {
            // one plane per Stokes component: the lanes of a warp, on
            // consecutive pixels of a ring, add to consecutive words
            unsigned long long* p = gsky_fx + pix;
            atomicAdd(p, fx(gI, ssky));
            atomicAdd(p + plane, fx(gQ, ssky));
            atomicAdd(p + 2 * plane, fx(gU, ssky));
            if (want_v) atomicAdd(p + 3 * plane, fx(gV, ssky));
        } else {
            atomicAdd(reinterpret_cast<float4*>(gsky) + pix, make_float4(gI, gQ, gU, gV));
        }
    }
};

// Sky and beam gradient: with the nearest lookup the action gets the beam
// pixel bp with its value; with the bilinear one it gets the stencil and
// spreads each pair's beam gradient over its (up to) four pixels by their
// weights.
template <bool kFixed>
struct ScatterBeam {
    static constexpr bool kSums = false;
    static constexpr bool kStencil = true;
    float ga, gb;
    const F8* beam_base;
    const float4* sky;
    float* gsky;
    unsigned long long* gsky_fx;
    float* gbeam;
    unsigned long long* gbeam_fx;
    float ssky, sbeam;
    int want_sky;
    int want_v;
    long long plane;

    __device__ __forceinline__ void stash(tuned::Pend& p) const
    {
        p.ga = ga;
        p.gb = gb;
    }
    __device__ __forceinline__ void deferred(const tuned::Pend& p, int pix, const F8& B, int bp,
                                            float c2, float s2, float&, float&) const
    {
        scatter(p.ga, p.gb, pix, fetch(pix), B, bp, c2, s2);
    }
    __device__ __forceinline__ float4 fetch(int pix) const { return __ldg(&sky[pix]); }
    __device__ __forceinline__ void pair(int pix, const float4& S, const F8& B, int bp, float c2,
                                         float s2) const
    {
        scatter(ga, gb, pix, S, B, bp, c2, s2);
    }

    __device__ __forceinline__ void pair_stencil(int pix, const float4& S, const int px[4],
                                                 const float w[4], float c2, float s2) const
    {
        scatter_stencil(ga, gb, pix, S, px, w, c2, s2);
    }
    __device__ __forceinline__ void deferred_stencil(const tuned::Pend& p, int pix, const int px[4],
                                                     const float w[4], float c2, float s2) const
    {
        scatter_stencil(p.ga, p.gb, pix, fetch(pix), px, w, c2, s2);
    }

    // d(tod)/d(beam) of one pair, times the TOD weights: 8 values (a.IQUV, b.IQUV)
    __device__ __forceinline__ static void beam_grad(float wa, float wb, const float4& S, float c2,
                                                     float s2, float v[8])
    {
        const float qa = S.y * c2 + S.z * s2, ua = S.z * c2 - S.y * s2;
        v[0] = wa * S.x; v[1] = wa * qa; v[2] = wa * ua; v[3] = wa * S.w;
        v[4] = wb * S.x; v[5] = -wb * qa; v[6] = -wb * ua; v[7] = wb * S.w;
    }
    __device__ __forceinline__ void add_beam(long long bp, const float v[8], float w) const
    {
        if (kFixed) {
            // an integer add of 0 changes nothing: zero values (the V
            // column of a sky without V, say) issue no atomic
            unsigned long long* p = gbeam_fx + 8 * bp;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const unsigned long long x = Scatter<kFixed>::fx(v[k] * w, sbeam);
                if (x) atomicAdd(p + k, x);
            }
        } else {
            float4* p = reinterpret_cast<float4*>(gbeam) + 2 * bp;
            atomicAdd(p, make_float4(v[0] * w, v[1] * w, v[2] * w, v[3] * w));
            atomicAdd(p + 1, make_float4(v[4] * w, v[5] * w, v[6] * w, v[7] * w));
        }
    }

    __device__ __forceinline__ void scatter(float wa, float wb, int pix, const float4& S,
                                           const F8& B, long long bp, float c2, float s2) const
    {
        if (want_sky) {
            const Scatter<kFixed> sc{wa,      wb,      gsky,  gsky_fx, nullptr,
                                     nullptr, nullptr, ssky,  sbeam,   want_v, plane};
            sc.scatter(wa, wb, pix, B, c2, s2);
        }
        float v[8];
        beam_grad(wa, wb, S, c2, s2, v);
        if (kFixed) {
            unsigned long long* p = gbeam_fx + 8 * bp;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const unsigned long long x = Scatter<kFixed>::fx(v[k], sbeam);
                if (x) atomicAdd(p + k, x);  // adding 0 changes nothing
            }
        } else {
            float4* p = reinterpret_cast<float4*>(gbeam) + 2 * bp;
            atomicAdd(p, make_float4(v[0], v[1], v[2], v[3]));
            atomicAdd(p + 1, make_float4(v[4], v[5], v[6], v[7]));
        }
    }

    // bilinear lookup: the pair's beam value is sum_i w_i beam[px_i] (w
    // renormalised over the stored map), so each stencil pixel gets w_i of
    // the pair's beam gradient; the sky gradient uses the interpolated value
    __device__ __forceinline__ void scatter_stencil(float wa, float wb, int pix, const float4& S,
                                                   const int px[4], const float w[4], float c2,
                                                   float s2) const
    {
        if (want_sky) {
            F8 B;
            B.a = make_float4(0.f, 0.f, 0.f, 0.f);
            B.b = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (w[i] == 0.0f) continue;
                const F8 v = tuned::load_beam_stencil(beam_base + px[i]);
                B.a.x = fmaf(v.a.x, w[i], B.a.x); B.a.y = fmaf(v.a.y, w[i], B.a.y);
                B.a.z = fmaf(v.a.z, w[i], B.a.z); B.a.w = fmaf(v.a.w, w[i], B.a.w);
                B.b.x = fmaf(v.b.x, w[i], B.b.x); B.b.y = fmaf(v.b.y, w[i], B.b.y);
                B.b.z = fmaf(v.b.z, w[i], B.b.z); B.b.w = fmaf(v.b.w, w[i], B.b.w);
            }
            const Scatter<kFixed> sc{wa,      wb,      gsky,  gsky_fx, nullptr,
                                     nullptr, nullptr, ssky,  sbeam,   want_v, plane};
            sc.scatter(wa, wb, pix, B, c2, s2);
        }
        float v[8];
        beam_grad(wa, wb, S, c2, s2, v);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (w[i] != 0.0f) add_beam(px[i], v, w[i]);
    }
};

// Sky gradient (optional) and the beam-parameter gradient of the elliptical
// Gaussian pair model, without a beam-map gradient.  The model beam is
// B[b] = c g[b] / N with c = (1 + eps, 1 - eps, 0, 0) for both detectors
// (beam_model.h), so a pair's share of dL/dB[b] . dB[b]/dt needs only
//   s = (1 + eps)(ga + gb) I + (1 - eps)(ga - gb)(Q cos 2chi + U sin 2chi),
// its TOD weights times c . dtod/dB: each lane adds s g[b] and s dg[b]/dt
// (t = F, e, phi0, dx, dy), read from the per-pixel table the adjoint entry
// point recomputes from the parameters, into six compensated FP32 sums.  The
// warp's sums are written to its own row of ppart (FP64, fixed shuffle
// tree); launch_fold_params adds the rows in warp order, so the result is
// the same on every run.  With the bilinear lookup the pair's beam value is
// sum_i w_i B[b_i], and each stencil pixel gets w_i of s.
template <bool kFixed>
struct ScatterParams {
    static constexpr bool kSums = false;
    static constexpr bool kStencil = true;
    float ga, gb;
    const F8* beam_base;
    const float4* sky;
    const F8* ptab;
    double* ppart;
    float ci, cq;  // 1 + eps, 1 - eps
    Scatter<kFixed> sc;
    int want_sky;
    float acc[6], cmp[6];

    __device__ __forceinline__ void stash(tuned::Pend& p) const
    {
        p.ga = ga;
        p.gb = gb;
    }
    __device__ __forceinline__ float4 fetch(int pix) const { return __ldg(&sky[pix]); }
    __device__ __forceinline__ void add(float wa, float wb, const float4& S, float c2, float s2,
                                        int b, float w)
    {
        const float qa = fmaf(S.y, c2, S.z * s2);
        const float sp = w * fmaf(ci * (wa + wb), S.x, cq * (wa - wb) * qa);
        const F8 t = tuned::load_beam(ptab + b);
        tuned::two_sum(acc[0], cmp[0], sp * t.a.x);
        tuned::two_sum(acc[1], cmp[1], sp * t.a.y);
        tuned::two_sum(acc[2], cmp[2], sp * t.a.z);
        tuned::two_sum(acc[3], cmp[3], sp * t.a.w);
        tuned::two_sum(acc[4], cmp[4], sp * t.b.x);
        tuned::two_sum(acc[5], cmp[5], sp * t.b.y);
    }
    __device__ __forceinline__ void pair(int pix, const float4& S, const F8& B, int bp, float c2,
                                         float s2)
    {
        if (want_sky) sc.scatter(ga, gb, pix, B, c2, s2);
        add(ga, gb, S, c2, s2, bp, 1.0f);
    }
    __device__ __forceinline__ void deferred(const tuned::Pend& p, int pix, const F8& B, int bp,
                                            float c2, float s2, float&, float&)
    {
        if (want_sky) sc.scatter(p.ga, p.gb, pix, B, c2, s2);
        add(p.ga, p.gb, fetch(pix), c2, s2, bp, 1.0f);
    }
    __device__ __forceinline__ void stencil(float wa, float wb, int pix, const float4& S,
                                            const int px[4], const float w[4], float c2, float s2)
    {
        if (want_sky) {
            F8 B;
            B.a = make_float4(0.f, 0.f, 0.f, 0.f);
            B.b = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (w[i] == 0.0f) continue;
                const F8 v = tuned::load_beam_stencil(beam_base + px[i]);
                B.a.x = fmaf(v.a.x, w[i], B.a.x); B.a.y = fmaf(v.a.y, w[i], B.a.y);
                B.a.z = fmaf(v.a.z, w[i], B.a.z); B.a.w = fmaf(v.a.w, w[i], B.a.w);
                B.b.x = fmaf(v.b.x, w[i], B.b.x); B.b.y = fmaf(v.b.y, w[i], B.b.y);
                B.b.z = fmaf(v.b.z, w[i], B.b.z); B.b.w = fmaf(v.b.w, w[i], B.b.w);
            }
            sc.scatter(wa, wb, pix, B, c2, s2);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (w[i] != 0.0f) add(wa, wb, S, c2, s2, px[i], w[i]);
    }
    __device__ __forceinline__ void pair_stencil(int pix, const float4& S, const int px[4],
                                                 const float w[4], float c2, float s2)
    {
        stencil(ga, gb, pix, S, px, w, c2, s2);
    }
    __device__ __forceinline__ void deferred_stencil(const tuned::Pend& p, int pix, const int px[4],
                                                     const float w[4], float c2, float s2)
    {
        stencil(p.ga, p.gb, pix, fetch(pix), px, w, c2, s2);
    }
    // the warp's six sums to row `warp` of ppart
    __device__ __forceinline__ void finish(int lane, long long warp) const
    {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            double v = (double)acc[k] + (double)cmp[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(tuned::kFull, v, o);
            if (lane == 0) ppart[6 * warp + k] = v;
        }
    }
};

template <class A, class = void>
struct HasFinish : std::false_type {};
template <class A>
struct HasFinish<A, std::void_t<decltype(&A::finish)>> : std::true_type {};

// Warps per SM of an instance: the planned nearest lookup runs 32 (register
// cap 64, its plan and descriptors in shared memory, as the forward does),
// the others 16 (cap 128).  The DETERMINISTIC beam-map gradient stays at 16:
// its action spills at 64 registers (c5: 95 ms against 87 ms).
template <class Act, bool kBil, bool kPlanned>
constexpr int adj_warps_per_sm()
{
    return kPlanned && !kBil && !std::is_same_v<Act, ScatterBeam<true>> ? 32 : 16;
}

// kBil: the transpose of the TUNED forward with the bilinear beam lookup.
// kPlanned: a.plans holds the samples' plans (index: position), built by
// adjoint_plan_kernel; otherwise each warp builds its own.
template <class Act, bool kBil, bool kPlanned>
__global__ void __launch_bounds__(kAW * 32, adj_warps_per_sm<Act, kBil, kPlanned>() / kAW)
    adjoint_kernel(AdjArgs a, Act proto)
{
    constexpr bool kDescSmem = adj_warps_per_sm<Act, kBil, kPlanned>() == 32;
    __shared__ tuned::WarpSmem sm[kAW];
    __shared__ Hpx s_hs, s_hb;
    __shared__ tuned::Beam s_B;
    const int lane = threadIdx.x & 31;
    tuned::WarpSmem& S = sm[threadIdx.x >> 5];
    const Hpx rhs = hpx_make(a.nside_sky);
    const Hpx rhb = hpx_make(a.nside_beam);
    const tuned::Beam rB = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    if constexpr (kDescSmem) {
        if (threadIdx.x == 0) {
            s_hs = rhs;
            s_hb = rhb;
            s_B = rB;
        }
        __syncthreads();
    }
    const Hpx& hs = kDescSmem ? s_hs : rhs;
    const Hpx& hb = kDescSmem ? s_hb : rhb;
    const tuned::Beam& B = kDescSmem ? s_B : rB;
    const long long gw = (long long)blockIdx.x * kAW + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kAW;
    unsigned long long nfall = 0, npairs = 0;
    float cmax = 0.0f;
    Act act = proto;
    tuned::Queue Q{0, 0};
    const tuned::Out none{nullptr, nullptr, 0, 0};
    for (long long i = gw; i < a.n; i += nw) {
        const long long j = a.order ? (long long)a.order[i] : i;  // sample of position i
        const long long s = a.begin + j;
        const double ga = a.g_f64 ? ((const double*)a.g_a)[j] : (double)((const float*)a.g_a)[j];
        const double gb = a.g_f64 ? ((const double*)a.g_b)[j] : (double)((const float*)a.g_b)[j];
        if (ga == 0.0 && gb == 0.0) continue;
        act.ga = (float)ga;
        act.gb = (float)gb;
        if constexpr (kPlanned)
            tuned::sample_planned<false, kBil>(a.plans[i], hs, a.rings, hb, B, a.ra[s], a.dec[s],
                                               a.pa[s], none, S, Q, lane, a.err, act, nfall, cmax,
                                               npairs);
        else
            tuned::sample<false, kBil>(hs, a.rings, hb, B, a.ra[s], a.dec[s], a.pa[s], none, S, Q,
                                       lane, a.err, act, nfall, cmax, npairs);
    }
    tuned::flush<kBil>(hs, S, Q, lane, a.err, act);
    if (lane == 0 && nfall && a.fallbacks) atomicAdd(a.fallbacks, nfall);
    if constexpr (HasFinish<Act>::value) act.finish(lane, gw);
}

template <class K>
int resident_blocks(K kernel, int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    return nb;
}

template <bool kPlanned, class Act>
cudaError_t launch_act(const AdjArgs& a, const Act& act, int sm_count, cudaStream_t st,
                       int* nwarps)
{
    const long long need = (a.n + kAW - 1) / kAW;
    long long blocks;
    if (a.interp == 1) {
        blocks = (long long)sm_count * resident_blocks(adjoint_kernel<Act, true, kPlanned>, kAW * 32);
        if (blocks > need) blocks = need;
        adjoint_kernel<Act, true, kPlanned><<<(int)blocks, kAW * 32, 0, st>>>(a, act);
    } else {
        blocks = (long long)sm_count * resident_blocks(adjoint_kernel<Act, false, kPlanned>, kAW * 32);
        if (blocks > need) blocks = need;
        adjoint_kernel<Act, false, kPlanned><<<(int)blocks, kAW * 32, 0, st>>>(a, act);
    }
    if (nwarps) *nwarps = (int)blocks * kAW;
    return cudaGetLastError();
}

// The action for the requested gradients, launched over a.n samples.
template <bool kPlanned>
cudaError_t launch_adjoint_impl(const AdjArgs& a, int sm_count, cudaStream_t st, int* nwarps)
{
    if (nwarps) *nwarps = 0;
    if (a.n <= 0) return cudaSuccess;
    const long long plane = 12LL * a.nside_sky * a.nside_sky;
    // fixed-point scales: powers of two of at most 2^126, exact in FP32
    const float fsky = (float)a.sky_scale, fbeam = (float)a.beam_scale;
    if (a.ptab) {
        if (a.fixed) {
            ScatterParams<true> act{};
            act.beam_base = a.beam32;
            act.sky = a.sky32;
            act.ptab = (const F8*)a.ptab;
            act.ppart = a.ppart;
            act.ci = a.ceps_i;
            act.cq = a.ceps_q;
            act.sc = Scatter<true>{0,       0,       nullptr,     a.gsky_fx,    nullptr,
                                   nullptr, a.sky32, fsky, fbeam, a.want_v, plane};
            act.want_sky = a.gsky_fx != nullptr;
            return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
        }
        ScatterParams<false> act{};
        act.beam_base = a.beam32;
        act.sky = a.sky32;
        act.ptab = (const F8*)a.ptab;
        act.ppart = a.ppart;
        act.ci = a.ceps_i;
        act.cq = a.ceps_q;
        act.sc = Scatter<false>{0,       0,   a.gsky32, nullptr, nullptr, nullptr, a.sky32, 0.0f, 0.0f,
                                a.want_v, plane};
        act.want_sky = a.gsky32 != nullptr;
        return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
    }
    const bool beam = a.gbeam32 || a.gbeam_fx;
    if (a.fixed) {
        if (beam) {
            ScatterBeam<true> act{0,          0,         a.beam32,     a.sky32,
                                  nullptr,    a.gsky_fx, nullptr,      a.gbeam_fx,
                                  fsky, fbeam, a.gsky_fx != nullptr, a.want_v,
                                  plane};
            return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
        }
        Scatter<true> act{0,       0,       nullptr,     a.gsky_fx,    nullptr,
                          nullptr, a.sky32, fsky, fbeam, a.want_v, plane};
        return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
    }
    if (beam) {
        ScatterBeam<false> act{0,         0,       a.beam32, a.sky32, a.gsky32,
                               nullptr,   a.gbeam32, nullptr, 0.0f,  0.0f,
                               a.gsky32 != nullptr, a.want_v};
        return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
    }
    Scatter<false> act{0, 0, a.gsky32, nullptr, nullptr, nullptr, a.sky32, 0.0f, 0.0f, a.want_v};
    return launch_act<kPlanned>(a, act, sm_count, st, nwarps);
}

}  // namespace
}  // namespace pisco
