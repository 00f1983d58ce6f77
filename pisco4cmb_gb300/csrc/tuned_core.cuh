// tuned_core.cuh -- per-sample body of the TUNED geometry, shared by the
// single-detector forward (fwd_tuned.cu), the batched multi-detector forward
// (fwd_batched.cu) and the adjoint (adjoint_kernels.cuh).
//
// A sample's FP64 set-up -- its disc plan, boresight frame and psi phasors
// (SamplePlan, make_plan) -- is built beforehand by a plan kernel with one
// thread per sample, or by the warp itself; the warp keeps it in its shared
// memory (WarpSmem::plan), so the pair loop's registers hold only the pair
// geometry (the kernels run 32 warps per SM at 64 registers).
//
// For one sample, a warp evaluates the HEALPix query_disc rings, one ring per
// lane, rounds per-ring small-offset constants to FP32 once, and strides the
// disc pairs across lanes.  Per pair, FP32 only: longitude offset from a
// per-ring anchor pixel, cancellation-free boresight-frame components, the
// beam grid's polar-cap indices and exp(2i chi) as a product of unit
// phasors.  Any of the three floor decisions lying within the margin of an
// integer, and any pair within 2e-6 rad of the boresight, is queued and redone
// with the FP64 chain of the PLAIN form (hpx.cuh pair_beam_pixel), so every
// pair lands on the same beam pixel as in PLAIN.
//
// The queue outlives the sample: each entry names a per-warp slot holding its
// sample's FP64 frame and output, and the warp redoes 32 entries at a time,
// whichever samples they came from (a sample queues about four pairs in a
// thousand, so a per-sample drain would run the long FP64 chain with a few
// lanes active).  The re-evaluated contributions of a sample are added in
// queue order, one lane per sample, into an FP64 sum, and its TOD is written
// (main-pass total + that sum) when its last entry is done: the result does
// not depend on where the drains cut the queue, hence not on the other
// samples of the warp.
//
// Disc edge: per ring, x and ysq of the HEALPix edge formula are formed in
// FP64 with exactly HEALPix's rounding, the edge angle atan2(sqrt(ysq), x) is
// taken in FP32, and the two floor decisions use FP64 positions; an edge
// within the FP32 angle's error bound of a pixel boundary is recomputed with
// the FP64 formula (disc_ring), so the disc is HEALPix query_disc's exactly.
//
// Geometry, with the pixel at ring height z (s = sqrt(1 - z^2)), longitude
// offset D from the boresight (z0, s0) and h = 1 - cos D:
//   east  u = s sin D                   north v = sin(dec - dec0) + s z0 h
//   1 - cos(rho) = (1 - cos(dec - dec0)) + s s0 h
//   toward the boresight at the pixel: (s0 sin D, sin(dec0 - dec) + s0 z h)
//   r = sqrt(3) nside_b sqrt(1 - cos rho),  sigma = pi - alpha - psi,
//   alpha = atan2(u, v),  exp(2i chi) = exp(2i beta) exp(2i alpha) exp(2i psi)
// (sphtrigo.cpp:27-54 rewritten in small-offset form).
//
// The per-pair work is handed to an Action (Gather below, Scatter in
// adjoint.cu):
//   kSums                     true: per-sample sums, TOD written per sample
//   void reset(), total(a, b) main-pass sums (kSums)
//   P fetch(int pix)          per-pixel data the action needs (Gather: the sky)
//   void pair(int pix, P fetched, const F8& beam, int bp, float c2, float s2)
//   void stash(Pend&)         per-sample data a queued pair needs later
//   void deferred(const Pend&, int pix, const F8& beam, int bp, float c2, float s2,
//                 float& ta, float& tb)      a re-evaluated pair
//   kStencil                  true: with the bilinear lookup the action gets
//                             the stencil instead of the interpolated value:
//   void pair_stencil(int pix, P fetched, const int px[4], const float w[4], c2, s2)
//   void deferred_stencil(const Pend&, int pix, const int px[4], const float w[4], c2, s2)
// (c2, s2 = cos 2chi, sin 2chi; `beam` is the beam pixel's value, bp its
// index, with the nearest lookup, and the interpolated value, bp = -1, with
// the bilinear one).
// Optional, detected at compile time (the forward and adjoint actions leave
// them out, so they cost nothing there):
//   void outside(int pix, int bp)                a disc pair whose beam pixel
//   void outside_deferred(const Pend&, int pix, int bp)   lies beyond the
//                             stored map (bp; -1: no bilinear stencil pixel in it)
#pragma once

#include <math_constants.h>

#include <type_traits>

#include "hpx.cuh"
#include "internal.h"

// Warps per block of the adjoint's and the diagnostics' kernels, and the
// minimum number of resident blocks per SM requested from the compiler (which
// caps their registers at 65536 / (32 x warps x blocks)); the adjoint's
// planned nearest-lookup instances take 4 blocks (adjoint_kernels.cuh).
#ifndef PISCO_TUNED_WARPS
#define PISCO_TUNED_WARPS 8
#endif
#ifndef PISCO_TUNED_MINB
#define PISCO_TUNED_MINB 2
#endif

namespace pisco {
namespace tuned {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kQCap = 64;

// Does the action want to hear of disc pairs outside the stored beam map?
template <class A, class = void>
struct HasOutside : std::false_type {};
template <class A>
struct HasOutside<A, std::void_t<decltype(&A::outside)>> : std::true_type {};
// Decisions whose FP32 value lies within kMarginRel * (value + 1) of an
// integer are redone in FP64 (about 20 FP32 ulps).  The observed worst case
// over a workload is measured by pisco_tuned_calibrate and must stay well
// below this bound.
constexpr float kMarginRel = 1.2e-6f;
// Pairs with 1 - cos(rho) below this take the reference's degenerate branch
// (rho <= 1e-6, sphtrigo.cpp:40-48) and are done in FP64.
constexpr float kTinyQ = 4.0e-12f;

// One disc ring of the current batch: FP32 offset constants and the pixel
// range(s), 64 bytes, read with four 16-byte loads.
struct alignas(16) RingC {
    float dc, dphi, si, Di;  // anchor offset, pixel spacing, s, sin(dec - dec0)
    float Ki, Zs, Wz, Pp;    // 1 - cos(dec - dec0), s z0, s0 z, s s0
    int s1, s2, b1, b2;      // range starts, anchor offsets of the ranges (second: minus n1)
    int n1, nr, incl, base;  // first range length, ring pixels, inclusive scan, first index
};

// Samples in flight per warp (a sample keeps its slot until its queued
// pairs are done).
constexpr int kPend = 16;

// A sample whose queued pairs may not all be re-evaluated yet.
struct alignas(16) Pend {
    Hpx hb;                  // beam grid
    double ra, dec, psi;     // FP64 frame (psi = -pa)
    double main_a, main_b;   // main-pass totals
    double fb_a, fb_b;       // re-evaluated pairs, summed in queue order
    const F8* beam;
    void* out_a;
    void* out_b;
    long long idx;           // output index
    float ga, gb;            // adjoint weights
    int npix_beam;
    int left;                // queued entries not yet re-evaluated
    int open;                // main pass still running
    int f64;                 // output type
};

// A sample's per-sample geometry: its disc (the rings it touches and the
// edge formula's constants), the boresight frame and the psi phasors.  Built
// by make_plan, either inside the pair kernel (one warp per sample, every
// lane redundantly) or beforehand by plan_kernel with one thread per sample:
// it is FP64 work (about three hundred FP64 instructions), which GB300 runs
// at a small fraction of its FP32 rate.  96 bytes.
struct alignas(16) SamplePlan {
    double z0, xa, phi;       // disc: cos(theta), 1 / sin(theta), longitude (disc_plan)
    double phi_f, dec0;       // frame: longitude reduced mod 2 pi, latitude
    double cosr;              // disc: cos(radius) (the beam's, as evaluated on the device)
    float z0f, s0f;           // frame: sin and |cos| of the latitude
    float sps, cps, c2p, s2p; // psi phasors (negated with the frame's flip)
    int ring_lo, ring_hi;     // rings on the edge formula
    int full_lo, full_hi;     // rings touched
    int flags;                // kPlanBad: non-finite pointing; kPlanAllSky
};
constexpr int kPlanBad = 1;
constexpr int kPlanAllSky = 2;

// Per-warp shared state: one ring batch, the samples in flight, the FP64
// re-evaluation queue (sky pixel, slot) and the current sample's plan (read
// from here where needed rather than held in registers across the pair loop).
struct WarpSmem {
    SamplePlan plan;
    RingC r[32];
    Pend p[kPend];
    int q[kQCap];
    unsigned char qs[kQCap];
    float ta[32], tb[32];
};

// Warp-uniform queue state, in registers.
struct Queue {
    int n;    // queued entries (< 32 between samples)
    int cur;  // next slot
};

// Where one sample's TOD goes.
struct Out {
    void* a;
    void* b;
    long long idx;
    int f64;
};

__device__ __forceinline__ void store_out(void* out, int f64, long long i, double v)
{
    if (!out) return;
    if (f64) ((double*)out)[i] = v;
    else ((float*)out)[i] = (float)v;
}

__device__ __forceinline__ void finalize(const Pend& P)
{
    store_out(P.out_a, P.f64, P.idx, P.main_a + P.fb_a);
    store_out(P.out_b, P.f64, P.idx, P.main_b + P.fb_b);
}

struct Beam {
    const F8* beam;
    int nside;
    int npix;
    double rho_max;
    double cosr;   // cos(rho_max), evaluated on the device
    float rscale;  // sqrt(3) * nside
};

__device__ __forceinline__ Beam make_beam(const F8* beam, int nside, int npix, double rho_max)
{
    Beam b;
    b.beam = beam;
    b.nside = nside;
    b.npix = npix;
    b.rho_max = rho_max;
    b.cosr = rho_max >= kPi ? 0.0 : cos(rho_max);
    b.rscale = (float)(1.7320508075688772 * (double)nside);
    return b;
}

struct Frame {
    double ra, dec, psi;
    float s0, sps, cps, c2p, s2p;
};

__device__ __forceinline__ void record(unsigned int* err, unsigned int code)
{
    if (err) atomicCAS(err, 0u, code);
}

__device__ __forceinline__ void two_sum(float& s, float& c, float x)
{
    const float t = s + x;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (x - bp);
    s = t;
    c += e;
}

// x within m of an integer (x - rint(x) is exact for |x| < 2^23).
__device__ __forceinline__ bool near_int(float x, float m)
{
    return fabsf(x - rintf(x)) < m;
}

#ifndef PISCO_FAST_FLOOR
#define PISCO_FAST_FLOOR 1
#endif
constexpr float kTwo23 = 8388608.0f;
constexpr int kTwo23Bits = 0x4B000000;  // the bits of 2^23

// floor(x) and its fractional part f = x - floor(x) for 0 <= x < 2^23 by
// FP32 additions: x + 2^23 rounded down is 2^23 + floor(x) exactly (the
// spacing of floats in [2^23, 2^24) is 1), and x - floor(x) is exact
// (Sterbenz).  f < m or 1 - f < m is |x - rint(x)| < m (1 - f is exact for
// f >= 1/2, and above 1/2 > m otherwise), so the decisions are near_int's.
__device__ __forceinline__ int split_floor(float x, float& f)
{
    const float t = __fadd_rd(x, kTwo23);
    f = x - (t - kTwo23);
    return __float_as_int(t) - kTwo23Bits;
}

// (float)k for |k| < 2^22 by FP32 addition: 1.5 * 2^23 + k lies in
// [2^23, 2^24), where floats are the integers and their bits are linear in
// the value, so no conversion instruction is needed (the same value).
__device__ __forceinline__ float small_int_to_float(int k)
{
    return __int_as_float(0x4B400000 + k) - 12582912.0f;
}

// The inverse for an integer-valued float f, |f| < 2^22 (exact, no conversion).
__device__ __forceinline__ int small_float_to_int(float f)
{
    return __float_as_int(f + 12582912.0f) - 0x4B400000;
}

// 1/x by the MUFU reciprocal approximation (relative error below 2^-22);
// used only for values, never for an index decision.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One beam pixel, both detectors (32 bytes, one sector): a single 256-bit
// load through the read-only path that does not allocate in L1, so the
// scattered beam reads (a beam of 10^4 - 10^6 pixels, L2-resident) leave L1
// to the sky pixels, which neighbouring samples re-read (measured on the
// c2 forward: 176.2 ms against 177.2 ms allocating in L1).  PISCO_BEAM_LOAD
// 0: the compiler's own loads (two 128-bit ones); 1: 256-bit, allocating in
// L1; 3: 256-bit, L2 only (.cg).
#ifndef PISCO_BEAM_LOAD
#define PISCO_BEAM_LOAD 2
#endif
__device__ __forceinline__ F8 load_beam(const F8* p)
{
#if PISCO_BEAM_LOAD == 0
    return *p;
#else
    F8 r;
#if PISCO_BEAM_LOAD == 2
#define PISCO_LDB "ld.global.nc.L1::no_allocate.v8.f32"
#elif PISCO_BEAM_LOAD == 3
#define PISCO_LDB "ld.global.cg.v8.f32"
#else
#define PISCO_LDB "ld.global.nc.v8.f32"
#endif
    asm(PISCO_LDB " {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y),
          "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
#undef PISCO_LDB
    return r;
#endif
}

// A beam pixel of the bilinear stencil: its four pixels are two pairs of
// ring neighbours, and neighbouring pairs of a sample share stencil pixels,
// so these reads do hit L1; the compiler's own (allocating, 2 x 128-bit)
// loads serve them best (c2 bilinear forward: 331.9 ms, against 348.4 ms
// for one allocating 256-bit load and 368.1 ms without L1 allocation).
// PISCO_BIL_L1 0: no allocation, as the nearest lookup; 1: one allocating
// 256-bit load; 2: the compiler's loads.
#ifndef PISCO_BIL_L1
#define PISCO_BIL_L1 2
#endif
__device__ __forceinline__ F8 load_beam_stencil(const F8* p)
{
#if PISCO_BIL_L1 == 2
    return *p;
#elif PISCO_BIL_L1
    F8 r;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y),
          "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
    return r;
#else
    return load_beam(p);
#endif
}

// The disc's pixel range(s) on one ring: FP32 edge angle, FP64 positions,
// exact FP64 HEALPix formula (disc_ring) whenever an edge decision is within
// the FP32 angle's error of a pixel boundary.  Same result as disc_ring.
__device__ __forceinline__ RingSpan fast_disc_ring(const Hpx& h, const SamplePlan& p, double cosr,
                                                   long long ring, const RingT& rt)
{
    RingSpan s = {0, 0, 0, 0};
    if (ring < p.full_lo || ring > p.full_hi) return s;
    const long long npix = rt.npix2 >> 1;
    if ((p.flags & kPlanAllSky) || ring < p.ring_lo || ring > p.ring_hi) {
        s.start1 = rt.start;
        s.n1 = npix;
        return s;
    }
    const double x = PD_MUL(PD_SUB(cosr, PD_MUL(rt.z, p.z0)), p.xa);
    const double ysq = PD_SUB(rt.omz2, PD_MUL(x, x));
    if (!(ysq > 0.0)) return s;  // no intersection (HEALPix: dphi = 0, ring skipped)
    const float de = atan2f(sqrtf((float)ysq), (float)x);
    const double shift = (rt.npix2 & 1) ? 0.5 : 0.0;
    const double fr = rt.fr;
    const double vlo = fr * (p.phi - (double)de) - shift;
    const double vhi = fr * (p.phi + (double)de) - shift;
    // |de - atan2(sqrt(ysq), x)| <= 3e-7 de (FP32 rounding of x, ysq and atan2f)
    const double m = fr * (4e-7 * (double)de) + 1e-9;
    const double flo = vlo - floor(vlo), fhi = vhi - floor(vhi);
    if (!(de > 0.0f) || flo < m || flo > 1.0 - m || fhi < m || fhi > 1.0 - m) {
        DiscPlan d;
        d.z0 = p.z0;
        d.xa = p.xa;
        d.cosr = cosr;
        d.phi = p.phi;
        d.ring_lo = p.ring_lo;
        d.ring_hi = p.ring_hi;
        d.full_lo = p.full_lo;
        d.full_hi = p.full_hi;
        d.all_sky = (p.flags & kPlanAllSky) != 0;
        return disc_ring(h, d, ring);
    }
    long long lo = (long long)floor(vlo) + 1;
    long long hi = (long long)floor(vhi);
    if (lo > hi) return s;
    if (hi >= npix) {
        lo -= npix;
        hi -= npix;
    }
    if (lo < 0) {
        s.start1 = rt.start;
        s.n1 = hi + 1;
        s.start2 = rt.start + lo + npix;
        s.n2 = -lo;
    } else {
        s.start1 = rt.start + lo;
        s.n1 = hi - lo + 1;
    }
    return s;
}

// Bilinear beam value of the PLAIN form (HEALPix get_interpol in FP64; the
// weights of stencil pixels outside the stored map are dropped and the rest
// renormalised; the value rounded to float).  false: no stencil pixel lies in
// the map.  Not inlined: only the degenerate boresight pairs take it, and
// inlined its FP64 stencil would spill registers of the main pair loop.
static __device__ __noinline__ bool bilinear_f64(const Hpx& hb, int npb, double rho,
                                                 double sig, const F8* beam, F8& out)
{
    int64_t px[4];
    double w[4];
    get_interpol(hb, rho, sig, px, w);
    double ws = 0.0, va[4] = {0.0, 0.0, 0.0, 0.0}, vb[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (px[i] < 0 || px[i] >= npb) continue;
        ws += w[i];
        const F8 B = beam[px[i]];
        va[0] += B.a.x * w[i]; va[1] += B.a.y * w[i]; va[2] += B.a.z * w[i]; va[3] += B.a.w * w[i];
        vb[0] += B.b.x * w[i]; vb[1] += B.b.y * w[i]; vb[2] += B.b.z * w[i]; vb[3] += B.b.w * w[i];
    }
    if (!(ws > 0.0)) return false;
    out.a = make_float4((float)(va[0] / ws), (float)(va[1] / ws), (float)(va[2] / ws),
                        (float)(va[3] / ws));
    out.b = make_float4((float)(vb[0] / ws), (float)(vb[1] / ws), (float)(vb[2] / ws),
                        (float)(vb[3] / ws));
    return true;
}

// get_interpol's stencil in FP64 with the weights renormalised over the
// pixels inside the stored map (pixels outside get weight 0), rounded to
// float: what a beam-gradient scatter needs.  false: no pixel in the map.
static __device__ __noinline__ bool stencil_f64(const Hpx& hb, int npb, double rho, double sig,
                                                int px[4], float w[4])
{
    int64_t p[4];
    double wd[4];
    get_interpol(hb, rho, sig, p, wd);
    double ws = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (p[i] >= 0 && p[i] < npb) ws += wd[i];
    if (!(ws > 0.0)) return false;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool in = p[i] >= 0 && p[i] < npb;
        px[i] = in ? (int)p[i] : 0;
        w[i] = in ? (float)(wd[i] / ws) : 0.0f;
    }
    return true;
}

// (f(a) - f(b)) / (2c (a - b)) for f(x) = 2 asin(c x), the colatitude of ring
// height x (x = nside sqrt(3 (1 - cos theta)), c = 1 / (sqrt(6) nside)), by
// the asin series to c^4 (relative truncation below 1e-8 for theta <= 0.5).
__device__ __forceinline__ float asin_slope(float a, float b, float c2)
{
    const float s2 = fmaf(a, a, fmaf(a, b, b * b));
    const float a2 = a * a, b2 = b * b;
    const float s4 = fmaf(a2, a2, fmaf(a2, a * b, fmaf(a2, b2, fmaf(a * b, b2, b2 * b2))));
    return fmaf(c2 * c2 * 0.075f, s4, fmaf(c2 * (1.0f / 6.0f), s2, 1.0f));
}

#ifndef PISCO_BIL_FASTDIV
#define PISCO_BIL_FASTDIV 1
#endif
// a / b for the stencil weights (b > 0, never an index decision): the MUFU
// reciprocal instead of the IEEE division (c2 bilinear forward: 313.3 ms
// against 332.0 ms; the weights move by about an ulp)
__device__ __forceinline__ float wdiv(float a, float b)
{
#if PISCO_BIL_FASTDIV
    return a * rcp_approx(b);
#else
    return a / b;
#endif
}

// The same stencil in FP32 from the pair's polar-cap coordinates on the beam
// grid: r = nside sqrt(3 (1 - cos rho)) and sigma = (qd + tp) pi/2.  Rings of
// the north cap: ring i holds 4i pixels from 2i(i - 1), half a pixel shifted;
// get_interpol takes the ring above (floor r) and the next one, interpolates
// in longitude on each and linearly in colatitude between them (ring 1 and
// its image across the pole when r < 1).  The weights are continuous across
// every floor decision, so FP32 index choices near a boundary change the
// value only by the FP32 error of r and tp: no FP64 re-evaluation is needed.
__device__ __forceinline__ bool bilinear_f32(const Beam& B, int qd, float tp, float r, F8& out)
{
    const float c = 1.0f / (2.4494897427831781f * (float)B.nside);  // 1 / (sqrt(6) nside)
    const float c2 = c * c;
    float kfr;
    const int k = split_floor(r, kfr);  // ring above (0 above the first ring); r >= 0
    // longitude interpolation on ring i: pixels start + i1, start + i1 + 1
    auto ring = [&](int i, int& p1, int& p2, float& w1, float& w2) {
        const float t = fmaf(tp, small_int_to_float(i), -0.5f);
        const float fl = floorf(t);
        const float f = t - fl;
        int i1 = small_float_to_int(fl) + qd * i, i2 = i1 + 1;
        const int np = 4 * i;
        if (i1 < 0) i1 += np;
        if (i2 >= np) i2 -= np;
        const int start = 2 * i * (i - 1);
        p1 = start + i1;
        p2 = start + i2;
        w1 = 1.0f - f;
        w2 = f;
    };
    // stencil pixels are added as soon as their weight is known, in
    // get_interpol's order; pixels beyond the stored map are dropped
    float ws = 0.0f;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = make_float4(0.f, 0.f, 0.f, 0.f);
    auto add = [&](int p, float w) {
        if (p >= B.npix) return;
        ws += w;
        const F8 v = load_beam_stencil(B.beam + p);
        a.x = fmaf(v.a.x, w, a.x); a.y = fmaf(v.a.y, w, a.y);
        a.z = fmaf(v.a.z, w, a.z); a.w = fmaf(v.a.w, w, a.w);
        b.x = fmaf(v.b.x, w, b.x); b.y = fmaf(v.b.y, w, b.y);
        b.z = fmaf(v.b.z, w, b.z); b.w = fmaf(v.b.w, w, b.w);
    };
    int p1, p2;
    float w1, w2;
    if (k == 0) {
        ring(1, p1, p2, w1, w2);
        const float wt = wdiv(r * asin_slope(r, 0.0f, c2), asin_slope(1.0f, 0.0f, c2));
        const float f = 0.25f * (1.0f - wt);
        add((p1 + 2) & 3, f);
        add((p2 + 2) & 3, f);
        add(p1, fmaf(w1, wt, f));
        add(p2, fmaf(w2, wt, f));
    } else {
        const float kf = small_int_to_float(k);
        const float wt = wdiv((r - kf) * asin_slope(r, kf, c2), asin_slope(kf + 1.0f, kf, c2));
        ring(k, p1, p2, w1, w2);
        add(p1, w1 * (1.0f - wt));
        add(p2, w2 * (1.0f - wt));
        ring(k + 1, p1, p2, w1, w2);
        add(p1, w1 * wt);
        add(p2, w2 * wt);
    }
    if (!(ws > 0.0f)) return false;
    const float iw = wdiv(1.0f, ws);
    out.a = make_float4(a.x * iw, a.y * iw, a.z * iw, a.w * iw);
    out.b = make_float4(b.x * iw, b.y * iw, b.z * iw, b.w * iw);
    return true;
}

// The stencil of bilinear_f32 itself: pixels and weights renormalised over
// the pixels inside the stored map (outside: weight 0), for actions that
// scatter into the beam (Action::kStencil).
__device__ __forceinline__ bool stencil_f32(const Beam& B, int qd, float tp, float r, int px[4],
                                            float w[4])
{
    const float c = 1.0f / (2.4494897427831781f * (float)B.nside);
    const float c2 = c * c;
    float kfr;
    const int k = split_floor(r, kfr);  // r >= 0
    auto ring = [&](int i, int& p1, int& p2, float& w1, float& w2) {
        const float t = fmaf(tp, small_int_to_float(i), -0.5f);
        const float fl = floorf(t);
        const float f = t - fl;
        int i1 = small_float_to_int(fl) + qd * i, i2 = i1 + 1;
        const int np = 4 * i;
        if (i1 < 0) i1 += np;
        if (i2 >= np) i2 -= np;
        const int start = 2 * i * (i - 1);
        p1 = start + i1;
        p2 = start + i2;
        w1 = 1.0f - f;
        w2 = f;
    };
    if (k == 0) {
        ring(1, px[2], px[3], w[2], w[3]);
        const float wt = wdiv(r * asin_slope(r, 0.0f, c2), asin_slope(1.0f, 0.0f, c2));
        const float f = 0.25f * (1.0f - wt);
        w[0] = f;
        w[1] = f;
        w[2] = fmaf(w[2], wt, f);
        w[3] = fmaf(w[3], wt, f);
        px[0] = (px[2] + 2) & 3;
        px[1] = (px[3] + 2) & 3;
    } else {
        ring(k, px[0], px[1], w[0], w[1]);
        ring(k + 1, px[2], px[3], w[2], w[3]);
        const float kf = small_int_to_float(k);
        const float wt = wdiv((r - kf) * asin_slope(r, kf, c2), asin_slope(kf + 1.0f, kf, c2));
        w[0] *= 1.0f - wt;
        w[1] *= 1.0f - wt;
        w[2] *= wt;
        w[3] *= wt;
    }
    float ws = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (px[i] >= B.npix) {
            px[i] = 0;
            w[i] = 0.0f;
        }
        ws += w[i];
    }
    if (!(ws > 0.0f)) return false;
    const float iw = wdiv(1.0f, ws);
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] *= iw;
    return true;
}

// Redoes the first m (<= 32, <= Q.n) queued pairs with the FP64 chain of the
// PLAIN form, one per lane; credits each to its sample (serially, in queue
// order, by the first lane of each run of one slot's entries), writes the TOD
// of every sample left with nothing queued, and drops the m entries.  kBil:
// the beam value is PLAIN's bilinear one instead of the nearest pixel's.
template <bool kBil = false, class Action>
__device__ __forceinline__ void drain(const Hpx& hs, int m, WarpSmem& S, Queue& Q, int lane,
                                      unsigned int* err, Action& act)
{
    float ta = 0.0f, tb = 0.0f;
    int slot = -1;
    if (lane < m) {
        slot = S.qs[lane];
        const Pend& P = S.p[slot];
        const int pix = S.q[lane];
        double rho, sig, chi;
        const long long bp = pair_beam_pixel(hs, P.hb, pix, P.ra, P.dec, P.psi, &rho, &sig, &chi);
        if constexpr (kBil && Action::kStencil) {
            int px[4];
            float w[4];
            if (stencil_f64(P.hb, P.npix_beam, rho, sig, px, w))
                act.deferred_stencil(P, pix, px, w, (float)cos(2.0 * chi), (float)sin(2.0 * chi));
            else if constexpr (HasOutside<Action>::value)
                act.outside_deferred(P, pix, -1);
        } else if constexpr (kBil) {
            F8 Bv;
            if (bilinear_f64(P.hb, P.npix_beam, rho, sig, P.beam, Bv))
                act.deferred(P, pix, Bv, -1, (float)cos(2.0 * chi), (float)sin(2.0 * chi), ta, tb);
            else if constexpr (HasOutside<Action>::value)
                act.outside_deferred(P, pix, -1);
        } else if (bp < 0) {
            record(err, kCheckBeamIndex);
        } else if (bp < P.npix_beam) {
            act.deferred(P, pix, load_beam(P.beam + bp), (int)bp, (float)cos(2.0 * chi),
                         (float)sin(2.0 * chi), ta, tb);
        } else if constexpr (HasOutside<Action>::value) {
            act.outside_deferred(P, pix, (int)bp);
        }
    }
    if (Action::kSums) {
        S.ta[lane] = ta;
        S.tb[lane] = tb;
    }
    __syncwarp();
    if (lane < m && (lane == 0 || S.qs[lane - 1] != slot)) {
        Pend& P = S.p[slot];
        int k = lane;
        if (Action::kSums) {
            double a = P.fb_a, b = P.fb_b;
            do {
                a += (double)S.ta[k];
                b += (double)S.tb[k];
                ++k;
            } while (k < m && S.qs[k] == slot);
            P.fb_a = a;
            P.fb_b = b;
        } else {
            do ++k;
            while (k < m && S.qs[k] == slot);
        }
        P.left -= k - lane;
        if (Action::kSums && P.left == 0 && !P.open) finalize(P);
    }
    // move the rest (<= 32 entries: the queue holds < 64) to the front
    const int rest = Q.n - m;
    int vq = 0, vs = 0;
    if (lane < rest) {
        vq = S.q[m + lane];
        vs = S.qs[m + lane];
    }
    __syncwarp();
    if (lane < rest) {
        S.q[lane] = vq;
        S.qs[lane] = (unsigned char)vs;
    }
    __syncwarp();
    Q.n = rest;
}

// Redoes every queued pair (at a sample boundary, where fewer than 32 are
// queued): all slots are free afterwards.  Called once more before a warp
// leaves the kernel.
template <bool kBil = false, class Action>
__device__ __forceinline__ void flush(const Hpx& hs, WarpSmem& S, Queue& Q, int lane,
                                      unsigned int* err, Action& act)
{
    if (Q.n > 0) drain<kBil>(hs, Q.n, S, Q, lane, err, act);
}

// sin(x) and 1 - cos(x): Taylor series for |x| <= 0.5 (truncation below
// 3e-11 relative), CUDA sincosf beyond.
__device__ __forceinline__ void sin_versin(float x, float& sn, float& h)
{
    if (fabsf(x) <= 0.5f) {
        const float x2 = x * x;
        sn = x * fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 2.75573192e-6f, -1.98412698e-4f),
                                        8.33333333e-3f), -1.66666667e-1f), 1.0f);
        h = x2 * fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 2.75573192e-7f, -2.48015873e-5f),
                                        1.38888889e-3f), -4.16666667e-2f), 0.5f);
    } else {
        float cs;
        sincosf(x, &sn, &cs);
        h = (cs > 0.0f) ? (sn * sn) / (1.0f + cs) : 1.0f - cs;
    }
}

// atan2(y, x) / (pi/2) for y, x >= 0, in [0, 1]: the arctangent of the
// ratio min/max by the minimax polynomial of Abramowitz & Stegun 4.4.49
// (|error| <= 2e-8 on [0, 1]; 1e-7 when evaluated in FP32), reflected for
// y > x.  y = x = 0 gives 0 (such pairs are re-done in FP64 anyway).
__device__ __forceinline__ float quarter_turns(float y, float x)
{
    const bool swap = y > x;
    const float mn = swap ? x : y, mx = swap ? y : x;
    const float t = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
    const float t2 = t * t;
    float p = 0.0028662257f;
    p = fmaf(p, t2, -0.0161657367f);
    p = fmaf(p, t2, 0.0429096138f);
    p = fmaf(p, t2, -0.0752896400f);
    p = fmaf(p, t2, 0.1065626393f);
    p = fmaf(p, t2, -0.1420889944f);
    p = fmaf(p, t2, 0.1999355085f);
    p = fmaf(p, t2, -0.3333314528f);
    p = fmaf(p, t2, 1.0f);
    const float a = t * p * 0.63661977236758134f;  // atan(t) / (pi/2)
    return swap ? 1.0f - a : a;
}

__device__ __forceinline__ SamplePlan make_plan(const Hpx& hs, const Beam& B, double ra,
                                                double dec, double pa)
{
    SamplePlan sp;
    const double psi = -pa;
    if (!(isfinite(ra) && isfinite(dec) && isfinite(psi))) {
        sp.flags = kPlanBad;
        sp.full_lo = 1;
        sp.full_hi = 0;
        return sp;
    }
    const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, dec), ra, B.rho_max, B.cosr);
    // Boresight frame.  The reference chain (sphtrigo.cpp:29-35) takes dec as
    // given; for cos(dec) < 0 the same point is (pi - dec, ra + pi), and the
    // chain's north direction then points the other way: its alpha is the
    // normalised frame's + pi, hence its sigma is - pi, while beta and
    // exp(2i chi) are unchanged.  So the geometry runs in the normalised frame
    // (s0 >= 0) with (sin psi, cos psi) negated, which adds exactly pi to
    // sigma.  ra is reduced mod 2pi (the anchor longitude of the rings).
    // The frame is disc_plan's (z0 = cos(theta), s0, phi, latitude
    // pi/2 - theta) whenever its reflection agrees with the sign of cos(dec),
    // which decides the flip as in the reference chain; they can differ
    // only within an ulp of the poles, where the frame is rebuilt from dec.
    const bool flip = fabs(dec) < 1.5707963 ? false : cos(dec) < 0.0;
    double z0d, s0d;
    if (flip == P.flip) {
        z0d = P.z0;
        s0d = P.s0;
        sp.phi_f = P.phi;
        sp.dec0 = PD_SUB(kHalfPi, P.theta);
    } else {
        double sdec, cdec;
        sincos(dec, &sdec, &cdec);
        z0d = sdec;
        s0d = fabs(cdec);
        sp.phi_f = fmodulo(flip ? ra + kPi : ra, kTwoPi);
        sp.dec0 = atan2(z0d, s0d);
    }
    sp.z0f = (float)z0d;
    sp.s0f = (float)s0d;
    // psi phasors in FP64, rounded once: exp(2i psi) multiplies every pair
    // of the sample, so its rounding error is coherent over the sample sum.
    double spsi, cpsi;
    sincos(psi, &spsi, &cpsi);
    sp.sps = (float)(flip ? -spsi : spsi);
    sp.cps = (float)(flip ? -cpsi : cpsi);
    sp.c2p = (float)__fma_rn(cpsi, cpsi, -__dmul_rn(spsi, spsi));
    sp.s2p = (float)__dmul_rn(__dmul_rn(2.0, spsi), cpsi);
    sp.z0 = P.z0;
    sp.xa = P.xa;
    sp.phi = P.phi;
    sp.cosr = B.cosr;
    sp.ring_lo = (int)P.ring_lo;
    sp.ring_hi = (int)P.ring_hi;
    sp.full_lo = (int)P.full_lo;
    sp.full_hi = (int)P.full_hi;
    sp.flags = P.all_sky ? kPlanAllSky : 0;
    return sp;
}

// Processes one sample from its plan.  A non-finite pointing gives NaN TOD
// (kSums) and no pairs.  With kSums the TOD is written to `o` now, or by the
// drain that redoes the sample's last queued pair.  nfall counts queued pairs
// and npairs the disc pairs (lane 0 only); cmax (kCalib) is the worst FP32
// decision error over the non-queued pairs, in units of the margin.  kBil:
// bilinear beam lookup (bilinear_f32; only the degenerate pairs are queued).
template <bool kCalib, bool kBil = false, class Action>
__device__ __forceinline__ void sample_planned(const SamplePlan& SP, const Hpx& hs,
                                               const RingT* rings, const Hpx& hb, const Beam& B,
                                               double ra, double dec, double pa, const Out& o,
                                               WarpSmem& S, Queue& Qs, int lane,
                                               unsigned int* err, Action& act,
                                               unsigned long long& nfall, float& cmax,
                                               unsigned long long& npairs)
{
    RingC* W = S.r;
    const unsigned lt_mask = (1u << lane) - 1u;
    Frame F;
    F.ra = ra;
    F.dec = dec;
    F.psi = -pa;
    if (SP.flags & kPlanBad) {
        if (Action::kSums && lane == 0) {
            store_out(o.a, o.f64, o.idx, CUDART_NAN);
            store_out(o.b, o.f64, o.idx, CUDART_NAN);
        }
        return;
    }
    // claim the next slot; one still waiting on queued pairs is freed by
    // redoing the whole queue
    const int slot = Qs.cur;
    Qs.cur = slot + 1 == kPend ? 0 : slot + 1;
    if (S.p[slot].left > 0) flush<kBil>(hs, S, Qs, lane, err, act);
    if (lane == 0) {
        Pend& Ps = S.p[slot];
        Ps.hb = hb;
        Ps.ra = F.ra;
        Ps.dec = F.dec;
        Ps.psi = F.psi;
        Ps.fb_a = Ps.fb_b = 0.0;
        Ps.beam = B.beam;
        Ps.out_a = o.a;
        Ps.out_b = o.b;
        Ps.idx = o.idx;
        Ps.npix_beam = B.npix;
        Ps.left = 0;
        Ps.open = 1;
        Ps.f64 = o.f64;
        act.stash(Ps);
    }
    static_assert(sizeof(SamplePlan) == 6 * sizeof(float4), "plan copy");
    if (lane < 6)
        reinterpret_cast<float4*>(&S.plan)[lane] = reinterpret_cast<const float4*>(&SP)[lane];
    __syncwarp();
    if constexpr (Action::kSums) act.reset();
    const SamplePlan& PL = S.plan;
    // what the pair loop reads on every pair, in registers
    F.s0 = PL.s0f;
    F.sps = PL.sps;
    F.cps = PL.cps;
    F.c2p = PL.c2p;
    F.s2p = PL.s2p;
    const Beam& Bh = B;

    for (long long r0 = PL.full_lo; r0 <= PL.full_hi; r0 += 32) {
        const long long ring = r0 + lane;
        int cnt = 0;
        RingC rc;
        rc.n1 = 0;
        if (ring <= PL.full_hi) {
            const RingT rt = rings[ring - 1];
            RingSpan sp = fast_disc_ring(hs, PL, PL.cosr, ring, rt);
            // every pixel of the ring's range(s) must lie in the sky map:
            // checked here, once per ring, instead of once per pair
            if (sp.start1 < 0 || sp.start1 + sp.n1 > hs.npix ||
                (sp.n2 > 0 && (sp.start2 < 0 || sp.start2 + sp.n2 > hs.npix))) {
                record(err, kCheckSkyIndex);
                sp = RingSpan{0, 0, 0, 0};
            }
            cnt = (int)(sp.n1 + sp.n2);
            if (cnt) {
                const double sh = (rt.npix2 & 1) ? 0.5 : 0.0;
                const double phi_f = PL.phi_f;
                const double jc = floor(phi_f * rt.fr - sh + 0.5);
                rc.dc = (float)((jc + sh) * rt.dphi - phi_f);
                rc.dphi = rt.dphif;
                rc.si = rt.s;
                // sin and 1 - cos of the latitude offset D: FP32 series at the
                // rounded offset, first-order correction by its rounding error
                const double dd = rt.dec - PL.dec0;
                const float df = (float)dd;
                const float de = (float)(dd - (double)df);
                float sD, hD;
                sin_versin(df, sD, hD);
                rc.Di = fmaf(de, 1.0f - hD, sD);
                rc.Ki = fmaf(de, sD, hD);
                rc.Zs = rt.s * PL.z0f;
                rc.Wz = PL.s0f * rt.zf;
                rc.Pp = rt.s * PL.s0f;
                rc.nr = rt.npix2 >> 1;
                rc.b1 = (int)(sp.start1 - rt.start) - (int)jc;
                rc.b2 = (int)(sp.start2 - rt.start) - (int)jc - (int)sp.n1;
            }
            rc.n1 = (int)sp.n1;
            rc.s1 = (int)sp.start1;
            rc.s2 = (int)sp.start2 - (int)sp.n1;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        rc.incl = incl;
        rc.base = incl - cnt;
        W[lane] = rc;
        __syncwarp();
        if (lane == 0) npairs += (unsigned long long)total;
        int k = 0;  // lane slot (ring) owning the current pair; only moves forward
        const int iters = (total + 31) >> 5;
        for (int it = 0; it < iters; ++it) {
            const int t = (it << 5) + lane;
            bool fb = false;
            int pix = 0;
            if (t < total) {
                while (W[k].incl <= t) ++k;
                const int4 R2 = *reinterpret_cast<const int4*>(&W[k].s1);
                const int4 R3 = *reinterpret_cast<const int4*>(&W[k].n1);
                const int u = t - R3.w;  // index within the ring's pixels
                const bool first = u < R3.x;
                pix = (first ? R2.x : R2.y) + u;
                int kk = (first ? R2.z : R2.w) + u;
                const int nr = R3.y;
                if (kk >= (nr >> 1)) kk -= nr;
                if (kk < -(nr >> 1)) kk += nr;
                {
                    const float4 R0 = *reinterpret_cast<const float4*>(&W[k].dc);
                    const float4 R1 = *reinterpret_cast<const float4*>(&W[k].Ki);
                    const float dl = fmaf(small_int_to_float(kk), R0.y, R0.x);
                    float sn, h;
                    sin_versin(dl, sn, h);
                    const float u_e = R0.z * sn;
                    const float v_n = fmaf(R1.y, h, R0.w);
                    const float q = fmaf(R1.w, h, R1.x);
                    const float nb = F.s0 * sn;
                    const float db = fmaf(R1.z, h, -R0.w);
                    const float X = fmaf(u_e, F.sps, -v_n * F.cps);
                    const float Y = fmaf(u_e, F.cps, v_n * F.sps);
                    int qd;
                    float yy, xx;
                    if (Y >= 0.0f) {
                        if (X > 0.0f) { qd = 0; yy = Y; xx = X; }
                        else { qd = 1; yy = -X; xx = Y; }
                    } else {
                        if (X <= 0.0f) { qd = 2; yy = -Y; xx = -X; }
                        else { qd = 3; yy = X; xx = -Y; }
                    }
                    const float tp = quarter_turns(yy, xx);
                    const float r = Bh.rscale * (q * rsqrtf(q));
                    // exp(2i (beta + alpha)) = w^2 / |w|^2, w = (db + i nb)(v + i u),
                    // then rotated by exp(2i psi)
                    auto phasor = [&](float& c2, float& s2) {
                        const float wr = fmaf(db, v_n, -nb * u_e);
                        const float wi = fmaf(db, u_e, nb * v_n);
                        const float iw = rcp_approx(fmaf(wr, wr, wi * wi));
                        const float er = fmaf(wr, wr, -wi * wi) * iw;
                        const float ei = 2.0f * wr * wi * iw;
                        c2 = fmaf(er, F.c2p, -ei * F.s2p);
                        s2 = fmaf(ei, F.c2p, er * F.s2p);
                    };
                    if constexpr (kBil && Action::kStencil) {
                        fb = q < kTinyQ;
                        int px[4];
                        float w[4];
                        if (!fb && stencil_f32(Bh, qd, tp, r, px, w)) {
                            float c2, s2;
                            phasor(c2, s2);
                            act.pair_stencil(pix, act.fetch(pix), px, w, c2, s2);
                        } else if constexpr (HasOutside<Action>::value) {
                            if (!fb) act.outside(pix, -1);
                        }
                    } else if constexpr (kBil) {
                        fb = q < kTinyQ;
                        F8 Bv;
                        if (!fb && bilinear_f32(Bh, qd, tp, r, Bv)) {
                            float c2, s2;
                            phasor(c2, s2);
                            act.pair(pix, act.fetch(pix), Bv, -1, c2, s2);
                        } else if constexpr (HasOutside<Action>::value) {
                            if (!fb) act.outside(pix, -1);
                        }
                    } else {
                        const float av = tp * r;
                        const float bv = (1.0f - tp) * r;
#if PISCO_FAST_FLOOR
                        // floors and fractional parts by FP32 additions (no
                        // conversion instructions), the same values as the
                        // conversions: see split_floor
                        float fa, fbv, fc;
                        const int jp = split_floor(av, fa), jm = split_floor(bv, fbv);
                        const int ir = jp + jm + 1;
                        const float irf = __int_as_float(ir + kTwo23Bits) - kTwo23;
                        const float cv = tp * irf;
                        const int ipr = split_floor(cv, fc);
                        const float m = kMarginRel * (r + 1.0f);
                        const float mc = kMarginRel * (irf + 1.0f);
                        fb = q < kTinyQ || fa < m || 1.0f - fa < m || fbv < m ||
                             1.0f - fbv < m || fc < mc || 1.0f - fc < mc;
#else
                        const int jp = (int)av, jm = (int)bv;
                        const int ir = jp + jm + 1;
                        const float cv = tp * (float)ir;
                        const int ipr = (int)cv;
                        const float m = kMarginRel * (r + 1.0f);
                        fb = q < kTinyQ || near_int(av, m) || near_int(bv, m) ||
                             near_int(cv, kMarginRel * ((float)ir + 1.0f));
#endif
                        if (kCalib && !fb) {
                            double rho, sig, chi;
                            (void)pair_beam_pixel(hs, hb, pix, F.ra, F.dec, F.psi, &rho, &sig, &chi);
                            const double tt = fmodulo(sig * kInvHalfPi, 4.0);
                            const double tpd = tt - floor(tt);
                            const double rd = (double)Bh.nside * sqrt(3.0 * (1.0 - cos(rho)));
                            const double e1 = fabs(av - tpd * rd) / (r + 1.0);
                            const double e2 = fabs(bv - (1.0 - tpd) * rd) / (r + 1.0);
                            const double e3 = fabs(cv - tpd * (double)ir) / ((double)ir + 1.0);
                            cmax = fmaxf(cmax, (float)fmax(fmax(e1, e2), e3) / kMarginRel);
                        }
                        if (!fb) {
                            const int bp = 2 * ir * (ir - 1) + qd * ir + ipr;
                            if ((unsigned)bp < (unsigned)Bh.npix) {  // 0 <= bp < npix
                                float c2, s2;
                                phasor(c2, s2);
                                act.pair(pix, act.fetch(pix), load_beam(Bh.beam + bp), bp, c2, s2);
                            } else if constexpr (HasOutside<Action>::value) {
                                act.outside(pix, bp);
                            }
                        }
                    }
                }
            }
            // queue near-edge pairs; redo them 32 at a time in FP64
            const unsigned mk = __ballot_sync(kFull, fb);
            if (mk) {
                if (fb) {
                    const int at = Qs.n + __popc(mk & lt_mask);
                    S.q[at] = pix;
                    S.qs[at] = (unsigned char)slot;
                }
                Qs.n += __popc(mk);
                if (lane == 0) {
                    nfall += __popc(mk);
                    S.p[slot].left += __popc(mk);
                }
                __syncwarp();
                if (Qs.n >= 32) drain<kBil>(hs, 32, S, Qs, lane, err, act);
            }
        }
        __syncwarp();
    }
    if constexpr (Action::kSums) {
        double ta, tb;
        act.total(ta, tb);
        if (lane == 0) {
            Pend& Ps = S.p[slot];
            Ps.main_a = ta;
            Ps.main_b = tb;
            Ps.open = 0;
            if (Ps.left == 0) finalize(Ps);
        }
    } else if (lane == 0) {
        S.p[slot].open = 0;
    }
    __syncwarp();
}

// Processes one sample, its plan built here by the warp.
template <bool kCalib, bool kBil = false, class Action>
__device__ __forceinline__ void sample(const Hpx& hs, const RingT* rings, const Hpx& hb,
                                       const Beam& B, double ra, double dec, double pa,
                                       const Out& o, WarpSmem& S, Queue& Qs, int lane,
                                       unsigned int* err, Action& act, unsigned long long& nfall,
                                       float& cmax, unsigned long long& npairs)
{
    sample_planned<kCalib, kBil>(make_plan(hs, B, ra, dec, pa), hs, rings, hb, B, ra, dec, pa, o,
                                 S, Qs, lane, err, act, nfall, cmax, npairs);
}

// Forward action: gather the sky, multiply by the beam, compensated sums.
struct Gather {
    static constexpr bool kSums = true;
    static constexpr bool kStencil = false;
    const float4* sky;
    float sa, ca, sb, cb;
    __device__ __forceinline__ void reset() { sa = ca = sb = cb = 0.0f; }
    __device__ __forceinline__ float4 fetch(int pix) const { return __ldg(&sky[pix]); }
    __device__ __forceinline__ static void contrib(const float4& S, const F8& B, float c2, float s2,
                                                  float& ta, float& tb)
    {
        ta = S.x * B.a.x + S.y * (B.a.y * c2 - B.a.z * s2) + S.z * (B.a.z * c2 + B.a.y * s2) +
             S.w * B.a.w;
        tb = S.x * B.b.x + S.y * (-B.b.y * c2 + B.b.z * s2) + S.z * (-B.b.z * c2 - B.b.y * s2) +
             S.w * B.b.w;
    }
    __device__ __forceinline__ void pair(int, const float4& S, const F8& B, int, float c2, float s2)
    {
        float ta, tb;
        contrib(S, B, c2, s2, ta, tb);
        two_sum(sa, ca, ta);
        two_sum(sb, cb, tb);
    }
    __device__ __forceinline__ void stash(Pend&) const {}
    __device__ __forceinline__ void deferred(const Pend&, int pix, const F8& B, int, float c2, float s2,
                                            float& ta, float& tb) const
    {
        contrib(fetch(pix), B, c2, s2, ta, tb);
    }
    // warp total (fixed shuffle tree: deterministic)
    __device__ __forceinline__ void total(double& a, double& b) const
    {
        a = (double)sa + (double)ca;
        b = (double)sb + (double)cb;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(kFull, a, o);
            b += __shfl_xor_sync(kFull, b, o);
        }
    }
};

}  // namespace tuned
}  // namespace pisco
