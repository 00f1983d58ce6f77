// tuned_core.cuh -- per-sample body of the TUNED geometry, shared by the
// single-detector forward (fwd_tuned.cu), the batched multi-detector forward
// (fwd_batched.cu) and the adjoint (adjoint.cu).
//
// For one sample, a warp evaluates the HEALPix query_disc rings in FP64 (the
// same code as the PLAIN form, so the disc is identical), rounds per-ring
// small-offset constants to FP32 once, and strides the disc pairs across
// lanes.  Per pair, FP32 only: longitude offset from a per-ring anchor pixel,
// cancellation-free boresight-frame components, the beam grid's polar-cap
// indices and exp(2i chi) as a product of unit phasors.  Any of the three
// floor decisions lying within the margin of an integer, and any pair within
// 2e-6 rad of the boresight, is queued and redone 32 at a time with the FP64
// chain of the PLAIN form (hpx.cuh pair_beam_pixel), so every pair lands on
// the same beam pixel as in the PLAIN form.
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
// The per-pair work is handed to an Action:
//   void pair(int pix, const F8& beam, float c2, float s2)
// (c2, s2 = cos 2chi, sin 2chi).
#pragma once

#include <math_constants.h>

#include "hpx.cuh"
#include "internal.h"

namespace pisco {
namespace tuned {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kQCap = 64;
// Decisions whose FP32 value lies within kMarginRel * (value + 1) of an
// integer are redone in FP64 (about 20 FP32 ulps).  The observed worst case
// over a workload is measured by pisco_tuned_calibrate and must stay well
// below this bound.
constexpr float kMarginRel = 1.2e-6f;
// Pairs with 1 - cos(rho) below this take the reference's degenerate branch
// (rho <= 1e-6, sphtrigo.cpp:40-48) and are done in FP64.
constexpr float kTinyQ = 4.0e-12f;

struct Batch {
    int incl[32];
    int cnt[32];
    int n1[32];
    int s1[32];
    int s2[32];
    int b1[32];
    int b2[32];
    int nr[32];
    float dc[32];
    float dphi[32];
    float si[32];
    float Di[32];
    float Ki[32];
    float Zs[32];
    float Wz[32];
    float Pp[32];
};

// Per-warp shared state: one ring batch and the FP64 re-evaluation queue.
struct WarpSmem {
    Batch b;
    int q[kQCap];
};

struct Beam {
    const F8* beam;
    int nside;
    int npix;
    double rho_max;
    float rscale;  // sqrt(3) * nside
};

struct Frame {
    double ra, dec, psi;
    float s0, z0, sps, cps, c2p, s2p;
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

__device__ __forceinline__ bool near_int(float x, float m)
{
    const float f = x - floorf(x);
    return f < m || f > 1.0f - m;
}

// FP64 chain of the PLAIN form for one queued pair.
template <class Action>
__device__ __forceinline__ void fallback_pair(const Hpx& hs, const Hpx& hb, const Beam& B, int pix,
                                           const Frame& F, unsigned int* err, Action& act)
{
    double rho, sig, chi;
    const long long bp = pair_beam_pixel(hs, hb, pix, F.ra, F.dec, F.psi, &rho, &sig, &chi);
    if (bp >= B.npix) return;
    if (bp < 0) {
        record(err, kCheckBeamIndex);
        return;
    }
    act.pair(pix, B.beam[bp], (float)cos(2.0 * chi), (float)sin(2.0 * chi));
}

// Processes one sample; returns false (and does nothing) for a non-finite
// pointing.  nfall counts queued pairs (lane 0 only); cmax (kCalib) is the
// worst FP32 decision error over the non-queued pairs, in units of the margin.
template <bool kCalib, class Action>
__device__ __forceinline__ bool sample(const Hpx& hs, const Hpx& hb, const Beam& B, double ra,
                                       double dec, double pa, WarpSmem& S, int lane,
                                       unsigned int* err, Action& act,
                                       unsigned long long& nfall, float& cmax)
{
    Batch& W = S.b;
    int* Q = S.q;
    const unsigned lt_mask = (1u << lane) - 1u;
    Frame F;
    F.ra = ra;
    F.dec = dec;
    F.psi = -pa;
    if (!(isfinite(F.ra) && isfinite(F.dec) && isfinite(F.psi))) return false;
    const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, F.dec), F.ra, B.rho_max);
    const double z0d = sin(F.dec), s0d = cos(F.dec);
    F.s0 = (float)s0d;
    F.z0 = (float)z0d;
    F.sps = (float)sin(F.psi);
    F.cps = (float)cos(F.psi);
    F.c2p = (float)cos(2.0 * F.psi);
    F.s2p = (float)sin(2.0 * F.psi);
    int qn = 0;

    for (long long r0 = P.full_lo; r0 <= P.full_hi; r0 += 32) {
        const long long ring = r0 + lane;
        int cnt = 0;
        if (ring <= P.full_hi) {
            const RingSpan sp = disc_ring(hs, P, ring);
            cnt = (int)(sp.n1 + sp.n2);
            if (cnt) {
                const RingInfo ri = ring_info(hs, ring);
                const double z = ring2z(hs, ring);
                const double si = sqrt(PD_MUL(PD_SUB(1.0, z), PD_ADD(1.0, z)));
                const double dz = z - z0d, ds = si - s0d;
                const double n = (double)ri.npix;
                const double dphi = kTwoPi / n;
                const double sh = ri.shifted ? 0.5 : 0.0;
                const double jc = floor(P.phi / dphi - sh + 0.5);
                W.dc[lane] = (float)((jc + sh) * dphi - P.phi);
                W.dphi[lane] = (float)dphi;
                W.si[lane] = (float)si;
                W.Di[lane] = (float)(z * s0d - si * z0d);
                W.Ki[lane] = (float)(0.5 * (dz * dz + ds * ds));
                W.Zs[lane] = (float)(si * z0d);
                W.Wz[lane] = (float)(s0d * z);
                W.Pp[lane] = (float)(si * s0d);
                W.nr[lane] = (int)ri.npix;
                W.b1[lane] = (int)(sp.start1 - ri.start) - (int)jc;
                W.b2[lane] = (int)(sp.start2 - ri.start) - (int)jc;
            }
            W.n1[lane] = (int)sp.n1;
            W.s1[lane] = (int)sp.start1;
            W.s2[lane] = (int)sp.start2;
        } else {
            W.n1[lane] = 0;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        W.incl[lane] = incl;
        W.cnt[lane] = cnt;
        __syncwarp();
        int k = 0;  // lane slot (ring) owning the current pair; only moves forward
        const int iters = (total + 31) >> 5;
        for (int it = 0; it < iters; ++it) {
            const int t = (it << 5) + lane;
            bool fb = false;
            int pix = 0;
            if (t < total) {
                while (W.incl[k] <= t) ++k;
                const int u = t - (W.incl[k] - W.cnt[k]);
                const int n1 = W.n1[k];
                int kk;
                if (u < n1) {
                    pix = W.s1[k] + u;
                    kk = W.b1[k] + u;
                } else {
                    pix = W.s2[k] + (u - n1);
                    kk = W.b2[k] + (u - n1);
                }
                const int nr = W.nr[k];
                if (kk >= (nr >> 1)) kk -= nr;
                if (kk < -(nr >> 1)) kk += nr;
                if (pix < 0 || pix >= hs.npix) {
                    record(err, kCheckSkyIndex);
                } else {
                    const float dl = fmaf((float)kk, W.dphi[k], W.dc[k]);
                    float sn, cs;
                    sincosf(dl, &sn, &cs);
                    const float h = (cs > 0.0f) ? (sn * sn) / (1.0f + cs) : 1.0f - cs;
                    const float u_e = W.si[k] * sn;
                    const float v_n = fmaf(W.Zs[k], h, W.Di[k]);
                    const float q = fmaf(W.Pp[k], h, W.Ki[k]);
                    const float nb = F.s0 * sn;
                    const float db = fmaf(W.Wz[k], h, -W.Di[k]);
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
                    const float tp = atan2f(yy, xx) * 0.63661977236758134f;
                    const float r = B.rscale * sqrtf(q);
                    const float av = tp * r;
                    const float bv = (1.0f - tp) * r;
                    const int jp = (int)av, jm = (int)bv;
                    const int ir = jp + jm + 1;
                    const float cv = tp * (float)ir;
                    const int ipr = (int)cv;
                    const float m = kMarginRel * (r + 1.0f);
                    fb = q < kTinyQ || near_int(av, m) || near_int(bv, m) ||
                         near_int(cv, kMarginRel * ((float)ir + 1.0f));
                    if (kCalib && !fb) {
                        double rho, sig, chi;
                        (void)pair_beam_pixel(hs, hb, pix, F.ra, F.dec, F.psi, &rho, &sig, &chi);
                        const double tt = fmodulo(sig * kInvHalfPi, 4.0);
                        const double tpd = tt - floor(tt);
                        const double rd = (double)B.nside * sqrt(3.0 * (1.0 - cos(rho)));
                        const double e1 = fabs(av - tpd * rd) / (r + 1.0);
                        const double e2 = fabs(bv - (1.0 - tpd) * rd) / (r + 1.0);
                        const double e3 = fabs(cv - tpd * (double)ir) / ((double)ir + 1.0);
                        cmax = fmaxf(cmax, (float)fmax(fmax(e1, e2), e3) / kMarginRel);
                    }
                    if (!fb) {
                        const int bp = 2 * ir * (ir - 1) + qd * ir + ipr;
                        if (bp >= 0 && bp < B.npix) {
                            const float ia = 1.0f / fmaf(u_e, u_e, v_n * v_n);
                            const float ca2 = (v_n * v_n - u_e * u_e) * ia;
                            const float sa2 = 2.0f * u_e * v_n * ia;
                            const float ib = 1.0f / fmaf(nb, nb, db * db);
                            const float cb2 = (db * db - nb * nb) * ib;
                            const float sb2 = 2.0f * nb * db * ib;
                            const float cx = cb2 * ca2 - sb2 * sa2;
                            const float sx = sb2 * ca2 + cb2 * sa2;
                            act.pair(pix, B.beam[bp], cx * F.c2p - sx * F.s2p,
                                     sx * F.c2p + cx * F.s2p);
                        }
                    }
                }
            }
            // queue near-edge pairs; redo them 32 at a time in FP64
            const unsigned mk = __ballot_sync(kFull, fb);
            if (mk) {
                if (fb) Q[qn + __popc(mk & lt_mask)] = pix;
                qn += __popc(mk);
                nfall += (lane == 0) ? __popc(mk) : 0;
                __syncwarp();
                if (qn >= 32) {
                    fallback_pair(hs, hb, B, Q[lane], F, err, act);
                    __syncwarp();
                    if (lane < qn - 32) Q[lane] = Q[32 + lane];
                    qn -= 32;
                    __syncwarp();
                }
            }
        }
        __syncwarp();
    }
    if (qn > 0) {
        if (lane < qn) fallback_pair(hs, hb, B, Q[lane], F, err, act);
        __syncwarp();
    }
    return true;
}

// Forward action: gather the sky, multiply by the beam, compensated sums.
struct Gather {
    const float4* sky;
    float sa, ca, sb, cb;
    __device__ __forceinline__ void reset() { sa = ca = sb = cb = 0.0f; }
    __device__ __forceinline__ void pair(int pix, const F8& B, float c2, float s2)
    {
        const float4 S = __ldg(&sky[pix]);
        const float ta = S.x * B.a.x + S.y * (B.a.y * c2 - B.a.z * s2) +
                         S.z * (B.a.z * c2 + B.a.y * s2) + S.w * B.a.w;
        const float tb = S.x * B.b.x + S.y * (-B.b.y * c2 + B.b.z * s2) +
                         S.z * (-B.b.z * c2 - B.b.y * s2) + S.w * B.b.w;
        two_sum(sa, ca, ta);
        two_sum(sb, cb, tb);
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

__device__ __forceinline__ void store_out(void* out, int f64, long long i, double v)
{
    if (!out) return;
    if (f64) ((double*)out)[i] = v;
    else ((float*)out)[i] = (float)v;
}

}  // namespace tuned
}  // namespace pisco
