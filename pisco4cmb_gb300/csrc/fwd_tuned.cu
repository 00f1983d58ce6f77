// fwd_tuned.cu -- TUNED forward: FP64 per-sample frame, FP32 per-pair
// geometry, FP64 re-evaluation of near-edge decisions, FP32 products with
// compensated accumulation.
//
// Same result as the reference chain (convolver.cpp:112-221) pair by pair:
// the disc is HEALPix query_disc evaluated in FP64 per (sample, ring) with
// the same code as the PLAIN form, and every nearest-beam-pixel decision is
// either taken in FP32 where it is at least `margin` away from a pixel edge
// or recomputed with the FP64 chain of the PLAIN form.  GB300 runs FP64 at
// a small fraction of its FP32 rate, so the per-pair FP64 transcendentals
// of the reference (about twelve per pair) cannot stay on the hot path.
//
// Per-pair geometry without cancellation.  With the pixel at ring height z
// (s = sqrt(1 - z^2)), longitude offset D from the boresight (z0, s0) and
// h = 1 - cos D, the boresight-frame quantities are
//   east  u  = s sin D                     north v = sin(dec - dec0) + s z0 h
//   1 - cos(rho) = (1 - cos(dec - dec0)) + s s0 h
//   toward-boresight at the pixel: (s0 sin D, sin(dec0 - dec) + s0 z h)
// where every per-ring term is formed in FP64 and rounded once, so each
// per-pair FP32 quantity carries a relative (not absolute) error.  The
// HEALPix polar-cap index of the beam grid follows from
//   r = sqrt(3) nside_b sqrt(1 - cos rho),  sigma = pi - alpha - psi
// (alpha = atan2(u, v)), and exp(2i chi) = exp(2i beta) exp(2i alpha)
// exp(2i psi) is a product of unit phasors (no trigonometric call).
#include <math_constants.h>

#include "hpx.cuh"
#include "internal.h"

namespace pisco {
namespace {

constexpr int kTW = 8;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kQCap = 64;
// Decisions whose FP32 value lies within kMarginRel * (value + 1) of an
// integer are redone in FP64.  ~20 FP32 ulps; the observed worst case
// (pisco_tuned_calibrate) is reported by the tests against this bound.
constexpr float kMarginRel = 1.2e-6f;
// Pairs closer than this to the boresight (1 - cos rho below it) take the
// reference's degenerate branch (rho <= 1e-6) and are done in FP64.
constexpr float kTinyQ = 4.0e-12f;

struct TBatch {
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

struct SampleFrame {
    double ra, dec, psi;
    float s0, z0, sps, cps, c2p, s2p;
};

// FP64 chain of the PLAIN form for one pair, then multiply-accumulate.
__device__ __noinline__ void fallback_pair(const FwdArgs& a, const Hpx& hs, const Hpx& hb,
                                           int pix, const SampleFrame& F, float& sa, float& ca,
                                           float& sb, float& cb)
{
    double rho, sig, chi;
    const long long bp = pair_beam_pixel(hs, hb, pix, F.ra, F.dec, F.psi, &rho, &sig, &chi);
    if (bp >= a.npix_beam) return;
    if (bp < 0) {
        record(a.err, kCheckBeamIndex);
        return;
    }
    const float c2 = (float)cos(2.0 * chi), s2 = (float)sin(2.0 * chi);
    const float4 S = __ldg(&a.sky32[pix]);
    const F8 B = a.beam32[bp];
    const float ta = S.x * B.a.x + S.y * (B.a.y * c2 - B.a.z * s2) +
                     S.z * (B.a.z * c2 + B.a.y * s2) + S.w * B.a.w;
    const float tb = S.x * B.b.x + S.y * (-B.b.y * c2 + B.b.z * s2) +
                     S.z * (-B.b.z * c2 - B.b.y * s2) + S.w * B.b.w;
    two_sum(sa, ca, ta);
    two_sum(sb, cb, tb);
}

template <bool kCalib>
__global__ void __launch_bounds__(kTW * 32, 2)
    tuned_kernel(FwdArgs a, float rscale, float* calib)
{
    __shared__ TBatch shb[kTW];
    __shared__ int shq[kTW][kQCap];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    TBatch& W = shb[wib];
    int* Q = shq[wib];
    const unsigned lt_mask = (1u << lane) - 1u;
    const Hpx hs = hpx_make(a.nside_sky);
    const Hpx hb = hpx_make(a.nside_beam);
    const long long gw = (long long)blockIdx.x * kTW + wib;
    const long long nw = (long long)gridDim.x * kTW;
    unsigned long long nfall = 0;
    float cmax = 0.0f;

    for (long long i = gw; i < a.n; i += nw) {
        const long long s = a.begin + i;
        SampleFrame F;
        F.ra = a.ra[s];
        F.dec = a.dec[s];
        F.psi = -a.pa[s];
        if (!(isfinite(F.ra) && isfinite(F.dec) && isfinite(F.psi))) {
            // non-finite pointing: NaN out (never let it reach the ring loop bounds)
            if (lane == 0) {
                if (a.out_f64) {
                    if (a.out_a) ((double*)a.out_a)[i] = CUDART_NAN;
                    if (a.out_b) ((double*)a.out_b)[i] = CUDART_NAN;
                } else {
                    if (a.out_a) ((float*)a.out_a)[i] = CUDART_NAN_F;
                    if (a.out_b) ((float*)a.out_b)[i] = CUDART_NAN_F;
                }
            }
            continue;
        }
        const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, F.dec), F.ra, a.rho_max);
        const double z0d = sin(F.dec), s0d = cos(F.dec);
        F.s0 = (float)s0d;
        F.z0 = (float)z0d;
        F.sps = (float)sin(F.psi);
        F.cps = (float)cos(F.psi);
        F.c2p = (float)cos(2.0 * F.psi);
        F.s2p = (float)sin(2.0 * F.psi);
        float sa = 0.f, ca = 0.f, sb = 0.f, cb = 0.f;
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
            int k = 0;  // owner ring (lane slot) of the current pair
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
                        record(a.err, kCheckSkyIndex);
                    } else {
                        // ---- FP32 per-pair geometry
                        const float dl = fmaf((float)kk, W.dphi[k], W.dc[k]);
                        float sn, cs;
                        sincosf(dl, &sn, &cs);
                        const float h = (cs > 0.0f) ? (sn * sn) / (1.0f + cs) : 1.0f - cs;
                        const float si = W.si[k];
                        const float u_e = si * sn;
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
                        const float r = rscale * sqrtf(q);
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
                            // FP64 reference values of the three decisions
                            double rho, sig, chi;
                            (void)pair_beam_pixel(hs, hb, pix, F.ra, F.dec, F.psi, &rho, &sig, &chi);
                            const double tt = fmodulo(sig * kInvHalfPi, 4.0);
                            const double tpd = tt - floor(tt);
                            const double rd = (double)a.nside_beam * sqrt(3.0 * (1.0 - cos(rho)));
                            const double e1 = fabs(av - tpd * rd) / (r + 1.0);
                            const double e2 = fabs(bv - (1.0 - tpd) * rd) / (r + 1.0);
                            const double e3 = fabs(cv - tpd * (double)ir) / ((double)ir + 1.0);
                            const double c2d = cos(2.0 * chi);
                            cmax = fmaxf(cmax, (float)fmax(fmax(e1, e2), e3) / kMarginRel);
                            (void)c2d;
                        }
                        if (!fb) {
                            const int bp = 2 * ir * (ir - 1) + qd * ir + ipr;
                            if (bp >= 0 && bp < a.npix_beam) {
                                // exp(2i chi) = exp(2i beta) exp(2i alpha) exp(2i psi)
                                const float ia = 1.0f / fmaf(u_e, u_e, v_n * v_n);
                                const float ca2 = (v_n * v_n - u_e * u_e) * ia;
                                const float sa2 = 2.0f * u_e * v_n * ia;
                                const float ib = 1.0f / fmaf(nb, nb, db * db);
                                const float cb2 = (db * db - nb * nb) * ib;
                                const float sb2 = 2.0f * nb * db * ib;
                                const float cx = cb2 * ca2 - sb2 * sa2;
                                const float sx = sb2 * ca2 + cb2 * sa2;
                                const float c2 = cx * F.c2p - sx * F.s2p;
                                const float s2 = sx * F.c2p + cx * F.s2p;
                                const float4 S = __ldg(&a.sky32[pix]);
                                const F8 B = a.beam32[bp];
                                const float ta = S.x * B.a.x + S.y * (B.a.y * c2 - B.a.z * s2) +
                                                 S.z * (B.a.z * c2 + B.a.y * s2) + S.w * B.a.w;
                                const float tb = S.x * B.b.x + S.y * (-B.b.y * c2 + B.b.z * s2) +
                                                 S.z * (-B.b.z * c2 - B.b.y * s2) + S.w * B.b.w;
                                two_sum(sa, ca, ta);
                                two_sum(sb, cb, tb);
                            }
                        }
                    }
                }
                // ---- queue near-edge pairs; drain 32 at a time in FP64
                const unsigned m = __ballot_sync(kFull, fb);
                if (m) {
                    if (fb) Q[qn + __popc(m & lt_mask)] = pix;
                    qn += __popc(m);
                    nfall += (lane == 0) ? __popc(m) : 0;
                    __syncwarp();
                    if (qn >= 32) {
                        fallback_pair(a, hs, hb, Q[lane], F, sa, ca, sb, cb);
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
            if (lane < qn) fallback_pair(a, hs, hb, Q[lane], F, sa, ca, sb, cb);
            qn = 0;
            __syncwarp();
        }
        double da = (double)sa + (double)ca;
        double dbb = (double)sb + (double)cb;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            da += __shfl_xor_sync(kFull, da, o);
            dbb += __shfl_xor_sync(kFull, dbb, o);
        }
        if (lane == 0) {
            if (a.out_f64) {
                if (a.out_a) ((double*)a.out_a)[i] = da;
                if (a.out_b) ((double*)a.out_b)[i] = dbb;
            } else {
                if (a.out_a) ((float*)a.out_a)[i] = (float)da;
                if (a.out_b) ((float*)a.out_b)[i] = (float)dbb;
            }
        }
    }
    if (lane == 0 && nfall && a.fallbacks) atomicAdd(a.fallbacks, nfall);
    if (kCalib && calib) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cmax = fmaxf(cmax, __shfl_xor_sync(kFull, cmax, o));
        if (lane == 0) atomicMax((int*)calib, __float_as_int(cmax));
    }
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

}  // namespace

bool tuned_supported(int nside_beam, int npix_beam, double rho_max)
{
    // The FP32 geometry uses the polar-cap branch of the beam grid's
    // ang2pix: every pair must land in a ring well inside the north cap.
    if (!(rho_max > 0.0) || rho_max > 0.5) return false;
    const double ring = nside_beam * sqrt(3.0 * (1.0 - cos(rho_max)));
    if (ring + 2.0 >= nside_beam) return false;
    const long long ncap = 2LL * nside_beam * (nside_beam - 1);
    return npix_beam <= ncap;
}

static cudaError_t launch_tuned_impl(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib)
{
    if (a.n <= 0) return cudaSuccess;
    const int threads = kTW * 32;
    const float rscale = (float)(1.7320508075688772 * (double)a.nside_beam);
    const long long need = (a.n + kTW - 1) / kTW;
    if (calib) {
        long long blocks = (long long)sm_count * resident_blocks(tuned_kernel<true>, threads);
        tuned_kernel<true><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, rscale, calib);
    } else {
        long long blocks = (long long)sm_count * resident_blocks(tuned_kernel<false>, threads);
        tuned_kernel<false><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, rscale, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_forward_tuned(const FwdArgs& a, int sm_count, cudaStream_t st)
{
    return launch_tuned_impl(a, sm_count, st, nullptr);
}

cudaError_t launch_tuned_calibrate(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib)
{
    return launch_tuned_impl(a, sm_count, st, calib);
}

}  // namespace pisco
