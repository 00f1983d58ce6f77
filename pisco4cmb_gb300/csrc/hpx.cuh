// hpx.cuh -- HEALPix RING geometry and the beam-frame rotation, shared by
// the device kernels and the host side of libpisco_gb300.
//
// Written from the published HEALPix algorithms (Gorski et al. 2005,
// ApJ 622:759; HEALPix C++ 3.x Healpix_Base: ring_above, ring2z,
// get_ring_info_small/get_ring_info2, pix2loc/pix2ang, loc2pix/ang2pix,
// query_disc (non-inclusive) and get_interpol), which the reference calls
// from Healpix C++ (src/Convolver/convolver.cpp:137-138,150,187;
// src/GpuConvolver/gpuconvolver.cu:490-492) and partly ports to the GPU
// (src/GpuConvolver/cuda/cudaHealpix.cu:45-259), and from the
// rho/sigma/chi rotation of src/Sphtrigo/sphtrigo.cpp:4-55 (device twin
// src/GpuConvolver/cuda/cudaSphtransf.cu:3-54).
//
// Every multiply/add/subtract on an index-determining path goes through
// PD_* so that the device never contracts it into a fused multiply-add:
// the pixel a point falls in is then decided by the same rounded
// operations on the host (compiled with -ffp-contract=off) and on the GPU.
// Only the transcendental functions (cos, sin, acos, atan2) may differ by
// an ulp between the host libm and the CUDA math library, which changes a
// decision only at exact ties.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define PHD __host__ __device__ __forceinline__
#else
#define PHD inline
#endif

#if defined(__CUDA_ARCH__)
#define PD_MUL(a, b) __dmul_rn((a), (b))
#define PD_ADD(a, b) __dadd_rn((a), (b))
#define PD_SUB(a, b) __dsub_rn((a), (b))
#define PD_DIV(a, b) __ddiv_rn((a), (b))
#else
#define PD_MUL(a, b) ((a) * (b))
#define PD_ADD(a, b) ((a) + (b))
#define PD_SUB(a, b) ((a) - (b))
#define PD_DIV(a, b) ((a) / (b))
#endif

namespace pisco {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr double kTwoPi = 6.283185307179586476925286766559005768394;
constexpr double kHalfPi = 1.570796326794896619231321691639751442099;
constexpr double kInvHalfPi = 0.6366197723675813430755350534900574;
constexpr double kInvTwoPi = 0.1591549430918953357688837633725143620345;
constexpr double kTwoThird = 2.0 / 3.0;

struct Hpx {
    int64_t nside, npix, ncap;
    double fact1, fact2;
};

PHD Hpx hpx_make(int64_t nside)
{
    Hpx h;
    h.nside = nside;
    h.npix = 12 * nside * nside;
    h.ncap = 2 * nside * (nside - 1);
    h.fact2 = PD_DIV(4.0, (double)h.npix);
    h.fact1 = PD_MUL((double)(2 * nside), h.fact2);
    return h;
}

PHD double fmodulo(double v1, double v2)
{
    if (v1 >= 0.0) return (v1 < v2) ? v1 : fmod(v1, v2);
    double t = PD_ADD(fmod(v1, v2), v2);
    return (t == v2) ? 0.0 : t;
}

PHD int64_t isqrt64(int64_t v)
{
    int64_t r = (int64_t)sqrt(PD_ADD((double)v, 0.5));
    if (r * r > v) --r;
    else if ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

// Ring index (1-based, counted from the north pole) of the last ring at or
// north of z.
PHD int64_t ring_above(const Hpx& h, double z)
{
    const double ns = (double)h.nside;
    double az = fabs(z);
    if (az <= kTwoThird) return (int64_t)PD_MUL(ns, PD_SUB(2.0, PD_MUL(1.5, z)));
    int64_t ir = (int64_t)PD_MUL(ns, sqrt(PD_MUL(3.0, PD_SUB(1.0, az))));
    return (z > 0.0) ? ir : 4 * h.nside - ir - 1;
}

PHD double ring2z(const Hpx& h, int64_t ring)
{
    const int64_t ns = h.nside;
    if (ring < ns) return PD_SUB(1.0, PD_MUL((double)(ring * ring), h.fact2));
    if (ring <= 3 * ns) return PD_MUL((double)(2 * ns - ring), h.fact1);
    int64_t r = 4 * ns - ring;
    return PD_SUB(PD_MUL((double)(r * r), h.fact2), 1.0);
}

struct RingInfo {
    int64_t start, npix;
    bool shifted;
};

PHD RingInfo ring_info(const Hpx& h, int64_t ring)
{
    const int64_t ns = h.nside;
    RingInfo ri;
    if (ring < ns) {
        ri.shifted = true;
        ri.npix = 4 * ring;
        ri.start = 2 * ring * (ring - 1);
    } else if (ring < 3 * ns) {
        ri.shifted = ((ring - ns) & 1) == 0;
        ri.npix = 4 * ns;
        ri.start = h.ncap + (ring - ns) * 4 * ns;
    } else {
        int64_t nr = 4 * ns - ring;
        ri.shifted = true;
        ri.npix = 4 * nr;
        ri.start = h.npix - 2 * nr * (nr + 1);
    }
    return ri;
}

// ring_info plus the ring colatitude (HEALPix get_ring_info2).
PHD RingInfo ring_info_theta(const Hpx& h, int64_t ring, double* theta)
{
    const int64_t ns = h.nside;
    int64_t north = (ring > 2 * ns) ? 4 * ns - ring : ring;
    RingInfo ri;
    if (north < ns) {
        double t = PD_MUL((double)(north * north), h.fact2);
        double ct = PD_SUB(1.0, t);
        double st = sqrt(PD_MUL(t, PD_SUB(2.0, t)));
        *theta = atan2(st, ct);
        ri.npix = 4 * north;
        ri.shifted = true;
        ri.start = 2 * north * (north - 1);
    } else {
        *theta = acos(PD_MUL((double)(2 * ns - north), h.fact1));
        ri.npix = 4 * ns;
        ri.shifted = ((north - ns) & 1) == 0;
        ri.start = h.ncap + (north - ns) * ri.npix;
    }
    if (north != ring) {
        *theta = PD_SUB(kPi, *theta);
        ri.start = h.npix - ri.start - ri.npix;
    }
    return ri;
}

// Pixel centre -> (z, phi, sin(theta) where accurate) (HEALPix pix2loc).
PHD void pix2loc(const Hpx& h, int64_t pix, double* z, double* phi, double* sth,
                 bool* have_sth)
{
    const int64_t ns = h.nside;
    *have_sth = false;
    *sth = 0.0;
    if (pix < h.ncap) {
        int64_t ir = (1 + isqrt64(1 + 2 * pix)) >> 1;
        int64_t iphi = (pix + 1) - 2 * ir * (ir - 1);
        double t = PD_MUL((double)(ir * ir), h.fact2);
        *z = PD_SUB(1.0, t);
        if (*z > 0.99) {
            *sth = sqrt(PD_MUL(t, PD_SUB(2.0, t)));
            *have_sth = true;
        }
        *phi = PD_DIV(PD_MUL(PD_SUB((double)iphi, 0.5), kHalfPi), (double)ir);
    } else if (pix < h.npix - h.ncap) {
        int64_t nl4 = 4 * ns;
        int64_t ip = pix - h.ncap;
        int64_t q = ip / nl4;
        int64_t ir = q + ns;
        int64_t iphi = ip - nl4 * q + 1;
        double fodd = ((ir + ns) & 1) ? 1.0 : 0.5;
        *z = PD_MUL((double)(2 * ns - ir), h.fact1);
        *phi = PD_MUL(PD_SUB((double)iphi, fodd), PD_MUL(PD_MUL(kPi, 0.75), h.fact1));
    } else {
        int64_t ip = h.npix - pix;
        int64_t ir = (1 + isqrt64(2 * ip - 1)) >> 1;
        int64_t iphi = 4 * ir + 1 - (ip - 2 * ir * (ir - 1));
        double t = PD_MUL((double)(ir * ir), h.fact2);
        *z = PD_SUB(t, 1.0);
        if (*z < -0.99) {
            *sth = sqrt(PD_MUL(t, PD_SUB(2.0, t)));
            *have_sth = true;
        }
        *phi = PD_DIV(PD_MUL(PD_SUB((double)iphi, 0.5), kHalfPi), (double)ir);
    }
}

PHD void pix2ang(const Hpx& h, int64_t pix, double* theta, double* phi)
{
    double z, sth;
    bool hs;
    pix2loc(h, pix, &z, phi, &sth, &hs);
    *theta = hs ? atan2(sth, z) : acos(z);
}

PHD int64_t loc2pix(const Hpx& h, double z, double phi, double sth, bool have_sth)
{
    const int64_t ns = h.nside;
    const double dns = (double)ns;
    double za = fabs(z);
    double tt = fmodulo(PD_MUL(phi, kInvHalfPi), 4.0);
    if (za <= kTwoThird) {
        int64_t nl4 = 4 * ns;
        double t1 = PD_MUL(dns, PD_ADD(0.5, tt));
        double t2 = PD_MUL(PD_MUL(dns, z), 0.75);
        int64_t jp = (int64_t)PD_SUB(t1, t2);
        int64_t jm = (int64_t)PD_ADD(t1, t2);
        int64_t ir = ns + 1 + jp - jm;
        int64_t kshift = 1 - (ir & 1);
        int64_t s = jp + jm - ns + kshift + 1 + nl4 + nl4;
        int64_t ip = (s >> 1) % nl4;
        return h.ncap + (ir - 1) * nl4 + ip;
    }
    double tp = PD_SUB(tt, (double)(int64_t)tt);
    double tmp = ((za < 0.99) || !have_sth)
                     ? PD_MUL(dns, sqrt(PD_MUL(3.0, PD_SUB(1.0, za))))
                     : PD_DIV(PD_MUL(dns, sth), sqrt(PD_DIV(PD_ADD(1.0, za), 3.0)));
    int64_t jp = (int64_t)PD_MUL(tp, tmp);
    int64_t jm = (int64_t)PD_MUL(PD_SUB(1.0, tp), tmp);
    int64_t ir = jp + jm + 1;
    int64_t ip = (int64_t)PD_MUL(tt, (double)ir);
    return (z > 0.0) ? 2 * ir * (ir - 1) + ip : h.npix - 2 * ir * (ir + 1) + ip;
}

PHD int64_t ang2pix(const Hpx& h, double theta, double phi)
{
    bool hs = (theta < 0.01) || (theta > 3.14159 - 0.01);
    return loc2pix(h, cos(theta), phi, hs ? sin(theta) : 0.0, hs);
}

// 4-pixel bilinear interpolation stencil (HEALPix get_interpol, RING).
PHD void interp_ring(const Hpx& h, int64_t ring, double phi, int64_t* pa, int64_t* pb,
                     double* wa, double* wb, double* th)
{
    RingInfo ri = ring_info_theta(h, ring, th);
    double dphi = PD_DIV(kTwoPi, (double)ri.npix);
    double sh = ri.shifted ? 1.0 : 0.0;
    double tmp = PD_SUB(PD_DIV(phi, dphi), PD_MUL(0.5, sh));
    int64_t i1 = (tmp < 0.0) ? (int64_t)tmp - 1 : (int64_t)tmp;
    double w1 = PD_DIV(PD_SUB(phi, PD_MUL(PD_ADD((double)i1, PD_MUL(0.5, sh)), dphi)), dphi);
    int64_t i2 = i1 + 1;
    if (i1 < 0) i1 += ri.npix;
    if (i2 >= ri.npix) i2 -= ri.npix;
    *pa = ri.start + i1;
    *pb = ri.start + i2;
    *wa = PD_SUB(1.0, w1);
    *wb = w1;
}

PHD void get_interpol(const Hpx& h, double theta, double phi, int64_t pix[4], double wgt[4])
{
    double z = cos(theta);
    int64_t ir1 = ring_above(h, z);
    int64_t ir2 = ir1 + 1;
    double th1 = 0.0, th2 = 0.0;
    if (ir1 > 0) interp_ring(h, ir1, phi, &pix[0], &pix[1], &wgt[0], &wgt[1], &th1);
    if (ir2 < 4 * h.nside) interp_ring(h, ir2, phi, &pix[2], &pix[3], &wgt[2], &wgt[3], &th2);
    if (ir1 == 0) {
        double wt = PD_DIV(theta, th2);
        wgt[2] = PD_MUL(wgt[2], wt);
        wgt[3] = PD_MUL(wgt[3], wt);
        double f = PD_MUL(PD_SUB(1.0, wt), 0.25);
        wgt[0] = f;
        wgt[1] = f;
        wgt[2] = PD_ADD(wgt[2], f);
        wgt[3] = PD_ADD(wgt[3], f);
        pix[0] = (pix[2] + 2) & 3;
        pix[1] = (pix[3] + 2) & 3;
    } else if (ir2 == 4 * h.nside) {
        double wt = PD_DIV(PD_SUB(theta, th1), PD_SUB(kPi, th1));
        wgt[0] = PD_MUL(wgt[0], PD_SUB(1.0, wt));
        wgt[1] = PD_MUL(wgt[1], PD_SUB(1.0, wt));
        double f = PD_MUL(wt, 0.25);
        wgt[0] = PD_ADD(wgt[0], f);
        wgt[1] = PD_ADD(wgt[1], f);
        wgt[2] = f;
        wgt[3] = f;
        pix[2] = ((pix[0] + 2) & 3) + h.npix - 4;
        pix[3] = ((pix[1] + 2) & 3) + h.npix - 4;
    } else {
        double wt = PD_DIV(PD_SUB(theta, th1), PD_SUB(th2, th1));
        wgt[0] = PD_MUL(wgt[0], PD_SUB(1.0, wt));
        wgt[1] = PD_MUL(wgt[1], PD_SUB(1.0, wt));
        wgt[2] = PD_MUL(wgt[2], wt);
        wgt[3] = PD_MUL(wgt[3], wt);
    }
}

// ---------------------------------------------------------------------------
// query_disc, split so that a warp can evaluate one ring per lane.
//
// DiscPlan holds the per-pointing quantities; disc_ring() gives the pixel
// range(s) of one ring.  Rings in [full_lo, ring_lo) and (ring_hi, full_hi]
// are entirely inside the disc (the pole caps HEALPix appends whole);
// rings in [ring_lo, ring_hi] are cut by the disc edge.  The union over
// rings, in ring order, is exactly HEALPix query_disc's pixel set in
// ascending pixel order.
// ---------------------------------------------------------------------------
struct DiscPlan {
    double z0, xa, cosr, phi;
    double theta, s0;  // normalised colatitude in [0, pi] and sqrt((1 - z0)(1 + z0))
    bool flip;         // the centre was reflected (colatitude beyond pi, phi + pi)
    int64_t ring_lo, ring_hi;  // rings evaluated with the edge formula
    int64_t full_lo, full_hi;  // first and last ring touched at all
    bool all_sky;
};

PHD DiscPlan disc_plan(const Hpx& h, double theta, double phi, double radius, double cosr);

PHD DiscPlan disc_plan(const Hpx& h, double theta, double phi, double radius)
{
    return disc_plan(h, theta, phi, radius, radius >= kPi ? 0.0 : cos(radius));
}

// Same, with cos(radius) supplied by the caller (hoisted out of a loop over
// pointings); it must be cos(radius) as evaluated on the same device.
PHD DiscPlan disc_plan(const Hpx& h, double theta, double phi, double radius, double cosr)
{
    DiscPlan p;
    theta = fmodulo(theta, kTwoPi);
    p.flip = theta > kPi;
    if (p.flip) {
        phi = PD_ADD(phi, kPi);
        theta = PD_SUB(kTwoPi, theta);
    }
    p.theta = theta;
    p.phi = fmodulo(phi, kTwoPi);
    p.all_sky = radius >= kPi;
    if (p.all_sky) {
        p.ring_lo = 1;
        p.ring_hi = 0;
        p.full_lo = 1;
        p.full_hi = 4 * h.nside - 1;
        p.z0 = p.xa = p.cosr = p.s0 = 0.0;
        return p;
    }
    p.cosr = cosr;
    p.z0 = cos(theta);
    p.s0 = sqrt(PD_MUL(PD_SUB(1.0, p.z0), PD_ADD(1.0, p.z0)));
    p.xa = PD_DIV(1.0, p.s0);
    double rlat1 = PD_SUB(theta, radius);
    p.ring_lo = ring_above(h, cos(rlat1)) + 1;
    p.full_lo = (rlat1 <= 0.0 && p.ring_lo > 1) ? 1 : p.ring_lo;
    double rlat2 = PD_ADD(theta, radius);
    p.ring_hi = ring_above(h, cos(rlat2));
    p.full_hi = (rlat2 >= kPi && p.ring_hi + 1 < 4 * h.nside) ? 4 * h.nside - 1 : p.ring_hi;
    return p;
}

struct RingSpan {
    int64_t start1, n1, start2, n2;  // up to two pixel ranges (wrap at phi = 0)
};

PHD RingSpan disc_ring(const Hpx& h, const DiscPlan& p, int64_t ring)
{
    RingSpan s = {0, 0, 0, 0};
    if (ring < p.full_lo || ring > p.full_hi) return s;
    RingInfo ri = ring_info(h, ring);
    if (p.all_sky || ring < p.ring_lo || ring > p.ring_hi) {
        s.start1 = ri.start;
        s.n1 = ri.npix;
        return s;
    }
    double z = ring2z(h, ring);
    double x = PD_MUL(PD_SUB(p.cosr, PD_MUL(z, p.z0)), p.xa);
    double ysq = PD_SUB(PD_SUB(1.0, PD_MUL(z, z)), PD_MUL(x, x));
    double dphi = (ysq <= 0.0) ? 0.0 : atan2(sqrt(ysq), x);
    if (!(dphi > 0.0)) return s;
    double shift = ri.shifted ? 0.5 : 0.0;
    double fr = PD_MUL((double)ri.npix, kInvTwoPi);
    int64_t lo = (int64_t)floor(PD_SUB(PD_MUL(fr, PD_SUB(p.phi, dphi)), shift)) + 1;
    int64_t hi = (int64_t)floor(PD_SUB(PD_MUL(fr, PD_ADD(p.phi, dphi)), shift));
    if (lo > hi) return s;
    if (hi >= ri.npix) {
        lo -= ri.npix;
        hi -= ri.npix;
    }
    if (lo < 0) {
        s.start1 = ri.start;
        s.n1 = hi + 1;
        s.start2 = ri.start + lo + ri.npix;
        s.n2 = -lo;
    } else {
        s.start1 = ri.start + lo;
        s.n1 = hi - lo + 1;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Beam-frame offsets of a sky position (Ludwig-3, CMB convention):
// rho radial offset, sigma polar offset from South (clockwise), chi
// polarisation angle.  Same operations as sphtrigo.cpp:27-54.
// ---------------------------------------------------------------------------
PHD void rho_sigma_chi(double ra_bc, double dec_bc, double psi_bc, double ra_pix,
                       double dec_pix, double* rho, double* sigma, double* chi)
{
    double cdc = cos(dec_bc), sdc = sin(dec_bc);
    double cdp = cos(dec_pix), sdp = sin(dec_pix);
    double dra = PD_SUB(ra_pix, ra_bc);
    double sd = sin(dra), cd = cos(dra);
    double crho = PD_ADD(PD_MUL(sdc, sdp), PD_MUL(PD_MUL(cdc, cdp), cd));
    *rho = (crho >= 1.0) ? 0.0 : acos(crho);
    double al, be;
    if (*rho > 1.0e-6) {
        be = atan2(PD_MUL(sd, cdc), PD_SUB(PD_MUL(sdc, cdp), PD_MUL(PD_MUL(cdc, sdp), cd)));
        al = atan2(PD_MUL(sd, cdp), PD_SUB(PD_MUL(sdp, cdc), PD_MUL(PD_MUL(cdp, sdc), cd)));
    } else {
        be = kHalfPi;
        al = kHalfPi;
    }
    double sg = PD_SUB(PD_SUB(kPi, al), psi_bc);
    if (sg < 0.0) sg = PD_ADD(sg, PD_MUL(2.0, kPi));
    else if (sg > PD_MUL(2.0, kPi)) sg = PD_SUB(sg, PD_MUL(2.0, kPi));
    *sigma = sg;
    double c = PD_SUB(be, sg);
    if (c < -kPi) c = PD_ADD(c, PD_MUL(2.0, kPi));
    *chi = c;
}

// Full per-pair geometry of the reference chain: sky pixel -> (theta, phi)
// -> (rho, sigma, chi) -> nearest beam pixel.
PHD int64_t pair_beam_pixel(const Hpx& hs, const Hpx& hb, int64_t skypix, double ra_bc,
                            double dec_bc, double psi_bc, double* rho, double* sigma,
                            double* chi)
{
    double th, ph;
    pix2ang(hs, skypix, &th, &ph);
    rho_sigma_chi(ra_bc, dec_bc, psi_bc, ph, PD_SUB(PD_DIV(kPi, 2.0), th), rho, sigma, chi);
    return ang2pix(hb, *rho, *sigma);
}

}  // namespace pisco
