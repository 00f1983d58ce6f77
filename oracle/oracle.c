/*
 * oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; never linked into the
 * product).  See oracle.h for what each part restates and where from.
 *
 * Build: -O2 -fopenmp -ffp-contract=off (no fused multiply-adds, so the
 * rounding of every index-determining expression is the same on x86-64 and
 * aarch64 and matches the device code, which uses explicitly rounded
 * operations for the same expressions).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_PI 3.141592653589793238462643383279502884197
#define O_TWOPI 6.283185307179586476925286766559005768394
#define O_HALFPI 1.570796326794896619231321691639751442099
#define O_INV_HALFPI 0.6366197723675813430755350534900574
#define O_INV_TWOPI 0.1591549430918953357688837633725143620345
#define O_TWOTHIRD (2.0 / 3.0)

/* ------------------------------------------------------------------ */
/* HEALPix RING geometry (published HEALPix algorithms, C++ 3.x form)  */
/* ------------------------------------------------------------------ */

/* v1 mod v2 into [0, v2) (HEALPix fmodulo). */
static double o_fmodulo(double v1, double v2)
{
    if (v1 >= 0.0) return (v1 < v2) ? v1 : fmod(v1, v2);
    double t = fmod(v1, v2) + v2;
    return (t == v2) ? 0.0 : t;
}

/* exact integer square root (HEALPix isqrt with its correction step). */
static int64_t o_isqrt(int64_t v)
{
    int64_t r = (int64_t)sqrt((double)v + 0.5);
    if (r * r > v) --r;
    else if ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

void orc_hpx_init(orc_hpx* h, int64_t nside)
{
    h->nside = nside;
    h->npix = 12 * nside * nside;
    h->ncap = 2 * nside * (nside - 1);
    h->fact2 = 4.0 / (double)h->npix;
    h->fact1 = (double)(2 * nside) * h->fact2;
}

int64_t orc_ring_above(const orc_hpx* h, double z)
{
    const double ns = (double)h->nside;
    double az = fabs(z);
    if (az <= O_TWOTHIRD) return (int64_t)(ns * (2.0 - 1.5 * z));
    int64_t ir = (int64_t)(ns * sqrt(3.0 * (1.0 - az)));
    return (z > 0.0) ? ir : 4 * h->nside - ir - 1;
}

double orc_ring2z(const orc_hpx* h, int64_t ring)
{
    const int64_t ns = h->nside;
    if (ring < ns) return 1.0 - (double)(ring * ring) * h->fact2;
    if (ring <= 3 * ns) return (double)(2 * ns - ring) * h->fact1;
    int64_t r = 4 * ns - ring;
    return (double)(r * r) * h->fact2 - 1.0;
}

void orc_ring_info_small(const orc_hpx* h, int64_t ring, int64_t* startpix,
                         int64_t* ringpix, int* shifted)
{
    const int64_t ns = h->nside;
    if (ring < ns) {
        *shifted = 1;
        *ringpix = 4 * ring;
        *startpix = 2 * ring * (ring - 1);
    } else if (ring < 3 * ns) {
        *shifted = (((ring - ns) & 1) == 0);
        *ringpix = 4 * ns;
        *startpix = h->ncap + (ring - ns) * 4 * ns;
    } else {
        int64_t nr = 4 * ns - ring;
        *shifted = 1;
        *ringpix = 4 * nr;
        *startpix = h->npix - 2 * nr * (nr + 1);
    }
}

void orc_ring_info2(const orc_hpx* h, int64_t ring, int64_t* startpix,
                    int64_t* ringpix, double* theta, int* shifted)
{
    const int64_t ns = h->nside;
    int64_t north = (ring > 2 * ns) ? 4 * ns - ring : ring;
    if (north < ns) {
        double t = (double)(north * north) * h->fact2;
        double ct = 1.0 - t;
        double st = sqrt(t * (2.0 - t));
        *theta = atan2(st, ct);
        *ringpix = 4 * north;
        *shifted = 1;
        *startpix = 2 * north * (north - 1);
    } else {
        *theta = acos((double)(2 * ns - north) * h->fact1);
        *ringpix = 4 * ns;
        *shifted = (((north - ns) & 1) == 0);
        *startpix = h->ncap + (north - ns) * (*ringpix);
    }
    if (north != ring) {
        *theta = O_PI - *theta;
        *startpix = h->npix - *startpix - *ringpix;
    }
}

void orc_pix2ang(const orc_hpx* h, int64_t pix, double* theta, double* phi)
{
    const int64_t ns = h->nside;
    double z, sth = 0.0;
    int have_sth = 0;
    if (pix < h->ncap) {
        int64_t ir = (1 + o_isqrt(1 + 2 * pix)) >> 1;
        int64_t iphi = (pix + 1) - 2 * ir * (ir - 1);
        double t = (double)(ir * ir) * h->fact2;
        z = 1.0 - t;
        if (z > 0.99) {
            sth = sqrt(t * (2.0 - t));
            have_sth = 1;
        }
        *phi = ((double)iphi - 0.5) * O_HALFPI / (double)ir;
    } else if (pix < h->npix - h->ncap) {
        int64_t nl4 = 4 * ns;
        int64_t ip = pix - h->ncap;
        int64_t q = ip / nl4;
        int64_t ir = q + ns;
        int64_t iphi = ip - nl4 * q + 1;
        double fodd = ((ir + ns) & 1) ? 1.0 : 0.5;
        z = (double)(2 * ns - ir) * h->fact1;
        *phi = ((double)iphi - fodd) * (O_PI * 0.75 * h->fact1);
    } else {
        int64_t ip = h->npix - pix;
        int64_t ir = (1 + o_isqrt(2 * ip - 1)) >> 1;
        int64_t iphi = 4 * ir + 1 - (ip - 2 * ir * (ir - 1));
        double t = (double)(ir * ir) * h->fact2;
        z = t - 1.0;
        if (z < -0.99) {
            sth = sqrt(t * (2.0 - t));
            have_sth = 1;
        }
        *phi = ((double)iphi - 0.5) * O_HALFPI / (double)ir;
    }
    *theta = have_sth ? atan2(sth, z) : acos(z);
}

static int64_t o_loc2pix(const orc_hpx* h, double z, double phi, double sth,
                         int have_sth)
{
    const int64_t ns = h->nside;
    const double dns = (double)ns;
    double za = fabs(z);
    double tt = o_fmodulo(phi * O_INV_HALFPI, 4.0);
    if (za <= O_TWOTHIRD) {
        int64_t nl4 = 4 * ns;
        double t1 = dns * (0.5 + tt);
        double t2 = dns * z * 0.75;
        int64_t jp = (int64_t)(t1 - t2);
        int64_t jm = (int64_t)(t1 + t2);
        int64_t ir = ns + 1 + jp - jm;
        int64_t kshift = 1 - (ir & 1);
        int64_t s = jp + jm - ns + kshift + 1 + nl4 + nl4;
        int64_t ip = (s >> 1) % nl4;
        return h->ncap + (ir - 1) * nl4 + ip;
    }
    double tp = tt - (double)(int64_t)tt;
    double tmp = ((za < 0.99) || !have_sth) ? dns * sqrt(3.0 * (1.0 - za))
                                            : dns * sth / sqrt((1.0 + za) / 3.0);
    int64_t jp = (int64_t)(tp * tmp);
    int64_t jm = (int64_t)((1.0 - tp) * tmp);
    int64_t ir = jp + jm + 1;
    int64_t ip = (int64_t)(tt * (double)ir);
    return (z > 0.0) ? 2 * ir * (ir - 1) + ip : h->npix - 2 * ir * (ir + 1) + ip;
}

int64_t orc_ang2pix(const orc_hpx* h, double theta, double phi)
{
    int have_sth = (theta < 0.01) || (theta > 3.14159 - 0.01);
    return o_loc2pix(h, cos(theta), phi, have_sth ? sin(theta) : 0.0,
                     have_sth);
}

/* Append [a, b) to a sorted range list, merging a touching range (the
 * HEALPix rangeset append rule). */
static int o_push(int64_t* rg, int64_t* n, int64_t cap, int64_t a, int64_t b)
{
    if (b <= a) return 0;
    if (*n > 0 && a <= rg[2 * (*n) - 1]) {
        if (b > rg[2 * (*n) - 1]) rg[2 * (*n) - 1] = b;
        return 0;
    }
    if (*n >= cap) return -1;
    rg[2 * (*n)] = a;
    rg[2 * (*n) + 1] = b;
    ++(*n);
    return 0;
}

int64_t orc_query_disc(const orc_hpx* h, double theta, double phi,
                       double radius, int64_t* rg, int64_t cap)
{
    int64_t n = 0, sp, rp;
    int sh;
    theta = o_fmodulo(theta, O_TWOPI);
    if (theta > O_PI) {
        phi += O_PI;
        theta = O_TWOPI - theta;
    }
    phi = o_fmodulo(phi, O_TWOPI);
    if (radius >= O_PI) {
        if (o_push(rg, &n, cap, 0, h->npix)) return -1;
        return n;
    }
    double cosr = cos(radius);
    double z0 = cos(theta);
    double xa = 1.0 / sqrt((1.0 - z0) * (1.0 + z0));
    double rlat1 = theta - radius;
    int64_t irmin = orc_ring_above(h, cos(rlat1)) + 1;
    if (rlat1 <= 0.0 && irmin > 1) {
        orc_ring_info_small(h, irmin - 1, &sp, &rp, &sh);
        if (o_push(rg, &n, cap, 0, sp + rp)) return -1;
    }
    double rlat2 = theta + radius;
    int64_t irmax = orc_ring_above(h, cos(rlat2));
    for (int64_t iz = irmin; iz <= irmax; ++iz) {
        double z = orc_ring2z(h, iz);
        double x = (cosr - z * z0) * xa;
        double ysq = 1.0 - z * z - x * x;
        double dphi = (ysq <= 0.0) ? 0.0 : atan2(sqrt(ysq), x);
        if (!(dphi > 0.0)) continue;
        int64_t p1, nr;
        orc_ring_info_small(h, iz, &p1, &nr, &sh);
        double shift = sh ? 0.5 : 0.0;
        double fr = (double)nr * O_INV_TWOPI;
        int64_t lo = (int64_t)floor(fr * (phi - dphi) - shift) + 1;
        int64_t hi = (int64_t)floor(fr * (phi + dphi) - shift);
        if (lo > hi) continue;
        if (hi >= nr) {
            lo -= nr;
            hi -= nr;
        }
        if (lo < 0) {
            if (o_push(rg, &n, cap, p1, p1 + hi + 1)) return -1;
            if (o_push(rg, &n, cap, p1 + lo + nr, p1 + nr)) return -1;
        } else {
            if (o_push(rg, &n, cap, p1 + lo, p1 + hi + 1)) return -1;
        }
    }
    if (rlat2 >= O_PI && irmax + 1 < 4 * h->nside) {
        orc_ring_info_small(h, irmax + 1, &sp, &rp, &sh);
        if (o_push(rg, &n, cap, sp, h->npix)) return -1;
    }
    return n;
}

static void o_interp_ring(const orc_hpx* h, int64_t ring, double phi,
                          int64_t* pa, int64_t* pb, double* wa, double* wb,
                          double* th)
{
    int64_t sp, nr;
    int sh;
    orc_ring_info2(h, ring, &sp, &nr, th, &sh);
    double dphi = O_TWOPI / (double)nr;
    double tmp = phi / dphi - 0.5 * (double)sh;
    int64_t i1 = (tmp < 0.0) ? (int64_t)tmp - 1 : (int64_t)tmp;
    double w1 = (phi - ((double)i1 + 0.5 * (double)sh) * dphi) / dphi;
    int64_t i2 = i1 + 1;
    if (i1 < 0) i1 += nr;
    if (i2 >= nr) i2 -= nr;
    *pa = sp + i1;
    *pb = sp + i2;
    *wa = 1.0 - w1;
    *wb = w1;
}

void orc_get_interpol(const orc_hpx* h, double theta, double phi,
                      int64_t pix[4], double wgt[4])
{
    double z = cos(theta);
    int64_t ir1 = orc_ring_above(h, z);
    int64_t ir2 = ir1 + 1;
    double th1 = 0.0, th2 = 0.0;
    if (ir1 > 0) o_interp_ring(h, ir1, phi, &pix[0], &pix[1], &wgt[0], &wgt[1], &th1);
    if (ir2 < 4 * h->nside)
        o_interp_ring(h, ir2, phi, &pix[2], &pix[3], &wgt[2], &wgt[3], &th2);
    if (ir1 == 0) {
        double wt = theta / th2;
        wgt[2] *= wt;
        wgt[3] *= wt;
        double f = (1.0 - wt) * 0.25;
        wgt[0] = f;
        wgt[1] = f;
        wgt[2] += f;
        wgt[3] += f;
        pix[0] = (pix[2] + 2) & 3;
        pix[1] = (pix[3] + 2) & 3;
    } else if (ir2 == 4 * h->nside) {
        double wt = (theta - th1) / (O_PI - th1);
        wgt[0] *= (1.0 - wt);
        wgt[1] *= (1.0 - wt);
        double f = wt * 0.25;
        wgt[0] += f;
        wgt[1] += f;
        wgt[2] = f;
        wgt[3] = f;
        pix[2] = ((pix[0] + 2) & 3) + h->npix - 4;
        pix[3] = ((pix[1] + 2) & 3) + h->npix - 4;
    } else {
        double wt = (theta - th1) / (th2 - th1);
        wgt[0] *= (1.0 - wt);
        wgt[1] *= (1.0 - wt);
        wgt[2] *= wt;
        wgt[3] *= wt;
    }
}

void orc_pix2ang_many(int64_t nside, int64_t n, const int64_t* pix,
                      double* theta, double* phi)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) orc_pix2ang(&h, pix[i], &theta[i], &phi[i]);
}

void orc_ang2pix_many(int64_t nside, int64_t n, const double* theta,
                      const double* phi, int64_t* pix)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) pix[i] = orc_ang2pix(&h, theta[i], phi[i]);
}

void orc_get_interpol_many(int64_t nside, int64_t n, const double* theta,
                           const double* phi, int64_t* pix4, double* wgt4)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        orc_get_interpol(&h, theta[i], phi[i], &pix4[4 * i], &wgt4[4 * i]);
}

static int64_t o_max_ranges(int64_t nside) { return 8 * nside + 8; }

int64_t orc_query_disc_count(int64_t nside, double theta, double phi,
                             double radius)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    int64_t cap = o_max_ranges(nside);
    int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
    int64_t n = orc_query_disc(&h, theta, phi, radius, rg, cap);
    int64_t c = 0;
    for (int64_t r = 0; r < n; ++r) c += rg[2 * r + 1] - rg[2 * r];
    free(rg);
    return (n < 0) ? -1 : c;
}

int64_t orc_query_disc_pixels(int64_t nside, double theta, double phi,
                              double radius, int64_t* out, int64_t cap_out)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    int64_t cap = o_max_ranges(nside);
    int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
    int64_t n = orc_query_disc(&h, theta, phi, radius, rg, cap);
    int64_t c = 0;
    for (int64_t r = 0; r < n; ++r)
        for (int64_t p = rg[2 * r]; p < rg[2 * r + 1]; ++p) {
            if (c >= cap_out) {
                free(rg);
                return -1;
            }
            out[c++] = p;
        }
    free(rg);
    return (n < 0) ? -1 : c;
}

/* ------------------------------------------------------------------ */
/* Beam-frame rotation (src/Sphtrigo/sphtrigo.cpp:4-55)                */
/* ------------------------------------------------------------------ */
void orc_rho_sigma_chi_pix(double* rho, double* sigma, double* chi,
                           double ra_bc, double dec_bc, double psi_bc,
                           double ra_pix, double dec_pix)
{
    double cdc = cos(dec_bc), sdc = sin(dec_bc);
    double cdp = cos(dec_pix), sdp = sin(dec_pix);
    double dra = ra_pix - ra_bc;
    double sd = sin(dra), cd = cos(dra);
    double crho = sdc * sdp + cdc * cdp * cd;
    double al, be;
    *rho = (crho >= 1.0) ? 0.0 : acos(crho);
    if (*rho > 1.0e-6) {
        be = atan2(sd * cdc, sdc * cdp - cdc * sdp * cd);
        al = atan2(sd * cdp, sdp * cdc - cdp * sdc * cd);
    } else {
        be = O_HALFPI;
        al = O_HALFPI;
    }
    *sigma = O_PI - al - psi_bc;
    if (*sigma < 0.0) *sigma += 2.0 * O_PI;
    else if (*sigma > 2.0 * O_PI) *sigma -= 2.0 * O_PI;
    *chi = be - *sigma;
    if (*chi < -O_PI) *chi += 2.0 * O_PI;
}

void orc_rho_sigma_chi_many(int64_t n, const double* ra_bc,
                            const double* dec_bc, const double* psi_bc,
                            const double* ra_pix, const double* dec_pix,
                            double* rho, double* sigma, double* chi)
{
    for (int64_t i = 0; i < n; ++i)
        orc_rho_sigma_chi_pix(&rho[i], &sigma[i], &chi[i], ra_bc[i], dec_bc[i],
                              psi_bc[i], ra_pix[i], dec_pix[i]);
}

/* ------------------------------------------------------------------ */
/* PolBeam builders (src/Polbeam/polbeam.cpp)                          */
/* ------------------------------------------------------------------ */
int64_t orc_beam_npix_for_radius(int64_t nside, double radius_rad)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    return orc_ang2pix(&h, radius_rad, 0.0);
}

double orc_beam_rho_max(int64_t nside, int64_t npix)
{
    orc_hpx h;
    double th, ph;
    orc_hpx_init(&h, nside);
    orc_pix2ang(&h, npix, &th, &ph);
    return th;
}

void orc_gaussian_fields(int64_t nside, int64_t npix, double fwhmx,
                         double fwhmy, double phi0, double* magEco,
                         double* phsEco, double* magEcx, double* phsEcx)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    double d2r = O_PI / 180.0;
    double sx = (d2r * fwhmx) / 2.35482;
    double sy = (d2r * fwhmy) / 2.35482;
    double p0 = d2r * phi0;
    double a = (cos(p0) * cos(p0)) / (2 * sx * sx) + (sin(p0) * sin(p0)) / (2 * sy * sy);
    double b = -(sin(2 * p0)) / (4 * sx * sx) + (sin(2 * p0)) / (4 * sy * sy);
    double c = (sin(p0) * sin(p0)) / (2 * sx * sx) + (cos(p0) * cos(p0)) / (2 * sy * sy);
    for (int64_t i = 0; i < npix; ++i) {
        double rho, sig;
        orc_pix2ang(&h, i, &rho, &sig);
        double v = exp(-(a * cos(sig) * cos(sig) + 2.0 * b * cos(sig) * sin(sig) +
                         c * sin(sig) * sin(sig)) * rho * rho);
        magEco[i] = sqrt(v);
        magEcx[i] = 0.0;
        phsEco[i] = 0.0;
        phsEcx[i] = 0.0;
    }
}

void orc_beam_from_fields(int64_t npix, const double* mco, const double* pco,
                          const double* mcx, const double* pcx, float* I,
                          float* Q, float* U, float* V)
{
    for (int64_t i = 0; i < npix; ++i) {
        double ar = mco[i] * cos(pco[i]), ai = mco[i] * sin(pco[i]);
        double br = mcx[i] * cos(pcx[i]), bi = mcx[i] * sin(pcx[i]);
        double nco = ar * ar + ai * ai;
        double ncx = br * br + bi * bi;
        /* Eco * conj(Ecx) */
        double pr = ar * br - ai * (-bi);
        double pi_ = ar * (-bi) + ai * br;
        I[i] = (float)(nco + ncx);
        Q[i] = (float)(nco - ncx);
        U[i] = (float)(2 * pr);
        V[i] = (float)(-2 * pi_);
    }
}

void orc_beam_build(int64_t nside_beam, int64_t npix, double eps, char en,
                    int64_t nside_sky, const float* ta, const float* tb,
                    float* oa, float* ob)
{
    const float *Ia = ta, *Qa = ta + npix, *Ua = ta + 2 * npix, *Va = ta + 3 * npix;
    const float *Ib = tb, *Qb = tb + npix, *Ub = tb + 2 * npix, *Vb = tb + 3 * npix;
    double sa = 0.0, sb = 0.0;
    for (int64_t i = 0; i < npix; ++i) {
        if (en == 'a' || en == 'p') sa += Ia[i];
        if (en == 'b' || en == 'p') sb += Ib[i];
    }
    double oc = (double)nside_sky / (double)nside_beam;
    oc = oc * oc;
    double an = sa * oc, bn = sb * oc;
    if (en == 'a') bn += 1e-8;
    if (en == 'b') an += 1e-8;
    for (int64_t i = 0; i < npix; ++i) {
        oa[i] = (float)((Ia[i] + eps * Ib[i]) / an);
        oa[npix + i] = (float)((Qa[i] - eps * Qb[i]) / an);
        oa[2 * npix + i] = (float)((Ua[i] - eps * Ub[i]) / an);
        oa[3 * npix + i] = (float)((Va[i] + eps * Vb[i]) / an);
        ob[i] = (float)((Ib[i] + eps * Ia[i]) / bn);
        ob[npix + i] = (float)((Qb[i] - eps * Qa[i]) / bn);
        ob[2 * npix + i] = (float)((Ub[i] - eps * Ua[i]) / bn);
        ob[3 * npix + i] = (float)((Vb[i] + eps * Va[i]) / bn);
    }
}

/* ------------------------------------------------------------------ */
/* Convolution (src/Convolver/convolver.cpp:60-221)                    */
/* ------------------------------------------------------------------ */

/* Beam value lookup for one pair: nearest pixel or renormalised bilinear.
 * Returns 0 when the pair falls outside the stored beam. */
static int o_beam_lookup_d(const orc_hpx* hb, int64_t npb, const double* ba,
                           const double* bb, double rho, double sigma,
                           int interp, double va[4], double vb[4])
{
    if (!interp) {
        int64_t bp = orc_ang2pix(hb, rho, sigma);
        if (bp >= npb) return 0;
        for (int k = 0; k < 4; ++k) {
            va[k] = ba[k * npb + bp];
            vb[k] = bb[k * npb + bp];
        }
        return 1;
    }
    int64_t px[4];
    double w[4], ws = 0.0;
    orc_get_interpol(hb, rho, sigma, px, w);
    for (int k = 0; k < 4; ++k) va[k] = vb[k] = 0.0;
    for (int i = 0; i < 4; ++i) {
        if (px[i] >= npb) continue;
        ws += w[i];
        for (int k = 0; k < 4; ++k) {
            va[k] += ba[k * npb + px[i]] * w[i];
            vb[k] += bb[k * npb + px[i]] * w[i];
        }
    }
    if (!(ws > 0.0)) return 0;
    for (int k = 0; k < 4; ++k) {
        va[k] /= ws;
        vb[k] /= ws;
    }
    return 1;
}

static int o_beam_lookup_f(const orc_hpx* hb, int64_t npb, const float* ba,
                           const float* bb, double rho, double sigma,
                           int interp, float va[4], float vb[4])
{
    if (!interp) {
        int64_t bp = orc_ang2pix(hb, rho, sigma);
        if (bp >= npb) return 0;
        for (int k = 0; k < 4; ++k) {
            va[k] = ba[k * npb + bp];
            vb[k] = bb[k * npb + bp];
        }
        return 1;
    }
    int64_t px[4];
    double w[4], ws = 0.0, da[4] = {0, 0, 0, 0}, db[4] = {0, 0, 0, 0};
    orc_get_interpol(hb, rho, sigma, px, w);
    for (int i = 0; i < 4; ++i) {
        if (px[i] >= npb) continue;
        ws += w[i];
        for (int k = 0; k < 4; ++k) {
            da[k] += (double)ba[k * npb + px[i]] * w[i];
            db[k] += (double)bb[k * npb + px[i]] * w[i];
        }
    }
    if (!(ws > 0.0)) return 0;
    for (int k = 0; k < 4; ++k) {
        va[k] = (float)(da[k] / ws);
        vb[k] = (float)(db[k] / ws);
    }
    return 1;
}

typedef struct {
    orc_hpx hs, hb;
    double rhomax;
    int64_t npb;
    int interp;
} o_conv_setup;

static void o_setup(o_conv_setup* s, int64_t nsky, int64_t nbeam, int64_t npb,
                    int interp)
{
    orc_hpx_init(&s->hs, nsky);
    orc_hpx_init(&s->hb, nbeam);
    s->npb = npb;
    s->rhomax = orc_beam_rho_max(nbeam, npb);
    s->interp = interp;
}

void orc_convolve_f32(int64_t ns, const float* ra, const float* dec,
                      const float* pa, int64_t nside_sky, const float* sky,
                      int64_t nside_beam, int64_t npb, const float* ba,
                      const float* bb, int interp, char pf, float* oa,
                      float* ob, int nthreads)
{
    o_conv_setup S;
    o_setup(&S, nside_sky, nside_beam, npb, interp);
    const int64_t np = S.hs.npix;
    const float *sI = sky, *sQ = sky + np, *sU = sky + 2 * np, *sV = sky + 3 * np;
    const int64_t cap = o_max_ranges(nside_sky);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < ns; ++i) {
            /* convolver.cpp:85-90: float ra, double dec, psi = -pa */
            float ra_f = ra[i];
            double rab = ra_f, decb = dec[i], pab = -pa[i];
            double acc_a = 0.0, acc_b = 0.0;
            int64_t nr = orc_query_disc(&S.hs, O_HALFPI - decb, rab, S.rhomax, rg, cap);
            for (int64_t r = 0; r < nr; ++r)
                for (int64_t p = rg[2 * r]; p < rg[2 * r + 1]; ++p) {
                    double th, ph, rho, sig, chi;
                    orc_pix2ang(&S.hs, p, &th, &ph);
                    orc_rho_sigma_chi_pix(&rho, &sig, &chi, rab, decb, pab, ph,
                                          O_PI / 2.0 - th);
                    float c2 = (float)cos(2.0 * chi), s2 = (float)sin(2.0 * chi);
                    float va[4], vb[4];
                    if (!o_beam_lookup_f(&S.hb, npb, ba, bb, rho, sig, interp, va, vb))
                        continue;
                    float I = sI[p], Q = sQ[p], U = sU[p], V = sV[p];
                    float ta = I * va[0] + Q * (va[1] * c2 - va[2] * s2) +
                               U * (va[2] * c2 + va[1] * s2) + V * va[3];
                    float tb = I * vb[0] + Q * (-vb[1] * c2 + vb[2] * s2) +
                               U * (-vb[2] * c2 - vb[1] * s2) + V * vb[3];
                    acc_a += ta;
                    acc_b += tb;
                }
            if (pf == 'a' || pf == 'p') oa[i] = (float)acc_a;
            if (pf == 'b' || pf == 'p') ob[i] = (float)acc_b;
        }
        free(rg);
    }
}

void orc_convolve_f64(int64_t ns, const double* ra, const double* dec,
                      const double* pa, int64_t nside_sky, const double* sky,
                      int64_t nside_beam, int64_t npb, const double* ba,
                      const double* bb, int interp, char pf, double* oa,
                      double* ob, int nthreads)
{
    o_conv_setup S;
    o_setup(&S, nside_sky, nside_beam, npb, interp);
    const int64_t np = S.hs.npix;
    const double *sI = sky, *sQ = sky + np, *sU = sky + 2 * np, *sV = sky + 3 * np;
    const int64_t cap = o_max_ranges(nside_sky);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < ns; ++i) {
            double rab = ra[i], decb = dec[i], pab = -pa[i];
            double acc_a = 0.0, acc_b = 0.0;
            int64_t nr = orc_query_disc(&S.hs, O_HALFPI - decb, rab, S.rhomax, rg, cap);
            for (int64_t r = 0; r < nr; ++r)
                for (int64_t p = rg[2 * r]; p < rg[2 * r + 1]; ++p) {
                    double th, ph, rho, sig, chi;
                    orc_pix2ang(&S.hs, p, &th, &ph);
                    orc_rho_sigma_chi_pix(&rho, &sig, &chi, rab, decb, pab, ph,
                                          O_PI / 2.0 - th);
                    double c2 = cos(2.0 * chi), s2 = sin(2.0 * chi);
                    double va[4], vb[4];
                    if (!o_beam_lookup_d(&S.hb, npb, ba, bb, rho, sig, interp, va, vb))
                        continue;
                    double I = sI[p], Q = sQ[p], U = sU[p], V = sV[p];
                    acc_a += I * va[0] + Q * (va[1] * c2 - va[2] * s2) +
                             U * (va[2] * c2 + va[1] * s2) + V * va[3];
                    acc_b += I * vb[0] + Q * (-vb[1] * c2 + vb[2] * s2) +
                             U * (-vb[2] * c2 - vb[1] * s2) + V * vb[3];
                }
            if (pf == 'a' || pf == 'p') oa[i] = acc_a;
            if (pf == 'b' || pf == 'p') ob[i] = acc_b;
        }
        free(rg);
    }
}

void orc_match_pairs(int64_t npairs, const double* ra, const double* dec,
                     const double* pa, const int64_t* skypix, int64_t nside_sky,
                     int64_t nside_beam, int64_t* beampix, double* chi)
{
    orc_hpx hs, hb;
    orc_hpx_init(&hs, nside_sky);
    orc_hpx_init(&hb, nside_beam);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < npairs; ++i) {
        double th, ph, rho, sig;
        orc_pix2ang(&hs, skypix[i], &th, &ph);
        orc_rho_sigma_chi_pix(&rho, &sig, &chi[i], ra[i], dec[i], -pa[i], ph,
                              O_PI / 2.0 - th);
        beampix[i] = orc_ang2pix(&hb, rho, sig);
    }
}

void orc_adjoint_f64(int64_t ns, const double* ra, const double* dec,
                     const double* pa, int64_t nside_sky, int64_t nside_beam,
                     int64_t npb, const double* ba, const double* bb,
                     const double* ga, const double* gb, double* g)
{
    o_conv_setup S;
    o_setup(&S, nside_sky, nside_beam, npb, 0);
    const int64_t np = S.hs.npix;
    const int64_t cap = o_max_ranges(nside_sky);
    int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
    for (int64_t i = 0; i < ns; ++i) {
        double rab = ra[i], decb = dec[i], pab = -pa[i];
        int64_t nr = orc_query_disc(&S.hs, O_HALFPI - decb, rab, S.rhomax, rg, cap);
        for (int64_t r = 0; r < nr; ++r)
            for (int64_t p = rg[2 * r]; p < rg[2 * r + 1]; ++p) {
                double th, ph, rho, sig, chi, va[4], vb[4];
                orc_pix2ang(&S.hs, p, &th, &ph);
                orc_rho_sigma_chi_pix(&rho, &sig, &chi, rab, decb, pab, ph,
                                      O_PI / 2.0 - th);
                if (!o_beam_lookup_d(&S.hb, npb, ba, bb, rho, sig, 0, va, vb)) continue;
                double c2 = cos(2.0 * chi), s2 = sin(2.0 * chi);
                g[p] += ga[i] * va[0] + gb[i] * vb[0];
                g[np + p] += ga[i] * (va[1] * c2 - va[2] * s2) + gb[i] * (-vb[1] * c2 + vb[2] * s2);
                g[2 * np + p] += ga[i] * (va[2] * c2 + va[1] * s2) + gb[i] * (-vb[2] * c2 - vb[1] * s2);
                g[3 * np + p] += ga[i] * va[3] + gb[i] * vb[3];
            }
    }
    free(rg);
}

/* ---------------- binned map-making (skymap.cpp:68-231) ---------------- */

/* One TOD value into the normal equations of its pixel (skymap.cpp:99-122). */
static void o_map_add(double* ata, double* atd, int64_t p, double pol, double pa, double d)
{
    const double psi = -(pol + pa);
    const double twopsi = 2.0 * psi;
    const double c = cos(twopsi), s = sin(twopsi);
    double* D = atd + 3 * p;
    double* A = ata + 9 * p;
    D[0] += 1.0 * d;
    D[1] += c * d;
    D[2] += s * d;
    A[0] += 1.0;
    A[1] += c;
    A[2] += s;
    A[3] += c;
    A[4] += c * c;
    A[5] += c * s;
    A[6] += s;
    A[7] += c * s;
    A[8] += s * s;
}

void orc_map_accumulate_f32(int64_t nside, int64_t ns, const float* ra, const float* dec,
                            const float* pa, int ndet, const float* pol, const float* data,
                            double* ata, double* atd)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    for (int d = 0; d < ndet; ++d)
        for (int64_t i = 0; i < ns; ++i) {
            const int64_t k = (int64_t)d * ns + i;
            const int64_t p = orc_ang2pix(&h, O_HALFPI - (double)dec[k], (double)ra[k]);
            o_map_add(ata, atd, p, (double)pol[d], (double)pa[k], (double)data[k]);
        }
}

void orc_map_accumulate_f64(int64_t nside, int64_t ns, const double* ra, const double* dec,
                            const double* pa, int ndet, const float* pol, const double* data,
                            double* ata, double* atd)
{
    orc_hpx h;
    orc_hpx_init(&h, nside);
    for (int d = 0; d < ndet; ++d)
        for (int64_t i = 0; i < ns; ++i) {
            const int64_t k = (int64_t)d * ns + i;
            const int64_t p = orc_ang2pix(&h, O_HALFPI - dec[k], ra[k]);
            o_map_add(ata, atd, p, (double)pol[d], pa[k], data[k]);
        }
}

/* Column-major element (r, c) of a 3 x 3 matrix, 0-based. */
#define O_A(r, c) a[(c) * 3 + (r)]

int orc_dgesv3(double* a, int* ipiv, double* b)
{
    const double sfmin = 2.2250738585072014e-308; /* safe minimum: 1/sfmin does not overflow */
    int info = 0;
    /* dgetf2 */
    for (int j = 0; j < 3; ++j) {
        int jp = j;
        double amax = fabs(O_A(j, j));
        for (int i = j + 1; i < 3; ++i)
            if (fabs(O_A(i, j)) > amax) {
                amax = fabs(O_A(i, j));
                jp = i;
            }
        ipiv[j] = jp + 1;
        if (O_A(jp, j) != 0.0) {
            if (jp != j)
                for (int c = 0; c < 3; ++c) {
                    const double t = O_A(j, c);
                    O_A(j, c) = O_A(jp, c);
                    O_A(jp, c) = t;
                }
            if (fabs(O_A(j, j)) >= sfmin) {
                const double r = 1.0 / O_A(j, j);
                for (int i = j + 1; i < 3; ++i) O_A(i, j) *= r;
            } else {
                for (int i = j + 1; i < 3; ++i) O_A(i, j) /= O_A(j, j);
            }
        } else if (info == 0) {
            info = j + 1;
        }
        /* rank-1 update of the trailing block: a(i, c) += a(i, j) * (-a(j, c)) */
        for (int c = j + 1; c < 3; ++c) {
            if (O_A(j, c) != 0.0) {
                const double t = -O_A(j, c);
                for (int i = j + 1; i < 3; ++i) O_A(i, c) += O_A(i, j) * t;
            }
        }
    }
    if (info != 0) return info;
    /* dgetrs: interchanges, then L y = P b (unit lower), then U x = y */
    for (int i = 0; i < 3; ++i) {
        const int ip = ipiv[i] - 1;
        if (ip != i) {
            const double t = b[i];
            b[i] = b[ip];
            b[ip] = t;
        }
    }
    for (int k = 0; k < 3; ++k)
        if (b[k] != 0.0)
            for (int i = k + 1; i < 3; ++i) b[i] -= b[k] * O_A(i, k);
    for (int k = 2; k >= 0; --k)
        if (b[k] != 0.0) {
            b[k] /= O_A(k, k);
            for (int i = 0; i < k; ++i) b[i] -= b[k] * O_A(i, k);
        }
    return 0;
}
#undef O_A

void orc_map_solve(int64_t npix, const double* ata, const double* atd, float* I, float* Q,
                   float* U, int* hits)
{
    for (int64_t p = 0; p < npix; ++p) {
        double a[9], b[3];
        int ipiv[3];
        /* column-major assembly as skymap.cpp:158-170 (AtA is symmetric) */
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) a[c * 3 + r] = ata[9 * p + 3 * r + c];
        for (int k = 0; k < 3; ++k) b[k] = atd[3 * p + k];
        double ii = 0.0, qq = 0.0, uu = 0.0;
        int h = (int)ata[9 * p];
        if (h >= 3) {
            const int info = orc_dgesv3(a, ipiv, b);
            ii = b[0];
            qq = b[1];
            uu = b[2];
            if (info != 0) h = 0;
        }
        I[p] = (float)ii;
        Q[p] = (float)qq;
        U[p] = (float)uu;
        hits[p] = h;
    }
}

/* ------------------------------------------------------------------ */
/* Focal plane to sky (src/Bpoint/bpoint.cpp:553-674)                   */
/* ------------------------------------------------------------------ */
/* Restates BPoint::focal_plane_to_sky, the spherical triangle between the
 * array centre, the detector and the pole (zenith, celestial pole or
 * source): the detector sits at angular distance r = acos(cos dx cos dy)
 * from the array centre, in the receiver-frame direction a = atan2(sin dy,
 * sin dx cos dy) from the receiver x axis; g = pi/2 - a - rot is the angle
 * detector -> array centre -> pole.  Outputs [det * nsamples + s]. */
void orc_focal_plane_to_sky(int ndets, const double* det_dx, const double* det_dy,
                            const double* det_pol, int64_t nsamples, const double* x_ac,
                            const double* y_ac, const double* rot_ac, int flag,
                            double* x_det, double* y_det, double* rot_det)
{
    for (int d = 0; d < ndets; ++d) {
        const double cx = cos(det_dx[d]), sx = sin(det_dx[d]);
        const double cy_r = cos(det_dy[d]), sy_r = sin(det_dy[d]);
        const double cr = cx * cy_r;                      /* cos r */
        const double sr = sqrt((1.0 - cr) * (1.0 + cr));  /* sin r */
        const double a = atan2(sy_r, sx * cy_r);
        for (int64_t s = 0; s < nsamples; ++s) {
            const int64_t k = (int64_t)d * nsamples + s;
            const double g = O_HALFPI - a - rot_ac[s];
            const double cg = cos(g), sg = sin(g);
            const double sl = sin(y_ac[s]), cl = cos(y_ac[s]);
            const double se = sin(rot_ac[s]), ce = cos(rot_ac[s]);
            /* latitude of the detector: law of cosines in the triangle */
            y_det[k] = asin(cr * sl + sr * cl * cg);
            /* position angle at the detector of the receiver-frame pole */
            const double num = cl * se * cx - sl * sx;
            const double den = cl * ce * cy_r - (sl * cx + cl * se * sx) * sy_r;
            const double pa = atan2(num, den);
            rot_det[k] = pa + det_pol[d];
            if (flag == 2) {
                x_det[k] = -pa;
            } else {
                /* longitude step from the array centre to the detector */
                const double dl = atan2(sr * sg, cr * cl - sr * sl * cg);
                x_det[k] = flag == 0 ? x_ac[s] + dl : x_ac[s] - dl;
            }
        }
    }
}
