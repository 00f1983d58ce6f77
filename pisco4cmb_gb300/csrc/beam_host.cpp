// beam_host.cpp -- host HEALPix queries and the PolBeam construction steps
// exported through the C ABI (include/pisco_gb300.h), so that the C++
// PolBeam wrapper (include/pisco/polbeam.hpp) builds beams exactly as the
// reference PolBeam does (src/Polbeam/polbeam.cpp:108-467).
// Compiled with -ffp-contract=off: the same rounding as the device code.
#include <cmath>
#include <complex>

#include "../../include/pisco_gb300.h"
#include "beam_model.h"
#include "hpx.cuh"

using namespace pisco;

extern "C" {

pisco_status pisco_hpx_pix2ang(int nside, long n, const long* pix, double* theta, double* phi)
{
    if (nside < 1 || nside > 8192 || n < 0 || (n && (!pix || !theta || !phi)))
        return PISCO_ERR_INVALID_ARGUMENT;
    const Hpx h = hpx_make(nside);
    for (long i = 0; i < n; ++i) {
        if (pix[i] < 0 || pix[i] >= h.npix) return PISCO_ERR_INVALID_ARGUMENT;
        pix2ang(h, pix[i], &theta[i], &phi[i]);
    }
    return PISCO_OK;
}

pisco_status pisco_hpx_ang2pix(int nside, long n, const double* theta, const double* phi, long* pix)
{
    if (nside < 1 || nside > 8192 || n < 0 || (n && (!pix || !theta || !phi)))
        return PISCO_ERR_INVALID_ARGUMENT;
    const Hpx h = hpx_make(nside);
    for (long i = 0; i < n; ++i) {
        if (!(theta[i] >= 0.0 && theta[i] <= kPi)) return PISCO_ERR_INVALID_ARGUMENT;
        pix[i] = (long)ang2pix(h, theta[i], phi[i]);
    }
    return PISCO_OK;
}

long pisco_beam_npix_for_radius(int nside, double radius_rad)
{
    if (nside < 1 || nside > 8192 || !(radius_rad >= 0.0 && radius_rad <= kPi)) return -1;
    return (long)ang2pix(hpx_make(nside), radius_rad, 0.0);
}

double pisco_beam_rho_max(int nside, long npix)
{
    if (nside < 1 || nside > 8192 || npix < 0 || npix >= 12L * nside * nside) return -1.0;
    double th, ph;
    pix2ang(hpx_make(nside), npix, &th, &ph);
    return th;
}

pisco_status pisco_beam_gaussian_fields(int nside, long npix, double fwhmx, double fwhmy,
                                        double phi0, double* magEco, double* phsEco,
                                        double* magEcx, double* phsEcx)
{
    if (nside < 1 || nside > 8192 || npix < 0 || npix >= 12L * nside * nside ||
        (npix && (!magEco || !phsEco || !magEcx || !phsEcx)) || !(fwhmx > 0.0) || !(fwhmy > 0.0))
        return PISCO_ERR_INVALID_ARGUMENT;
    const Hpx h = hpx_make(nside);
    // FWHM (deg) -> Gaussian sigma (rad) and rotated-ellipse coefficients
    const double d2r = kPi / 180.0;
    const double sx = (d2r * fwhmx) / 2.35482;
    const double sy = (d2r * fwhmy) / 2.35482;
    const double p0 = d2r * phi0;
    const double ca = (cos(p0) * cos(p0)) / (2 * sx * sx) + (sin(p0) * sin(p0)) / (2 * sy * sy);
    const double cb = -(sin(2 * p0)) / (4 * sx * sx) + (sin(2 * p0)) / (4 * sy * sy);
    const double cc = (sin(p0) * sin(p0)) / (2 * sx * sx) + (cos(p0) * cos(p0)) / (2 * sy * sy);
    for (long i = 0; i < npix; ++i) {
        double rho, sig;
        pix2ang(h, i, &rho, &sig);
        const double cs = cos(sig), sn = sin(sig);
        const double v = exp(-(ca * cs * cs + 2.0 * cb * cs * sn + cc * sn * sn) * rho * rho);
        magEco[i] = sqrt(v);
        magEcx[i] = 0.0;
        phsEco[i] = 0.0;
        phsEcx[i] = 0.0;
    }
    return PISCO_OK;
}

pisco_status pisco_beam_from_fields(long npix, const double* mco, const double* pco,
                                    const double* mcx, const double* pcx, float* I, float* Q,
                                    float* U, float* V)
{
    if (npix < 0 || (npix && (!mco || !pco || !mcx || !pcx || !I || !Q || !U || !V)))
        return PISCO_ERR_INVALID_ARGUMENT;
    for (long i = 0; i < npix; ++i) {
        // Rosset et al. 2010 tilde Stokes beams from co/cross-polar fields
        const std::complex<double> eco = std::polar(mco[i], pco[i]);
        const std::complex<double> ecx = std::polar(mcx[i], pcx[i]);
        const std::complex<double> x = eco * std::conj(ecx);
        I[i] = (float)(std::norm(eco) + std::norm(ecx));
        Q[i] = (float)(std::norm(eco) - std::norm(ecx));
        U[i] = (float)(2 * x.real());
        V[i] = (float)(-2 * x.imag());
    }
    return PISCO_OK;
}

pisco_status pisco_beam_build(int nside_beam, long npix, double eps, char en, int nside_sky,
                              const float* const ta[4], const float* const tb[4],
                              float* const oa[4], float* const ob[4])
{
    if (nside_beam < 1 || nside_sky < 1 || npix < 0 || !ta || !tb || !oa || !ob ||
        (en != 'a' && en != 'b' && en != 'p'))
        return PISCO_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 4; ++k)
        if (npix && (!ta[k] || !tb[k] || !oa[k] || !ob[k])) return PISCO_ERR_INVALID_ARGUMENT;
    double sa = 0.0, sb = 0.0;
    for (long i = 0; i < npix; ++i) {
        if (en == 'a' || en == 'p') sa += ta[0][i];
        if (en == 'b' || en == 'p') sb += tb[0][i];
    }
    double oc = (double)nside_sky / (double)nside_beam;
    oc = oc * oc;
    double an = sa * oc, bn = sb * oc;
    if (en == 'a') bn += 1e-8;  // same guard as the reference against an unused detector
    if (en == 'b') an += 1e-8;
    for (long i = 0; i < npix; ++i) {
        oa[0][i] = (float)((ta[0][i] + eps * tb[0][i]) / an);
        oa[1][i] = (float)((ta[1][i] - eps * tb[1][i]) / an);
        oa[2][i] = (float)((ta[2][i] - eps * tb[2][i]) / an);
        oa[3][i] = (float)((ta[3][i] + eps * tb[3][i]) / an);
        ob[0][i] = (float)((tb[0][i] + eps * ta[0][i]) / bn);
        ob[1][i] = (float)((tb[1][i] - eps * ta[1][i]) / bn);
        ob[2][i] = (float)((tb[2][i] - eps * ta[2][i]) / bn);
        ob[3][i] = (float)((tb[3][i] + eps * ta[3][i]) / bn);
    }
    return PISCO_OK;
}

// Gradient of a loss with respect to the parameters of the elliptical Gaussian
// detector-pair beam model (beam_model.h), from its gradient with respect to
// the beam maps.  The beam weights are recomputed here (not stored); the
// derivative is analytic:
//   dL/dt = (1/N) [sum_p G_p dg_p/dt - (sum_p G_p g_p) (sum_p dg_p/dt) / sum_p g_p],
//   G_p = sum_k c_k dL/dB[p][k],  dg/dt = -g dQ/dt.
pisco_status pisco_beam_gaussian_param_grad(int nside_beam, long npix, double eps, int nside_sky,
                                            double fwhm_deg, double ellipticity, double phi0_deg,
                                            double dx, double dy, const double* gbeam,
                                            double grad[5])
{
    if (nside_beam < 1 || nside_beam > 8192 || nside_sky < 1 || npix < 1 || !gbeam || !grad ||
        !(fwhm_deg > 0.0) || !(std::fabs(ellipticity) < 1.0))
        return PISCO_ERR_INVALID_ARGUMENT;
    if (npix > 12L * nside_beam * nside_beam) return PISCO_ERR_INVALID_ARGUMENT;
    const Hpx h = hpx_make(nside_beam);
    const GaussModel m = gauss_model(fwhm_deg, ellipticity, phi0_deg);
    const double ca = m.ca, cb = m.cb, cc = m.cc;
    const double aF = m.aF, bF = m.bF, cF = m.cF, ae = m.ae, be = m.be, ce = m.ce;
    const double ap = m.ap, bp = m.bp, cp = m.cp;
    const double cw[8] = {1.0 + eps, 1.0 - eps, 0.0, 0.0, 1.0 + eps, 1.0 - eps, 0.0, 0.0};
    double sg = 0.0, sGg = 0.0, sdg[5] = {0, 0, 0, 0, 0}, sGdg[5] = {0, 0, 0, 0, 0};
    for (long p = 0; p < npix; ++p) {
        double th, phi;
        pix2ang(h, p, &th, &phi);
        const double x = th * std::cos(phi) - dx, y = th * std::sin(phi) - dy;
        const double g = std::exp(-(ca * x * x + 2.0 * cb * x * y + cc * y * y));
        double G = 0.0;
        for (int k = 0; k < 8; ++k) G += cw[k] * gbeam[8 * p + k];
        // dQ/dt for t = F, e, phi0, dx, dy
        const double dQ[5] = {x * x * aF + 2.0 * x * y * bF + y * y * cF,
                              x * x * ae + 2.0 * x * y * be + y * y * ce,
                              x * x * ap + 2.0 * x * y * bp + y * y * cp,
                              -2.0 * (ca * x + cb * y), -2.0 * (cb * x + cc * y)};
        sg += g;
        sGg += G * g;
        for (int t = 0; t < 5; ++t) {
            const double dg = -g * dQ[t];
            sdg[t] += dg;
            sGdg[t] += G * dg;
        }
    }
    double oc = (double)nside_sky / (double)nside_beam;
    oc = oc * oc;
    const double N = oc * sg;
    if (!(N > 0.0)) return PISCO_ERR_INVALID_ARGUMENT;
    for (int t = 0; t < 5; ++t) grad[t] = (sGdg[t] - sGg * sdg[t] / sg) / N;
    return PISCO_OK;
}

}  // extern "C"
