// beam_model.h -- coefficients of the elliptical Gaussian detector-pair beam
// model shared by the host and device beam code: the beam (both detectors
// alike) is B[p] = c g[p] / N, c = (1 + eps, 1 - eps, 0, 0) per detector,
// g = exp(-(ca x^2 + 2 cb x y + cc y^2)), x = rho cos sigma - dx,
// y = rho sin sigma - dy at the beam pixel centres, N = (nside_sky /
// nside_beam)^2 sum_p g[p] (the PolBeam build normalisation,
// polbeam.cpp:204-268), with ca, cb, cc of PolBeam's elliptical Gaussian
// (polbeam.cpp:290-340) for sigma_x,y = fwhm_x,y / 2.35482, fwhm_x =
// F sqrt((1+e)/(1-e)), fwhm_y = F sqrt((1-e)/(1+e)), rotated by phi0.
#pragma once

#include <cmath>

namespace pisco {

struct GaussModel {
    double ca, cb, cc;           // quadratic form
    double aF, bF, cF;           // its derivatives with respect to F (deg)
    double ae, be, ce;           // ... with respect to e
    double ap, bp, cp;           // ... with respect to phi0 (deg)
};

// Host-side coefficients; fwhm_deg > 0 and |e| < 1 are the caller's checks.
inline GaussModel gauss_model(double fwhm_deg, double e, double phi0_deg)
{
    const double pi = 3.14159265358979323846;
    const double d2r = pi / 180.0;
    const double fx = fwhm_deg * std::sqrt((1.0 + e) / (1.0 - e));
    const double fy = fwhm_deg * std::sqrt((1.0 - e) / (1.0 + e));
    const double sx = d2r * fx / 2.35482, sy = d2r * fy / 2.35482;
    const double ph = d2r * phi0_deg;
    const double c = std::cos(ph), s = std::sin(ph), s2 = std::sin(2.0 * ph), c2 = std::cos(2.0 * ph);
    const double ux = 1.0 / (2.0 * sx * sx), uy = 1.0 / (2.0 * sy * sy);
    GaussModel m;
    m.ca = c * c * ux + s * s * uy;
    m.cb = 0.5 * s2 * (uy - ux);
    m.cc = s * s * ux + c * c * uy;
    // (ux, uy) scale as 1/F^2; with e, ux ~ (1-e)/(1+e) and uy ~ (1+e)/(1-e)
    const double dux_dF = -2.0 * ux / fwhm_deg, duy_dF = -2.0 * uy / fwhm_deg;
    const double dux_de = -2.0 * ux / (1.0 - e * e), duy_de = 2.0 * uy / (1.0 - e * e);
    m.aF = c * c * dux_dF + s * s * duy_dF;
    m.bF = 0.5 * s2 * (duy_dF - dux_dF);
    m.cF = s * s * dux_dF + c * c * duy_dF;
    m.ae = c * c * dux_de + s * s * duy_de;
    m.be = 0.5 * s2 * (duy_de - dux_de);
    m.ce = s * s * dux_de + c * c * duy_de;
    m.ap = d2r * s2 * (uy - ux);
    m.bp = d2r * c2 * (uy - ux);
    m.cp = d2r * s2 * (ux - uy);
    return m;
}

}  // namespace pisco
