/*
 * ref_harness.cpp -- C entry points around the reference's own CPU sources
 * (TEST INFRASTRUCTURE ONLY; built by oracle/build_ref.sh into oracle/_ref/).
 *
 * The reference classes Sky, Scan, PolBeam and Convolver
 * (src/Sky/sky.cpp, src/Scan/scan.cpp, src/Polbeam/polbeam.cpp,
 * src/Convolver/convolver.cpp) and SphericalTransformations
 * (src/Sphtrigo/sphtrigo.cpp) are compiled unmodified from the reference
 * tree; this file only adapts plain arrays to their constructors.
 */
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "Convolver/convolver.hpp"
#include "Polbeam/polbeam.hpp"
#include "Scan/scan.hpp"
#include "Sky/sky.hpp"
#include "Sphtrigo/sphtrigo.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

/* PolBeam(nside, npix, eps, dets).make_unpol_gaussian_elliptical_beams(...)
 * then build(nside_sky); copies aBeams/bBeams out as 4 planes each. */
int ref_polbeam_gaussian(int nside, long npix, double eps, char dets,
                         double fwhmx, double fwhmy, double phi0,
                         int nside_sky, float* out_a, float* out_b,
                         double* rho_max)
{
    PolBeam b(nside, npix, eps, dets);
    b.make_unpol_gaussian_elliptical_beams(fwhmx, fwhmy, phi0);
    b.build(nside_sky);
    for (int k = 0; k < 4; ++k) {
        std::memcpy(out_a + k * npix, b.aBeams[k], sizeof(float) * npix);
        std::memcpy(out_b + k * npix, b.bBeams[k], sizeof(float) * npix);
    }
    *rho_max = b.get_rho_max();
    return 0;
}

/* Convolver(scan, sky, beam).exec_convolution(polflag, a, b) with the
 * beam planes supplied by the caller (copied into PolBeam::aBeams/bBeams). */
int ref_convolve(long ns, float* ra, float* dec, float* pa, int nside_sky,
                 const float* I, const float* Q, const float* U,
                 const float* V, int nside_beam, long npix_beam,
                 const float* beam_a, const float* beam_b, char polflag,
                 float* out_a, float* out_b, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    Scan scan(ns, ra, dec, pa);
    Sky sky(nside_sky, I, Q, U, V);
    PolBeam beam(nside_beam, npix_beam, 0.0, 'p');
    for (int k = 0; k < 4; ++k) {
        std::memcpy(beam.aBeams[k], beam_a + k * npix_beam, sizeof(float) * npix_beam);
        std::memcpy(beam.bBeams[k], beam_b + k * npix_beam, sizeof(float) * npix_beam);
    }
    Convolver conv(&scan, &sky, &beam);
    try {
        conv.exec_convolution(polflag, out_a, out_b);
    } catch (const std::invalid_argument&) {
        return 1;
    }
    return 0;
}

void ref_rho_sigma_chi(long n, const double* ra_bc, const double* dec_bc,
                       const double* psi_bc, const double* ra_pix,
                       const double* dec_pix, double* rho, double* sigma,
                       double* chi)
{
    for (long i = 0; i < n; ++i)
        SphericalTransformations::rho_sigma_chi_pix(&rho[i], &sigma[i], &chi[i],
                                                    ra_bc[i], dec_bc[i], psi_bc[i],
                                                    ra_pix[i], dec_pix[i]);
}
}
