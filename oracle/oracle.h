/*
 * oracle.h -- CPU oracle for the pixel-space polarized-beam convolution.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the pisco4cmb_gb300
 * package, its CUDA kernels or its C-ABI library) may link, load or call
 * this code.  Only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py use it, and only as the checker.
 *
 * Contents (all plain C99, compiled with -ffp-contract=off so that results
 * are identical on x86-64 and aarch64):
 *   - HEALPix RING geometry restated from the published HEALPix algorithms
 *     (Gorski et al. 2005, ApJ 622:759; HEALPix C++ 3.x Healpix_Base):
 *     ring geometry, pix2ang, ang2pix, query_disc (non-inclusive),
 *     get_interpol.  The reference calls these from the absent Healpix C++
 *     library at src/Convolver/convolver.cpp:137-138,150,187,
 *     src/Polbeam/polbeam.cpp:130,441 and ports three of them to the GPU
 *     in src/GpuConvolver/cuda/cudaHealpix.cu:45-259.
 *   - rho_sigma_chi_pix restated from src/Sphtrigo/sphtrigo.cpp:4-55.
 *   - beam_times_sky / exec_convolution restated from
 *     src/Convolver/convolver.cpp:60-221 (float sky and beams, float
 *     per-pair products, double accumulation) plus an all-double form and
 *     a bilinear-beam option (the commented-out block at
 *     convolver.cpp:162-185, with the weight renormalisation it intends).
 *   - the PolBeam builders restated from src/Polbeam/polbeam.cpp:108-133,
 *     212-279, 281-383, 385-467.
 *   - BPoint::focal_plane_to_sky restated from src/Bpoint/bpoint.cpp:553-674
 *     (spherical trigonometry only; the ephemeris part of BPoint needs SOFA
 *     and JPL data, absent from the reference tree).
 *
 * Parity pins: see tests/test_oracle_*.py.  The HEALPix part is pinned
 * against the reference's own device port (cudaHealpix.cu compiled for the
 * host) and against the brute-force definition of query_disc; the
 * convolution part against the reference Convolver sources compiled
 * against a HEALPix shim built on this file (oracle/build_ref.sh).
 */
#ifndef PISCO_ORACLE_H
#define PISCO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- HEALPix RING geometry ---------------- */
typedef struct {
    int64_t nside;
    int64_t npix;
    int64_t ncap;
    double fact1;
    double fact2;
} orc_hpx;

void orc_hpx_init(orc_hpx* h, int64_t nside);
int64_t orc_ring_above(const orc_hpx* h, double z);
double orc_ring2z(const orc_hpx* h, int64_t ring);
void orc_ring_info_small(const orc_hpx* h, int64_t ring, int64_t* startpix,
                         int64_t* ringpix, int* shifted);
void orc_ring_info2(const orc_hpx* h, int64_t ring, int64_t* startpix,
                    int64_t* ringpix, double* theta, int* shifted);
void orc_pix2ang(const orc_hpx* h, int64_t pix, double* theta, double* phi);
int64_t orc_ang2pix(const orc_hpx* h, double theta, double phi);
/* Pixel ranges [begin, end) whose centres lie inside the disc, ascending.
 * Returns the number of ranges written (<= max_ranges), or -1 if the
 * output array is too small. */
int64_t orc_query_disc(const orc_hpx* h, double theta, double phi,
                       double radius, int64_t* ranges, int64_t max_ranges);
void orc_get_interpol(const orc_hpx* h, double theta, double phi,
                      int64_t pix[4], double wgt[4]);

/* Batched wrappers used from Python (ctypes). */
void orc_pix2ang_many(int64_t nside, int64_t n, const int64_t* pix,
                      double* theta, double* phi);
void orc_ang2pix_many(int64_t nside, int64_t n, const double* theta,
                      const double* phi, int64_t* pix);
void orc_get_interpol_many(int64_t nside, int64_t n, const double* theta,
                           const double* phi, int64_t* pix4, double* wgt4);
/* Counts, then fills, the flattened disc pixel list for each pointing. */
int64_t orc_query_disc_count(int64_t nside, double theta, double phi,
                             double radius);
int64_t orc_query_disc_pixels(int64_t nside, double theta, double phi,
                              double radius, int64_t* out, int64_t cap);

/* ---------------- beam-frame rotation ---------------- */
void orc_rho_sigma_chi_pix(double* rho, double* sigma, double* chi,
                           double ra_bc, double dec_bc, double psi_bc,
                           double ra_pix, double dec_pix);

void orc_rho_sigma_chi_many(int64_t n, const double* ra_bc,
                            const double* dec_bc, const double* psi_bc,
                            const double* ra_pix, const double* dec_pix,
                            double* rho, double* sigma, double* chi);

/* ---------------- PolBeam builders ---------------- */
/* nPixels convention of the beam maps: ang2pix(nside, radius, 0). */
int64_t orc_beam_npix_for_radius(int64_t nside, double radius_rad);
double orc_beam_rho_max(int64_t nside, int64_t npix);
/* Elliptical Gaussian co-polar field magnitude (polbeam.cpp:385-467). */
void orc_gaussian_fields(int64_t nside, int64_t npix, double fwhmx_deg,
                         double fwhmy_deg, double phi0_deg, double* magEco,
                         double* phsEco, double* magEcx, double* phsEcx);
/* Tilde Stokes beams from fields (polbeam.cpp:212-279). Outputs float. */
void orc_beam_from_fields(int64_t npix, const double* magEco,
                          const double* phsEco, const double* magEcx,
                          const double* phsEcx, float* I, float* Q,
                          float* U, float* V);
/* Polarized beams with cross-talk epsilon (polbeam.cpp:281-383).
 * tilde_a/tilde_b: 4 x npix (I,Q,U,V); out_a/out_b: 4 x npix. */
void orc_beam_build(int64_t nside_beam, int64_t npix, double epsilon,
                    char enabled, int64_t nside_sky, const float* tilde_a,
                    const float* tilde_b, float* out_a, float* out_b);

/* ---------------- convolution ---------------- */
/* interp: 0 = nearest beam pixel (reference live path), 1 = bilinear. */
/* float form: ra, dec, pa as the caller's float pointing; sky 4 x npix
 * float (I,Q,U,V planes); beams 4 x npixB float (planes).  Outputs float. */
void orc_convolve_f32(int64_t nsamples, const float* ra, const float* dec,
                      const float* pa, int64_t nside_sky, const float* sky,
                      int64_t nside_beam, int64_t npix_beam,
                      const float* beam_a, const float* beam_b, int interp,
                      char polflag, float* out_a, float* out_b, int nthreads);
/* double form: every input, product and output in double. */
void orc_convolve_f64(int64_t nsamples, const double* ra, const double* dec,
                      const double* pa, int64_t nside_sky, const double* sky,
                      int64_t nside_beam, int64_t npix_beam,
                      const double* beam_a, const double* beam_b, int interp,
                      char polflag, double* out_a, double* out_b,
                      int nthreads);
/* Per-pair geometry for a list of (sample, sky pixel) pairs: beam pixel,
 * chi.  Used to pin the device per-pair matching bit-for-bit. */
void orc_match_pairs(int64_t npairs, const double* ra, const double* dec,
                     const double* pa, const int64_t* skypix,
                     int64_t nside_sky, int64_t nside_beam, int64_t* beampix,
                     double* chi);
/* Adjoint (transpose) of orc_convolve_f64, nearest-pixel beams:
 * gsky (4 x npix, zero-initialised by the caller) += sum over pairs. */
void orc_adjoint_f64(int64_t nsamples, const double* ra, const double* dec,
                     const double* pa, int64_t nside_sky, int64_t nside_beam,
                     int64_t npix_beam, const double* beam_a,
                     const double* beam_b, const double* g_a,
                     const double* g_b, double* gsky);

/* ---------------- binned map-making (src/SkyMap/skymap.cpp) ---------------- */
/* SkyMap::accumulate_data (skymap.cpp:68-132).  Arrays indexed
 * [det * nsamples + s]; for every (det, s) in that order, in double:
 *   pixel = ang2pix(pi/2 - dec, ra), psi = -(pol[det] + pa), c = cos 2psi,
 *   s = sin 2psi, AtD[3p..] += (d, c d, s d),
 *   AtA[9p..] += (1, c, s, c, c c, c s, s, c s, s s).
 * ata (9 x npix) and atd (3 x npix) are accumulated into (the caller zeroes
 * them first: the reference's constructor leaves them uninitialised). */
void orc_map_accumulate_f32(int64_t nside, int64_t nsamples, const float* ra, const float* dec,
                            const float* pa, int ndet, const float* pol, const float* data,
                            double* ata, double* atd);
void orc_map_accumulate_f64(int64_t nside, int64_t nsamples, const double* ra, const double* dec,
                            const double* pa, int ndet, const float* pol, const double* data,
                            double* ata, double* atd);
/* LAPACK dgesv for one 3 x 3 system (the reference links it at
 * skymap.cpp:13-19 and calls it at :186-193; LAPACK is not in the reference
 * tree and its version is unpinned).  Restates the published reference
 * LAPACK/BLAS algorithm: dgetf2 (unblocked LU, partial pivoting by the first
 * largest |a|, multipliers by the reciprocal of the pivot when it is at least
 * the safe minimum, rank-1 updates a + l (-u)), then, only when no pivot is
 * exactly zero, dgetrs (row interchanges; unit-lower and upper triangular
 * solves, column-oriented as the reference dtrsm).  a: column-major 3 x 3,
 * overwritten with the factors; b: right-hand side, overwritten with the
 * solution (unchanged when info != 0).  Returns info (0, or k if U(k,k) is
 * exactly zero, 1-based). */
int orc_dgesv3(double* a, int* ipiv, double* b);
/* SkyMap::solve_map (skymap.cpp:134-231): per pixel, hits = (int)AtA[0];
 * hits >= 3: solve AtA x = AtD (dgesv); x to I, Q, U; a singular system
 * keeps AtD as I, Q, U and sets hits to 0.  hits < 3: I = Q = U = 0. */
void orc_map_solve(int64_t npix, const double* ata, const double* atd, float* I, float* Q,
                   float* U, int* hits);

/* ---------------- focal plane to sky (src/Bpoint/bpoint.cpp:553-674) ---- */
/* BPoint::focal_plane_to_sky: detector pointing from the array centre's
 * (x_ac, y_ac, rot_ac) and the receiver-frame offsets (det_dx right,
 * det_dy up) and polarization angles; flag 0 Az/El, 1 Ra/Dec, 2
 * source-relative.  Outputs ndets x nsamples, [det * nsamples + s]. */
void orc_focal_plane_to_sky(int ndets, const double* det_dx, const double* det_dy,
                            const double* det_pol, int64_t nsamples, const double* x_ac,
                            const double* y_ac, const double* rot_ac, int flag,
                            double* x_det, double* y_det, double* rot_det);

#ifdef __cplusplus
}
#endif
#endif
