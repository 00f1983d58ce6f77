/*
 * refdev_harness.cpp -- host entry points around the reference's own
 * device HEALPix port (src/GpuConvolver/cuda/cudaHealpix.cu) and device
 * rotation (src/GpuConvolver/cuda/cudaSphtransf.cu), which oracle/build_ref.sh
 * compiles for the host with __device__ defined away.
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle's HEALPix restatement.
 */
#include "GpuConvolver/cuda/cudaHealpix.h"
#include "GpuConvolver/cuda/cudaSphtransf.h"

extern "C" {
void refdev_pix2ang(int nside, long n, const long* pix, double* theta, double* phi)
{
    for (long i = 0; i < n; ++i) cudaHealpix::pix2ang(nside, pix[i], &theta[i], &phi[i]);
}
void refdev_ang2pix(int nside, long n, const double* theta, const double* phi, long* pix)
{
    for (long i = 0; i < n; ++i) pix[i] = cudaHealpix::ang2pix(nside, theta[i], phi[i]);
}
void refdev_get_interpol(int nside, long n, const double* theta, const double* phi,
                         long* pix4, double* wgt4)
{
    for (long i = 0; i < n; ++i) {
        int p[4];
        double w[4];
        cudaHealpix::get_interpol(nside, theta[i], phi[i], p, w);
        for (int k = 0; k < 4; ++k) {
            pix4[4 * i + k] = p[k];
            wgt4[4 * i + k] = w[k];
        }
    }
}
void refdev_rho_sigma_chi(long n, const double* ra_bc, const double* dec_bc,
                          const double* psi_bc, const double* ra_pix,
                          const double* dec_pix, double* rho, double* sigma,
                          double* chi)
{
    for (long i = 0; i < n; ++i)
        cudaSphericalTransformations::rho_sigma_chi_pix(&rho[i], &sigma[i], &chi[i],
                                                        ra_bc[i], dec_bc[i], psi_bc[i],
                                                        ra_pix[i], dec_pix[i]);
}
}
