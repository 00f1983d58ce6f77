// pointing.cu -- detector pointing from the array centre's pointing, on the
// GPU: BPoint::focal_plane_to_sky (src/Bpoint/bpoint.cpp:553-674,
// src/Bpoint/BPoint.h:99-103), the step that turns the telescope's boresight
// track into the per-detector (ra, dec, pa) the convolver takes.
//
// It is the part of BPoint that is geometry only: the spherical triangle
// array centre -- detector -- pole (zenith, celestial pole or source).  A
// detector at receiver-frame offsets (dx right, dy up) lies at angular
// distance r = acos(cos dx cos dy) from the array centre, in the direction
// a = atan2(sin dy, sin dx cos dy) from the receiver's x axis; with the
// array centre at latitude y and the receiver's up axis at position angle
// rot (the angle from the pole, counter-clockwise on the sky), the angle
// detector -> array centre -> pole is g = pi/2 - a - rot, and
//   latitude   asin(cos r sin y + sin r cos y cos g)
//   longitude  x -/+ atan2(sin r sin g, cos r cos y - sin r sin y cos g)
//              (Ra/Dec: minus, Az/El: plus)
//   position angle of the detector (of the receiver-frame pole seen from it)
//              atan2(cos y sin rot cos dx - sin y sin dx,
//                    cos y cos rot cos dy - (sin y cos dx + cos y sin rot sin dx) sin dy)
// plus the detector's polarization angle.  BPoint's ephemeris part (SOFA and
// the JPL tables, absent from the reference tree) is not on this path.
//
// One thread per (detector, sample), FP64 throughout (the pointing feeds the
// FP64 per-sample frame of the convolver); outputs [det * nsamples + s].
#include <cuda_runtime.h>

#include <string>

#include "../../include/pisco_gb300.h"
#include "hpx.cuh"
#include "internal.h"

namespace pisco {
void set_null_ctx_error(const char* msg);  // capi.cu
}

using namespace pisco;

namespace {

__global__ void focal_plane_kernel(int ndets, const double* __restrict__ det_dx,
                                   const double* __restrict__ det_dy,
                                   const double* __restrict__ det_pol, long long ns,
                                   const double* __restrict__ x_ac, const double* __restrict__ y_ac,
                                   const double* __restrict__ rot_ac, int flag,
                                   double* __restrict__ x_det, double* __restrict__ y_det,
                                   double* __restrict__ rot_det)
{
    const long long total = (long long)ndets * ns;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int d = (int)(k / ns);
        const long long s = k - (long long)d * ns;
        double sx, cx, sdy, cdy;
        sincos(det_dx[d], &sx, &cx);
        sincos(det_dy[d], &sdy, &cdy);
        const double cr = cx * cdy;
        const double sr = sqrt((1.0 - cr) * (1.0 + cr));
        const double a = atan2(sdy, sx * cdy);
        const double rot = rot_ac[s];
        double sg, cg, sl, cl, se, ce;
        sincos(kHalfPi - a - rot, &sg, &cg);
        sincos(y_ac[s], &sl, &cl);
        sincos(rot, &se, &ce);
        y_det[k] = asin(cr * sl + sr * cl * cg);
        const double pa = atan2(cl * se * cx - sl * sx, cl * ce * cdy - (sl * cx + cl * se * sx) * sdy);
        rot_det[k] = pa + det_pol[d];
        if (flag == 2) {
            x_det[k] = -pa;
        } else {
            const double dl = atan2(sr * sg, cr * cl - sr * sl * cg);
            x_det[k] = flag == 0 ? x_ac[s] + dl : x_ac[s] - dl;
        }
    }
}

pisco_status reject(pisco_status st, const std::string& msg)
{
    set_null_ctx_error(msg.c_str());
    return st;
}

pisco_status check_args(int ndets, long nsamples, int flag, bool ptrs)
{
    if (ndets < 0 || nsamples < 0) return reject(PISCO_ERR_INVALID_ARGUMENT, "focal_plane_to_sky: negative size");
    if ((long long)ndets * nsamples > (1LL << 40))
        return reject(PISCO_ERR_INVALID_ARGUMENT, "focal_plane_to_sky: more than 2^40 outputs");
    if (flag < 0 || flag > 2) return reject(PISCO_ERR_INVALID_ARGUMENT, "focal_plane_to_sky: flag must be 0, 1 or 2");
    if (!ptrs && ndets > 0 && nsamples > 0)
        return reject(PISCO_ERR_INVALID_ARGUMENT, "focal_plane_to_sky: NULL array");
    return PISCO_OK;
}

cudaError_t launch(int ndets, const double* dx, const double* dy, const double* pol, long long ns,
                   const double* x, const double* y, const double* rot, int flag, double* xo,
                   double* yo, double* ro, cudaStream_t st)
{
    const long long total = (long long)ndets * ns;
    if (total <= 0) return cudaSuccess;
    const long long b = (total + 255) / 256;
    focal_plane_kernel<<<(int)(b < 8192 ? b : 8192), 256, 0, st>>>(ndets, dx, dy, pol, ns, x, y,
                                                                    rot, flag, xo, yo, ro);
    return cudaGetLastError();
}

}  // namespace

extern "C" {

pisco_status pisco_focal_plane_to_sky_device(int ndets, const double* d_det_dx,
                                             const double* d_det_dy, const double* d_det_pol,
                                             long nsamples, const double* d_x_ac,
                                             const double* d_y_ac, const double* d_rot_ac, int flag,
                                             double* d_x_det, double* d_y_det, double* d_rot_det,
                                             void* stream)
{
    set_null_ctx_error("");
    pisco_status st = check_args(ndets, nsamples, flag,
                                 d_det_dx && d_det_dy && d_det_pol && d_x_ac && d_y_ac &&
                                     d_rot_ac && d_x_det && d_y_det && d_rot_det);
    if (st != PISCO_OK) return st;
    const cudaError_t e = launch(ndets, d_det_dx, d_det_dy, d_det_pol, nsamples, d_x_ac, d_y_ac,
                                 d_rot_ac, flag, d_x_det, d_y_det, d_rot_det, (cudaStream_t)stream);
    if (e != cudaSuccess) return reject(PISCO_ERR_CUDA, std::string("focal_plane_to_sky: ") + cudaGetErrorString(e));
    return PISCO_OK;
}

pisco_status pisco_focal_plane_to_sky(int ndets, const double* det_dx, const double* det_dy,
                                      const double* det_pol, long nsamples, const double* x_ac,
                                      const double* y_ac, const double* rot_ac, int flag,
                                      double* x_det, double* y_det, double* rot_det)
{
    set_null_ctx_error("");
    pisco_status st = check_args(ndets, nsamples, flag,
                                 det_dx && det_dy && det_pol && x_ac && y_ac && rot_ac && x_det &&
                                     y_det && rot_det);
    if (st != PISCO_OK || ndets == 0 || nsamples == 0) return st;
    const size_t nd = sizeof(double) * ndets, ns = sizeof(double) * nsamples;
    const size_t no = sizeof(double) * (size_t)ndets * nsamples;
    double* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, 3 * nd + 3 * ns + 3 * no);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return reject(e == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY : PISCO_ERR_CUDA,
                      std::string("focal_plane_to_sky: ") + cudaGetErrorString(e));
    }
    double* d[9];
    d[0] = buf;
    d[1] = d[0] + ndets;
    d[2] = d[1] + ndets;
    d[3] = d[2] + ndets;
    d[4] = d[3] + nsamples;
    d[5] = d[4] + nsamples;
    d[6] = d[5] + nsamples;
    d[7] = d[6] + (size_t)ndets * nsamples;
    d[8] = d[7] + (size_t)ndets * nsamples;
    const double* in[6] = {det_dx, det_dy, det_pol, x_ac, y_ac, rot_ac};
    for (int k = 0; k < 6 && e == cudaSuccess; ++k)
        e = cudaMemcpy(d[k], in[k], k < 3 ? nd : ns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = launch(ndets, d[0], d[1], d[2], nsamples, d[3], d[4], d[5], flag, d[6], d[7], d[8], 0);
    double* out[3] = {x_det, y_det, rot_det};
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpy(out[k], d[6 + k], no, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return reject(PISCO_ERR_CUDA, std::string("focal_plane_to_sky: ") + cudaGetErrorString(e));
    }
    return PISCO_OK;
}

}  // extern "C"
