// beam_dev.cu -- detector-pair beams built on the GPU, straight into the
// npix x 8 float layout (a.I,Q,U,V, b.I,Q,U,V) that pisco_set_beam_device and
// the batched descriptors take, and the beam-parameter gradient of the
// elliptical Gaussian model reduced on the GPU.
//
// * pisco_beam_build_device: PolBeam::beam_from_fields + PolBeam::build
//   (polbeam.cpp:117-288) from device field planes.  Per pixel the same
//   rounded FP64 operations as the host steps (explicitly rounded, no
//   contraction); the normalisation sums of tilde I run as a fixed tree
//   instead of the reference's left-to-right loop, and cos/sin are the
//   device's, so beams agree with the host builder to about one float ulp.
// * pisco_beam_gaussian_device / pisco_beam_gaussian_param_grad_device: the
//   model of beam_model.h and its analytic gradient (the host function
//   pisco_beam_gaussian_param_grad), so a beam-fitting loop (beam -> forward
//   -> adjoint -> parameter gradient) never leaves the device.
//
// Every sum is deterministic: the grid depends on npix only, each thread adds
// its pixels in order, blocks reduce by a fixed shuffle tree, and one block
// adds the block partials in block order.  Work per pixel is a few hundred
// flops on 64 B (fields) or 32 B (beam) of traffic; npix is 10^4 - 10^6, so
// the launches are latency-bound (microseconds).
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/pisco_gb300.h"
#include "beam_model.h"
#include "ctx.h"
#include "hpx.cuh"
#include "internal.h"

using namespace pisco;

namespace {

constexpr int kBT = 256;         // threads per block
constexpr int kMaxBlocks = 1024; // block partials reduced by one block
constexpr int kSums = 12;        // widest reduction (the parameter gradient)

int beam_grid(long npix)
{
    const long b = (npix + kBT - 1) / kBT;
    return (int)(b < 1 ? 1 : (b > kMaxBlocks ? kMaxBlocks : b));
}

// Block sum of K doubles per thread; thread 0 ends with the totals.  sh holds
// K x 32 doubles.  Shuffle-down trees: the same order on every run.
template <int K>
__device__ __forceinline__ void block_sums(double (&v)[K], double* sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = __dadd_rn(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) sh[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double x = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = __dadd_rn(x, __shfl_down_sync(0xffffffffu, x, o));
            v[k] = x;
        }
    }
}

// Tilde I, Q, U, V (Rosset et al. 2010) of one detector at pixel p from its
// field planes f (magEco, phsEco, magEcx, phsEcx; npix each), with the
// operations of std::polar / std::norm / complex multiply of the host step.
__device__ __forceinline__ void tilde_at(const double* __restrict__ f, long npix, long p, float t[4])
{
    const double mco = f[p], pco = f[npix + p], mcx = f[2 * npix + p], pcx = f[3 * npix + p];
    double sco, cco, scx, ccx;
    sincos(pco, &sco, &cco);
    sincos(pcx, &scx, &ccx);
    const double ar = PD_MUL(mco, cco), ai = PD_MUL(mco, sco);
    const double br = PD_MUL(mcx, ccx), bi = -PD_MUL(mcx, scx);  // conj(ecx)
    const double n0 = PD_ADD(PD_MUL(ar, ar), PD_MUL(ai, ai));
    const double n1 = PD_ADD(PD_MUL(br, br), PD_MUL(bi, bi));
    const double xr = PD_SUB(PD_MUL(ar, br), PD_MUL(ai, bi));
    const double xi = PD_ADD(PD_MUL(ar, bi), PD_MUL(ai, br));
    t[0] = (float)PD_ADD(n0, n1);
    t[1] = (float)PD_SUB(n0, n1);
    t[2] = (float)PD_MUL(2.0, xr);
    t[3] = (float)PD_MUL(-2.0, xi);
}

// Tilde beams of both detectors into ab (8 floats per pixel) and the block
// partial sums of tilde I of the enabled detectors.
__global__ void __launch_bounds__(kBT) tilde_kernel(long npix, const double* __restrict__ fa,
                                                    const double* __restrict__ fb, int sum_a,
                                                    int sum_b, float4* __restrict__ ab,
                                                    double* __restrict__ part)
{
    __shared__ double sh[2 * 32];
    double v[2] = {0.0, 0.0};
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        float ta[4] = {0.f, 0.f, 0.f, 0.f}, tb[4] = {0.f, 0.f, 0.f, 0.f};
        if (fa) tilde_at(fa, npix, p, ta);
        if (fb) tilde_at(fb, npix, p, tb);
        ab[2 * p] = make_float4(ta[0], ta[1], ta[2], ta[3]);
        ab[2 * p + 1] = make_float4(tb[0], tb[1], tb[2], tb[3]);
        if (sum_a) v[0] = __dadd_rn(v[0], (double)ta[0]);
        if (sum_b) v[1] = __dadd_rn(v[1], (double)tb[0]);
    }
    block_sums<2>(v, sh);
    if (threadIdx.x == 0) {
        part[kSums * blockIdx.x] = v[0];
        part[kSums * blockIdx.x + 1] = v[1];
    }
}

__device__ __forceinline__ float4 mix(float4 x, float4 y, double eps, double n)
{
    return make_float4((float)PD_DIV(PD_ADD((double)x.x, PD_MUL(eps, (double)y.x)), n),
                       (float)PD_DIV(PD_SUB((double)x.y, PD_MUL(eps, (double)y.y)), n),
                       (float)PD_DIV(PD_SUB((double)x.z, PD_MUL(eps, (double)y.z)), n),
                       (float)PD_DIV(PD_ADD((double)x.w, PD_MUL(eps, (double)y.w)), n));
}

// PolBeam::build's mixing with the cross-polar leakage eps, in place.
__global__ void __launch_bounds__(kBT) build_kernel(long npix, double eps,
                                                    const double* __restrict__ norms,
                                                    float4* __restrict__ ab)
{
    const double an = norms[0], bn = norms[1];
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        const float4 ta = ab[2 * p], tb = ab[2 * p + 1];
        ab[2 * p] = mix(ta, tb, eps, an);
        ab[2 * p + 1] = mix(tb, ta, eps, bn);
    }
}

struct GaussDev {
    GaussModel m;
    double dx, dy;
};

// Model weight g at beam pixel p, with the offsets (x, y) from its centre.
__device__ __forceinline__ double gauss_at(const Hpx& h, const GaussDev& gd, long p, double* xo,
                                           double* yo)
{
    double th, ph, s, c;
    pix2ang(h, p, &th, &ph);
    sincos(ph, &s, &c);
    const double x = th * c - gd.dx, y = th * s - gd.dy;
    *xo = x;
    *yo = y;
    return exp(-(gd.m.ca * x * x + 2.0 * gd.m.cb * x * y + gd.m.cc * y * y));
}

// Model weights into g and their block partial sums.
__global__ void __launch_bounds__(kBT) gauss_kernel(Hpx h, long npix, GaussDev gd,
                                                    double* __restrict__ g,
                                                    double* __restrict__ part)
{
    __shared__ double sh[32];
    double v[1] = {0.0};
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        double x, y;
        const double w = gauss_at(h, gd, p, &x, &y);
        g[p] = w;
        v[0] = __dadd_rn(v[0], w);
    }
    block_sums<1>(v, sh);
    if (threadIdx.x == 0) part[kSums * blockIdx.x] = v[0];
}

// B = ((1 + eps) g, (1 - eps) g, 0, 0) / N for both detectors.
__global__ void __launch_bounds__(kBT) gauss_out_kernel(long npix, double eps,
                                                        const double* __restrict__ g,
                                                        const double* __restrict__ norms,
                                                        float4* __restrict__ ab)
{
    const double n = norms[0];
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        const float4 b = make_float4((float)((1.0 + eps) * g[p] / n), (float)((1.0 - eps) * g[p] / n),
                                     0.f, 0.f);
        ab[2 * p] = b;
        ab[2 * p + 1] = b;
    }
}

// Per-pixel terms of the parameter gradient: sums of g, G g, dg/dt, G dg/dt
// (t = F, e, phi0, dx, dy), G = sum_k c_k dL/dB[p][k].
template <typename T>
__global__ void __launch_bounds__(kBT) param_grad_kernel(Hpx h, long npix, GaussDev gd, double eps,
                                                         const T* __restrict__ gbeam,
                                                         double* __restrict__ part)
{
    __shared__ double sh[kSums * 32];
    double v[kSums];
#pragma unroll
    for (int k = 0; k < kSums; ++k) v[k] = 0.0;
    const GaussModel& m = gd.m;
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        double x, y;
        const double g = gauss_at(h, gd, p, &x, &y);
        const T* gb = gbeam + 8 * p;
        const double G = (1.0 + eps) * ((double)gb[0] + (double)gb[4]) +
                         (1.0 - eps) * ((double)gb[1] + (double)gb[5]);
        const double dQ[5] = {x * x * m.aF + 2.0 * x * y * m.bF + y * y * m.cF,
                              x * x * m.ae + 2.0 * x * y * m.be + y * y * m.ce,
                              x * x * m.ap + 2.0 * x * y * m.bp + y * y * m.cp,
                              -2.0 * (m.ca * x + m.cb * y), -2.0 * (m.cb * x + m.cc * y)};
        v[0] += g;
        v[1] += G * g;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const double dg = -g * dQ[t];
            v[2 + t] += dg;
            v[7 + t] += G * dg;
        }
    }
    block_sums<kSums>(v, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < kSums; ++k) part[kSums * blockIdx.x + k] = v[k];
}

// The model's weight and its derivatives at every beam pixel, for the fused
// adjoint (adjoint.cu, ScatterParams): tab[p] = (g, dg/dF, dg/de, dg/dphi0 |
// dg/ddx, dg/ddy, 0, 0) as floats, one 32-byte row per pixel; and the block
// partials of sum g (column 0) and sum dg/dt (columns 2..6) in
// param_grad_kernel's layout.  Columns 1 and 7..11 -- the sums weighted by
// the beam-map gradient -- are left zero: the fused adjoint adds them as one
// more row, and finish_kernel completes the gradient as for
// param_grad_kernel.
__global__ void __launch_bounds__(kBT) param_table_kernel(Hpx h, long npix, GaussDev gd,
                                                          float4* __restrict__ tab,
                                                          double* __restrict__ part)
{
    __shared__ double sh[kSums * 32];
    double v[kSums];
#pragma unroll
    for (int k = 0; k < kSums; ++k) v[k] = 0.0;
    const GaussModel& m = gd.m;
    for (long p = blockIdx.x * (long)kBT + threadIdx.x; p < npix; p += (long)gridDim.x * kBT) {
        double x, y;
        const double g = gauss_at(h, gd, p, &x, &y);
        const double dQ[5] = {x * x * m.aF + 2.0 * x * y * m.bF + y * y * m.cF,
                              x * x * m.ae + 2.0 * x * y * m.be + y * y * m.ce,
                              x * x * m.ap + 2.0 * x * y * m.bp + y * y * m.cp,
                              -2.0 * (m.ca * x + m.cb * y), -2.0 * (m.cb * x + m.cc * y)};
        double dg[5];
        v[0] += g;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            dg[t] = -g * dQ[t];
            v[2 + t] += dg[t];
        }
        tab[2 * p] = make_float4((float)g, (float)dg[0], (float)dg[1], (float)dg[2]);
        tab[2 * p + 1] = make_float4((float)dg[3], (float)dg[4], 0.f, 0.f);
    }
    block_sums<kSums>(v, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < kSums; ++k) part[kSums * blockIdx.x + k] = v[k];
}

// One block adds the first K columns of nblk partial rows, in block order per
// thread then by the fixed tree, and finishes:
//   kind 0 (PolBeam build): out[0..1] = sums x oc, + 1e-8 on the disabled side;
//   kind 1 (Gaussian model): out[0] = sum x oc;
//   kind 2 (parameter gradient): out[0..4] = dL/d(F, e, phi0, dx, dy), NaN
//   when the model's weights sum to zero.
template <int K>
__global__ void __launch_bounds__(kBT) finish_kernel(int nblk, const double* __restrict__ part,
                                                     int kind, double oc, int add_a, int add_b,
                                                     double* __restrict__ out)
{
    __shared__ double sh[K * 32];
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kBT)
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = __dadd_rn(v[k], part[kSums * b + k]);
    block_sums<K>(v, sh);
    if (threadIdx.x != 0) return;
    if (kind == 0) {
        double an = __dmul_rn(v[0], oc), bn = __dmul_rn(v[K > 1 ? 1 : 0], oc);
        if (add_b) bn = __dadd_rn(bn, 1e-8);
        if (add_a) an = __dadd_rn(an, 1e-8);
        out[0] = an;
        out[1] = bn;
    } else if (kind == 1) {
        out[0] = v[0] * oc;
    }
    if constexpr (K >= 12) {
        if (kind == 2) {
            const double sg = v[0], sGg = v[1], n = oc * sg;
            for (int t = 0; t < 5; ++t)
                out[t] = n > 0.0 ? (v[7 + t] - sGg * v[2 + t] / sg) / n
                                 : __longlong_as_double(0x7ff8000000000000ll);
        }
    }
}

pisco_status fail(pisco_ctx* c, pisco_status s, const std::string& m)
{
    c->error = m;
    return s;
}

pisco_status cuda_fail(pisco_ctx* c, cudaError_t e, const char* what)
{
    cudaGetLastError();
    return fail(c, e == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY : PISCO_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

// Scratch: kMaxBlocks partial rows, 16 results, then npix doubles (model weights).
pisco_status scratch(pisco_ctx* c, long npix, double** part, double** res, double** g)
{
    const size_t need = sizeof(double) * ((size_t)kMaxBlocks * kSums + 16 + (size_t)npix);
    pisco_status st = c->ensure((void**)&c->beam_scr, &c->beam_scr_cap, need, "beam scratch");
    if (st != PISCO_OK) return st;
    *part = c->beam_scr;
    *res = c->beam_scr + (size_t)kMaxBlocks * kSums;
    *g = *res + 16;
    return PISCO_OK;
}

pisco_status check_grid(pisco_ctx* c, int nside_beam, long npix, int nside_sky)
{
    if (nside_beam < 1 || nside_beam > 8192) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nside must be in [1, 8192]");
    if (nside_sky < 1 || nside_sky > 8192) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky nside must be in [1, 8192]");
    if (npix < 1 || npix >= 12L * nside_beam * nside_beam)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nPixels must be in [1, 12 nside^2)");
    return PISCO_OK;
}

pisco_status check_model(pisco_ctx* c, double fwhm_deg, double e, double phi0, double dx, double dy)
{
    if (!(fwhm_deg > 0.0) || !std::isfinite(fwhm_deg)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "fwhm must be > 0");
    if (!(std::fabs(e) < 1.0)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "ellipticity must be in (-1, 1)");
    if (!std::isfinite(phi0) || !std::isfinite(dx) || !std::isfinite(dy))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "phi0, dx, dy must be finite");
    return PISCO_OK;
}

double ratio_sq(int nside_sky, int nside_beam)
{
    double oc = (double)nside_sky / (double)nside_beam;
    return oc * oc;
}

}  // namespace

namespace pisco {

int gauss_table_rows(long npix) { return beam_grid(npix); }

cudaError_t launch_gauss_param_table(int nside_beam, long npix, double fwhm_deg, double e,
                                     double phi0_deg, double dx, double dy, float* tab,
                                     double* part, cudaStream_t st)
{
    const GaussDev gd{gauss_model(fwhm_deg, e, phi0_deg), dx, dy};
    param_table_kernel<<<beam_grid(npix), kBT, 0, st>>>(hpx_make(nside_beam), npix, gd,
                                                         (float4*)tab, part);
    return cudaGetLastError();
}

cudaError_t launch_gauss_param_finish(const double* part, int nrows, double oc, double* out,
                                      cudaStream_t st)
{
    finish_kernel<kSums><<<1, kBT, 0, st>>>(nrows, part, 2, oc, 0, 0, out);
    return cudaGetLastError();
}

}  // namespace pisco

extern "C" {

pisco_status pisco_beam_build_device(pisco_ctx* c, int nside_beam, long npix, double epsilon,
                                     char en, int nside_sky, const double* d_fields_a,
                                     const double* d_fields_b, float* d_ab, int set_beam,
                                     void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = check_grid(c, nside_beam, npix, nside_sky);
    if (st != PISCO_OK) return st;
    if (en != 'a' && en != 'b' && en != 'p') return fail(c, PISCO_ERR_INVALID_ARGUMENT, "enabledDets must be 'a', 'b' or 'p'");
    if ((en != 'b' && !d_fields_a) || (en != 'a' && !d_fields_b))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "fields of an enabled detector are NULL");
    if (!d_ab || ((uintptr_t)d_ab & 15)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam output must be a 16-B aligned device pointer");
    if (!std::isfinite(epsilon)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "epsilon must be finite");
    if ((st = c->activate()) != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    double *part, *res, *g;
    if ((st = scratch(c, npix, &part, &res, &g)) != PISCO_OK) return st;
    const int grid = beam_grid(npix);
    float4* ab = reinterpret_cast<float4*>(d_ab);
    tilde_kernel<<<grid, kBT, 0, s>>>(npix, d_fields_a, d_fields_b, en != 'b', en != 'a', ab, part);
    finish_kernel<2><<<1, kBT, 0, s>>>(grid, part, 0, ratio_sq(nside_sky, nside_beam), en == 'b',
                                       en == 'a', res);
    build_kernel<<<grid, kBT, 0, s>>>(npix, epsilon, res, ab);
    CK(cudaGetLastError(), "beam build kernels");
    return set_beam ? pisco_set_beam_device(c, nside_beam, npix, d_ab, PISCO_FLOAT32, s) : PISCO_OK;
}

pisco_status pisco_beam_gaussian_device(pisco_ctx* c, int nside_beam, long npix, double epsilon,
                                        int nside_sky, double fwhm_deg, double ellipticity,
                                        double phi0_deg, double dx, double dy, float* d_ab,
                                        int set_beam, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = check_grid(c, nside_beam, npix, nside_sky);
    if (st != PISCO_OK) return st;
    if ((st = check_model(c, fwhm_deg, ellipticity, phi0_deg, dx, dy)) != PISCO_OK) return st;
    if (!d_ab || ((uintptr_t)d_ab & 15)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam output must be a 16-B aligned device pointer");
    if (!std::isfinite(epsilon)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "epsilon must be finite");
    if ((st = c->activate()) != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    double *part, *res, *g;
    if ((st = scratch(c, npix, &part, &res, &g)) != PISCO_OK) return st;
    const int grid = beam_grid(npix);
    const GaussDev gd{gauss_model(fwhm_deg, ellipticity, phi0_deg), dx, dy};
    gauss_kernel<<<grid, kBT, 0, s>>>(hpx_make(nside_beam), npix, gd, g, part);
    finish_kernel<1><<<1, kBT, 0, s>>>(grid, part, 1, ratio_sq(nside_sky, nside_beam), 0, 0, res);
    gauss_out_kernel<<<grid, kBT, 0, s>>>(npix, epsilon, g, res, reinterpret_cast<float4*>(d_ab));
    CK(cudaGetLastError(), "gaussian beam kernels");
    return set_beam ? pisco_set_beam_device(c, nside_beam, npix, d_ab, PISCO_FLOAT32, s) : PISCO_OK;
}

pisco_status pisco_beam_gaussian_param_grad_device(pisco_ctx* c, int nside_beam, long npix,
                                                   double epsilon, int nside_sky, double fwhm_deg,
                                                   double ellipticity, double phi0_deg, double dx,
                                                   double dy, const void* d_gbeam, pisco_dtype dt,
                                                   double* d_grad, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = check_grid(c, nside_beam, npix, nside_sky);
    if (st != PISCO_OK) return st;
    if ((st = check_model(c, fwhm_deg, ellipticity, phi0_deg, dx, dy)) != PISCO_OK) return st;
    if (!d_gbeam || !d_grad) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "gbeam and grad must not be NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    if ((st = c->activate()) != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    double *part, *res, *g;
    if ((st = scratch(c, npix, &part, &res, &g)) != PISCO_OK) return st;
    const int grid = beam_grid(npix);
    const GaussDev gd{gauss_model(fwhm_deg, ellipticity, phi0_deg), dx, dy};
    const Hpx h = hpx_make(nside_beam);
    if (dt == PISCO_FLOAT32)
        param_grad_kernel<float><<<grid, kBT, 0, s>>>(h, npix, gd, epsilon, (const float*)d_gbeam, part);
    else
        param_grad_kernel<double><<<grid, kBT, 0, s>>>(h, npix, gd, epsilon, (const double*)d_gbeam, part);
    finish_kernel<kSums><<<1, kBT, 0, s>>>(grid, part, 2, ratio_sq(nside_sky, nside_beam), 0, 0, d_grad);
    CK(cudaGetLastError(), "beam parameter gradient kernels");
    return PISCO_OK;
}

}  // extern "C"
