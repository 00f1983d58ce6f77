// capi_adjoint.cu -- C ABI of the adjoint (pisco_adjoint, pisco_adjoint_device)
// and of the device-side beam setter used by the autograd binding.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pisco_gb300.h"
#include "ctx.h"
#include "internal.h"

using namespace pisco;

namespace {

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

__global__ void interleaved_to_f8(const float* in, F8* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float* p = in + 8 * i;
        out[i].a = make_float4(p[0], p[1], p[2], p[3]);
        out[i].b = make_float4(p[4], p[5], p[6], p[7]);
    }
}

__global__ void d_interleaved_to_f8(const double* in, F8* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double* p = in + 8 * i;
        out[i].a = make_float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
        out[i].b = make_float4((float)p[4], (float)p[5], (float)p[6], (float)p[7]);
    }
}

__global__ void widen_f32(const float* in, double* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// smallest power of two >= 2^62 / bound, as the fixed-point scale
// (at most 2^126, so that the kernels can apply it in FP32; a bound below
// 2^-64 keeps every total far below 2^62 all the same)
double fixed_scale(double bound)
{
    if (!(bound > 0.0) || !std::isfinite(bound)) return 0.0;
    const int e = (int)std::ceil(std::log2(bound));
    return std::ldexp(1.0, std::min(62 - e, 126));
}

// The fused Gaussian beam-parameter gradient of one adjoint call: the model
// table and its partial rows (rows + 1 rows: the adjoint adds the last), the
// per-warp partials, the result (5 device doubles) and the model's c.
struct ParamPlan {
    const float* tab;
    double* part;
    int rows;
    double* ppart;
    double* grad;
    double oc;  // (nside_sky / nside_beam)^2
    float ci, cq;
};

pisco_status adjoint_core(pisco_ctx* c, long begin, long n, const void* d_ga, const void* d_gb,
                          pisco_dtype g_dtype, void* d_gsky, void* d_gbeam, pisco_dtype out_dtype,
                          pisco_adjoint_mode mode, cudaStream_t s, const ParamPlan* pp);

}  // namespace

extern "C" {

pisco_status pisco_set_beam_device(pisco_ctx* c, int nside, long npix, const void* d_ab,
                                   pisco_dtype dt, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (nside < 1 || nside > 8192) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nside must be in [1, 8192]");
    if (npix < 1 || npix >= 12L * nside * nside)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nPixels must be in [1, 12 nside^2)");
    if (!d_ab) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam pointer is NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    st = c->ensure((void**)&c->beam32, &c->beam32_cap, sizeof(F8) * npix, "beam buffer");
    if (st != PISCO_OK) return st;
    if (dt == PISCO_FLOAT32) interleaved_to_f8<<<256, 256, 0, s>>>((const float*)d_ab, c->beam32, npix);
    else d_interleaved_to_f8<<<256, 256, 0, s>>>((const double*)d_ab, c->beam32, npix);
    CK(cudaGetLastError(), "beam conversion");
    if (s != c->stream) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(c->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    c->beam64_valid = false;
    c->nside_beam = nside;
    c->npix_beam = npix;
    c->rho_max = pisco_beam_rho_max(nside, npix);
    c->pairs_valid = false;
    return PISCO_OK;
}

pisco_status pisco_adjoint_device(pisco_ctx* c, long begin, long n, const void* d_ga, const void* d_gb,
                                  pisco_dtype g_dtype, void* d_gsky, void* d_gbeam,
                                  pisco_dtype out_dtype, pisco_adjoint_mode mode, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!d_gsky && !d_gbeam) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "no gradient output requested");
    return adjoint_core(c, begin, n, d_ga, d_gb, g_dtype, d_gsky, d_gbeam, out_dtype, mode,
                        stream ? (cudaStream_t)stream : c->stream, nullptr);
}

pisco_status pisco_adjoint_gaussian_device(pisco_ctx* c, long begin, long n, const void* d_ga,
                                           const void* d_gb, pisco_dtype g_dtype, void* d_gsky,
                                           pisco_dtype out_dtype, pisco_adjoint_mode mode,
                                           double epsilon, int nside_sky, double fwhm_deg,
                                           double ellipticity, double phi0_deg, double dx,
                                           double dy, double* d_grad, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!d_grad) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "grad must not be NULL");
    if (nside_sky < 1 || nside_sky > 8192) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky nside must be in [1, 8192]");
    if (!(fwhm_deg > 0.0) || !std::isfinite(fwhm_deg) || !(std::fabs(ellipticity) < 1.0) ||
        !std::isfinite(phi0_deg) || !std::isfinite(dx) || !std::isfinite(dy) || !std::isfinite(epsilon))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT,
                    "model parameters: fwhm > 0, |ellipticity| < 1, the rest finite");
    if (!c->beam32 || !c->nside_beam) return fail(c, PISCO_ERR_NOT_READY, "sky and beam required");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const long npb = c->npix_beam;
    const int rows = gauss_table_rows(npb);
    const int max_warps = adjoint_max_warps(c->sm_count);
    st = c->ensure((void**)&c->adj_ptab, &c->adj_ptab_cap, sizeof(float) * 8 * npb, "parameter table");
    if (st != PISCO_OK) return st;
    st = c->ensure((void**)&c->adj_ppart, &c->adj_ppart_cap,
                   sizeof(double) * ((size_t)kParamCols * (rows + 1) + 6 * (size_t)max_warps),
                   "parameter partials");
    if (st != PISCO_OK) return st;
    ParamPlan pp;
    pp.tab = c->adj_ptab;
    pp.part = c->adj_ppart;
    pp.rows = rows;
    pp.ppart = c->adj_ppart + (size_t)kParamCols * (rows + 1);
    pp.grad = d_grad;
    const double oc = (double)nside_sky / (double)c->nside_beam;
    pp.oc = oc * oc;
    pp.ci = (float)(1.0 + epsilon);
    pp.cq = (float)(1.0 - epsilon);
    CK(launch_gauss_param_table(c->nside_beam, npb, fwhm_deg, ellipticity, phi0_deg, dx, dy,
                                c->adj_ptab, c->adj_ppart, s),
       "parameter table");
    return adjoint_core(c, begin, n, d_ga, d_gb, g_dtype, d_gsky, nullptr, out_dtype, mode, s, &pp);
}

}  // extern "C"

namespace {

// Sample plans of one adjoint launch: up to 16M (1.5 GB of scratch); a
// longer range plans in its warps.
constexpr long long kAdjointPlans = 1LL << 24;

pisco_status adjoint_core(pisco_ctx* c, long begin, long n, const void* d_ga, const void* d_gb,
                          pisco_dtype g_dtype, void* d_gsky, void* d_gbeam, pisco_dtype out_dtype,
                          pisco_adjoint_mode mode, cudaStream_t s, const ParamPlan* pp)
{
    if (!c->sky32 || !c->nside_sky || !c->beam32)
        return fail(c, PISCO_ERR_NOT_READY, "sky and beam required");
    if (begin < 0 || n < 0 || begin + n > c->nsamples)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sample range outside the scan");
    if (n > 0 && (!d_ga || !d_gb)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "TOD gradients are NULL");
    if ((g_dtype != PISCO_FLOAT32 && g_dtype != PISCO_FLOAT64) ||
        (out_dtype != PISCO_FLOAT32 && out_dtype != PISCO_FLOAT64))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    if ((int)mode & ~(PISCO_ADJ_DETERMINISTIC | PISCO_ADJ_SKY_IQU))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad adjoint mode");
    const bool deterministic = ((int)mode & PISCO_ADJ_DETERMINISTIC) != 0;
    const bool sky_iqu = ((int)mode & PISCO_ADJ_SKY_IQU) != 0;
    if (!tuned_supported(c->nside_beam, (int)c->npix_beam, c->rho_max))
        return fail(c, PISCO_ERR_UNSUPPORTED, "beam outside the adjoint's (TUNED) domain");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    const long long npix = 12LL * c->nside_sky * c->nside_sky;
    const long long nsky = 4 * npix, nbeam = 8LL * c->npix_beam;
    AdjArgs a{};
    a.nside_sky = c->nside_sky;
    a.sky32 = c->sky32;
    a.rings = c->rings;
    a.nside_beam = c->nside_beam;
    a.npix_beam = (int)c->npix_beam;
    a.beam32 = c->beam32;
    a.rho_max = c->rho_max;
    a.begin = begin;
    a.n = n;
    a.ra = c->ra;
    a.dec = c->dec;
    a.pa = c->pa;
    a.g_a = d_ga;
    a.g_b = d_gb;
    a.g_f64 = g_dtype == PISCO_FLOAT64;
    a.want_v = sky_iqu ? 0 : 1;
    a.interp = (int)c->interp;
    st = c->range_order(begin, n, s, &a.order);
    if (st != PISCO_OK) return st;
    a.err = c->d_err;
    a.fallbacks = c->d_fallbacks;
    if (pp) {
        a.ptab = pp->tab;
        a.ppart = pp->ppart;
        a.ceps_i = pp->ci;
        a.ceps_q = pp->cq;
    }
    // the samples' plans, if the whole range fits the scratch (the launch is
    // not split: the parameter gradient's per-warp rows cover one launch);
    // taken after every other buffer of the call, which may free the scratch
    auto take_plans = [&]() {
        void* plans = nullptr;
        long long plan_cap = 0;
        a.plans = nullptr;
        if (n > 0) c->plan_scratch(n, s, &plans, &plan_cap, kAdjointPlans);
        if (plans && plan_cap >= n) a.plans = static_cast<tuned::SamplePlan*>(plans);
    };
    int nwarps = 0;
    CK(cudaMemsetAsync(c->d_fallbacks, 0, sizeof(unsigned long long), s), "reset fallbacks");
    if (!deterministic) {
        a.fixed = 0;
        float* gs = nullptr;
        float* gbm = nullptr;
        if (d_gsky) {
            if (out_dtype == PISCO_FLOAT32) gs = (float*)d_gsky;
            else {
                st = c->ensure((void**)&c->adj_sky32, &c->adj_sky32_cap, sizeof(float) * nsky, "adjoint sky scratch");
                if (st != PISCO_OK) return st;
                gs = c->adj_sky32;
            }
            CK(cudaMemsetAsync(gs, 0, sizeof(float) * nsky, s), "zero sky gradient");
        }
        if (d_gbeam) {
            if (out_dtype == PISCO_FLOAT32) gbm = (float*)d_gbeam;
            else {
                st = c->ensure((void**)&c->adj_beam32, &c->adj_beam32_cap, sizeof(float) * nbeam, "adjoint beam scratch");
                if (st != PISCO_OK) return st;
                gbm = c->adj_beam32;
            }
            CK(cudaMemsetAsync(gbm, 0, sizeof(float) * nbeam, s), "zero beam gradient");
        }
        a.gsky32 = gs;
        a.gbeam32 = gbm;
        take_plans();
        if (n > 0) CK(launch_adjoint(a, c->sm_count, s, &nwarps), "adjoint launch");
        if (a.order) c->order_used(s);
        if (a.plans) c->plans_used(s);
        if (d_gsky && out_dtype == PISCO_FLOAT64) {
            widen_f32<<<1024, 256, 0, s>>>(gs, (double*)d_gsky, nsky);
            CK(cudaGetLastError(), "widen sky gradient");
        }
        if (d_gbeam && out_dtype == PISCO_FLOAT64) {
            widen_f32<<<256, 256, 0, s>>>(gbm, (double*)d_gbeam, nbeam);
            CK(cudaGetLastError(), "widen beam gradient");
        }
    } else {
        a.fixed = 1;
        // rigorous bounds on any accumulated total, from fixed-order reductions
        st = c->ensure((void**)&c->red, &c->red_cap, sizeof(double) * 3 * 256, "reduction scratch");
        if (st != PISCO_OK) return st;
        double h[3] = {0.0, 0.0, 0.0};
        if (n > 0) {
            CK(launch_abs_sum((const char*)d_ga, (const char*)d_gb, a.g_f64, n, c->red, s), "sum |g|");
            CK(launch_abs_max((const float*)c->beam32, nbeam, c->red + 256, s), "max |beam|");
            CK(launch_abs_max((const float*)c->sky32, nsky, c->red + 512, s), "max |sky|");
            CK(cudaMemcpyAsync(&h[0], c->red, sizeof(double), cudaMemcpyDeviceToHost, s), "bound D2H");
            CK(cudaMemcpyAsync(&h[1], c->red + 256, sizeof(double), cudaMemcpyDeviceToHost, s), "bound D2H");
            CK(cudaMemcpyAsync(&h[2], c->red + 512, sizeof(double), cudaMemcpyDeviceToHost, s), "bound D2H");
            CK(cudaStreamSynchronize(s), "bound sync");
        }
        // |contribution to a sky total| <= 2 max|beam| (|ga| + |gb|), one per sample
        // (an interpolated beam value is a convex combination of beam values);
        // |contribution to a beam total| <= 2 max|sky| (|ga| + |gb|), at most K per sample
        // (with the bilinear lookup a beam pixel is in the stencil of the pairs
        // within one ring and one pixel of it: at most 4 K, weights <= 1)
        const double ratio = (double)c->nside_sky / (double)c->nside_beam;
        double K2 = std::ceil(2.0 * ratio * ratio) + 4.0;  // sky pixels per beam pixel
        if (c->interp != PISCO_BEAM_NEAREST) K2 = 4.0 * K2 + 8.0;
        a.sky_scale = fixed_scale(2.0001 * h[1] * h[0]);
        a.beam_scale = fixed_scale(2.0001 * h[2] * h[0] * K2);
        if (d_gsky) {
            st = c->ensure((void**)&c->adj_sky_fx, &c->adj_sky_fx_cap, 8 * nsky, "adjoint sky accumulator");
            if (st != PISCO_OK) return st;
            CK(cudaMemsetAsync(c->adj_sky_fx, 0, 8 * nsky, s), "zero sky accumulator");
            a.gsky_fx = c->adj_sky_fx;
        }
        if (d_gbeam) {
            st = c->ensure((void**)&c->adj_beam_fx, &c->adj_beam_fx_cap, 8 * nbeam, "adjoint beam accumulator");
            if (st != PISCO_OK) return st;
            CK(cudaMemsetAsync(c->adj_beam_fx, 0, 8 * nbeam, s), "zero beam accumulator");
            a.gbeam_fx = c->adj_beam_fx;
        }
        take_plans();
        if (n > 0 && (a.sky_scale > 0.0 || a.beam_scale > 0.0 || pp))
            CK(launch_adjoint(a, c->sm_count, s, &nwarps), "adjoint launch");
        if (a.order) c->order_used(s);
        if (a.plans) c->plans_used(s);
        if (d_gsky)
            CK(launch_fixed_planes_to_float(c->adj_sky_fx, d_gsky, out_dtype == PISCO_FLOAT64, npix,
                                            a.sky_scale > 0.0 ? 1.0 / a.sky_scale : 0.0, s),
               "sky gradient");
        if (d_gbeam)
            CK(launch_fixed_to_float(c->adj_beam_fx, d_gbeam, out_dtype == PISCO_FLOAT64, nbeam,
                                     a.beam_scale > 0.0 ? 1.0 / a.beam_scale : 0.0, s),
               "beam gradient");
    }
    if (pp) {
        CK(launch_fold_params(pp->ppart, nwarps, pp->part + (size_t)kParamCols * pp->rows, s),
           "parameter sums");
        CK(launch_gauss_param_finish(pp->part, pp->rows + 1, pp->oc, pp->grad, s),
           "parameter gradient");
    }
    if (s != c->stream) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(c->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    return PISCO_OK;
}

}  // namespace

extern "C" {

pisco_status pisco_adjoint(pisco_ctx* c, const void* g_a, const void* g_b, pisco_dtype g_dtype,
                           void* gI, void* gQ, void* gU, void* gV, pisco_dtype out_dtype,
                           pisco_adjoint_mode mode)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (g_dtype != PISCO_FLOAT32 && g_dtype != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    if (out_dtype != PISCO_FLOAT32 && out_dtype != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    if (!c->nside_sky) return fail(c, PISCO_ERR_NOT_READY, "no sky set");
    const long n = c->nsamples;
    if (n > 0 && (!g_a || !g_b)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "TOD gradients are NULL");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    const size_t gsz = g_dtype == PISCO_FLOAT64 ? 8 : 4, osz = out_dtype == PISCO_FLOAT64 ? 8 : 4;
    const long long npix = 12LL * c->nside_sky * c->nside_sky;
    void *dg = nullptr, *dout = nullptr;
    CK(cudaMalloc(&dg, gsz * 2 * (size_t)std::max<long>(n, 1)), "adjoint input staging");
    cudaError_t e = cudaMalloc(&dout, osz * 4 * (size_t)npix);
    if (e != cudaSuccess) {
        cudaFree(dg);
        return cuda_fail(c, e, "adjoint output staging");
    }
    struct Free {
        void* a;
        void* b;
        ~Free() {
            cudaFree(a);
            cudaFree(b);
        }
    } guard{dg, dout};
    if (n > 0) {
        CK(cudaMemcpyAsync(dg, g_a, gsz * n, cudaMemcpyHostToDevice, c->stream), "g_a H2D");
        CK(cudaMemcpyAsync((char*)dg + gsz * n, g_b, gsz * n, cudaMemcpyHostToDevice, c->stream), "g_b H2D");
    }
    st = pisco_adjoint_device(c, 0, n, dg, (char*)dg + gsz * n, g_dtype, dout, nullptr, out_dtype, mode,
                              c->stream);
    if (st != PISCO_OK) return st;
    std::vector<char> h(osz * 4 * (size_t)npix);
    CK(cudaMemcpyAsync(h.data(), dout, h.size(), cudaMemcpyDeviceToHost, c->stream), "gradient D2H");
    st = c->check_device();
    if (st != PISCO_OK) return st;
    void* planes[4] = {gI, gQ, gU, gV};
    for (int k = 0; k < 4; ++k) {
        if (!planes[k]) continue;
        for (long long i = 0; i < npix; ++i)
            std::memcpy((char*)planes[k] + osz * i, h.data() + osz * (4 * i + k), osz);
    }
    return PISCO_OK;
}

}  // extern "C"
