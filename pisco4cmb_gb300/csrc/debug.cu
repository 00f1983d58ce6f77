// debug.cu -- diagnostic entry points (no reference counterpart): the
// per-pair decisions of each form, and HEALPix RING pix2ang / ang2pix /
// get_interpol run on the device for whole arrays.
//
// pisco_debug_pairs records what the forward kernels decide for every
// (sample, disc pixel) pair: the disc itself, the beam pixel of the nearest
// lookup or the four-pixel stencil of the bilinear one, and the polarization
// angle.  The TUNED record runs the TUNED per-sample body itself
// (tuned::sample with a recording action in place of the sky gather); the
// PLAIN record runs the PLAIN form's disc walk and per-pair functions.  The
// reference checks the same decisions with its own device tests
// (tests/cudaConvolution/test_sky_to_beam_matching_kernel.cu:188-216,
// tests/cudaHealpix/test_pix2ang.cu:80-114, test_interpol.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/pisco_gb300.h"
#include "ctx.h"
#include "tuned_core.cuh"

using namespace pisco;

namespace pisco {
void set_null_ctx_error(const char* msg);  // capi.cu
}

namespace {

constexpr int kTW = PISCO_TUNED_WARPS;

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

// Action of tuned::sample that writes each pair's decisions instead of
// gathering the sky.
struct Record {
    static constexpr bool kSums = false;
    static constexpr bool kStencil = true;
    PairDump d;
    unsigned int* err;
    long long cur;  // position of the sample of the main pass

    __device__ __forceinline__ float4 fetch(int) const { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ __forceinline__ void stash(tuned::Pend&) const {}
    __device__ __forceinline__ void put(long long j, int pix, int bp, float c2, float s2, int flags,
                                        const int* px, const float* w) const
    {
        const long long k = d.offset[j] + (long long)atomicAdd(&d.fill[j], 1u);
        if (k >= d.offset[j + 1]) {
            tuned::record(err, kCheckDump);
            return;
        }
        d.sample[k] = (int)j;
        d.sky_pix[k] = pix;
        d.beam_pix[k] = bp;
        d.c2[k] = c2;
        d.s2[k] = s2;
        d.chi[k] = CUDART_NAN;
        d.flags[k] = flags;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            d.st_pix[4 * k + i] = px ? px[i] : -1;
            d.st_w[4 * k + i] = px ? (double)w[i] : 0.0;
        }
    }
    __device__ __forceinline__ void pair(int pix, const float4&, const F8&, int bp, float c2,
                                         float s2) const
    {
        put(cur, pix, bp, c2, s2, 0, nullptr, nullptr);
    }
    __device__ __forceinline__ void deferred(const tuned::Pend& P, int pix, const F8&, int bp,
                                            float c2, float s2, float&, float&) const
    {
        put(P.idx, pix, bp, c2, s2, kPairRedone, nullptr, nullptr);
    }
    __device__ __forceinline__ void pair_stencil(int pix, const float4&, const int px[4],
                                                const float w[4], float c2, float s2) const
    {
        put(cur, pix, -1, c2, s2, 0, px, w);
    }
    __device__ __forceinline__ void deferred_stencil(const tuned::Pend& P, int pix, const int px[4],
                                                    const float w[4], float c2, float s2) const
    {
        put(P.idx, pix, -1, c2, s2, kPairRedone, px, w);
    }
    __device__ __forceinline__ void outside(int pix, int bp) const
    {
        put(cur, pix, bp, 0.0f, 0.0f, kPairOutside, nullptr, nullptr);
    }
    __device__ __forceinline__ void outside_deferred(const tuned::Pend& P, int pix, int bp) const
    {
        put(P.idx, pix, bp, 0.0f, 0.0f, kPairOutside | kPairRedone, nullptr, nullptr);
    }
};

template <bool kBil>
__global__ void __launch_bounds__(kTW * 32, PISCO_TUNED_MINB) tuned_dump_kernel(FwdArgs a, PairDump d)
{
    __shared__ tuned::WarpSmem sm[kTW];
    const int lane = threadIdx.x & 31;
    tuned::WarpSmem& S = sm[threadIdx.x >> 5];
    const Hpx hs = hpx_make(a.nside_sky);
    const Hpx hb = hpx_make(a.nside_beam);
    const tuned::Beam B = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    const long long gw = (long long)blockIdx.x * kTW + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kTW;
    unsigned long long nfall = 0, npairs = 0;
    float cmax = 0.0f;
    Record rec{d, a.err, 0};
    tuned::Queue Q{0, 0};
    for (long long j = gw; j < a.n; j += nw) {
        const long long s = a.begin + j;
        rec.cur = j;
        const tuned::Out o{nullptr, nullptr, j, 0};
        tuned::sample<false, kBil>(hs, a.rings, hb, B, a.ra[s], a.dec[s], a.pa[s], o, S, Q, lane,
                                   a.err, rec, nfall, cmax, npairs);
    }
    tuned::flush<kBil>(hs, S, Q, lane, a.err, rec);
}

// Disc size of every sample (HEALPix query_disc's FP64 edge formula).
__global__ void disc_sizes_kernel(int nside_sky, double rho_max, long long begin, long long n,
                                  const double* ra, const double* dec, long long* sizes)
{
    const int lane = threadIdx.x & 31;
    const Hpx hs = hpx_make(nside_sky);
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long j = gw; j < n; j += nw) {
        const long long s = begin + j;
        long long mine = 0;
        if (isfinite(ra[s]) && isfinite(dec[s])) {
            const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, dec[s]), ra[s], rho_max);
            for (long long r0 = P.full_lo; r0 <= P.full_hi; r0 += 32) {
                const long long ring = r0 + lane;
                if (ring <= P.full_hi) {
                    const RingSpan sp = disc_ring(hs, P, ring);
                    mine += sp.n1 + sp.n2;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
        if (lane == 0) sizes[j] = mine;
    }
}

__global__ void pix2ang_kernel(int nside, long long n, const long long* pix, double* th, double* ph,
                               unsigned int* bad)
{
    const Hpx h = hpx_make(nside);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long p = pix[i];
        if (p < 0 || p >= h.npix) {
            atomicCAS(bad, 0u, 1u);
            th[i] = ph[i] = CUDART_NAN;
            continue;
        }
        pix2ang(h, p, &th[i], &ph[i]);
    }
}

__global__ void ang2pix_kernel(int nside, long long n, const double* th, const double* ph,
                               long long* pix, unsigned int* bad)
{
    const Hpx h = hpx_make(nside);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double t = th[i], f = ph[i];
        if (!(t >= 0.0 && t <= kPi && isfinite(f))) {
            atomicCAS(bad, 0u, 1u);
            pix[i] = -1;
            continue;
        }
        pix[i] = ang2pix(h, t, f);
    }
}

__global__ void get_interpol_kernel(int nside, long long n, const double* th, const double* ph,
                                    long long* pix4, double* w4, unsigned int* bad)
{
    const Hpx h = hpx_make(nside);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double t = th[i], f = ph[i];
        if (!(t >= 0.0 && t <= kPi && isfinite(f))) {
            atomicCAS(bad, 0u, 1u);
            for (int k = 0; k < 4; ++k) {
                pix4[4 * i + k] = -1;
                w4[4 * i + k] = CUDART_NAN;
            }
            continue;
        }
        int64_t p[4];
        double w[4];
        get_interpol(h, t, f, p, w);
        for (int k = 0; k < 4; ++k) {
            pix4[4 * i + k] = p[k];
            w4[4 * i + k] = w[k];
        }
    }
}

template <class K>
int resident_blocks(K kernel, int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    return nb;
}

// One-shot device arrays of a diagnostic call, freed on every return path.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t get(T** p, size_t count)
    {
        void* v = nullptr;
        const cudaError_t e = cudaMalloc(&v, sizeof(T) * (count > 0 ? count : 1));
        if (e == cudaSuccess) ptrs.push_back(v);
        *p = (T*)v;
        return e;
    }
};

// The element-wise HEALPix entry points need no context: they run on the
// calling thread's current device and stream.
pisco_status hpx_args(int nside, long long n, bool ok_ptrs)
{
    if (nside < 1 || nside > 8192) {
        set_null_ctx_error("nside must be in [1, 8192]");
        return PISCO_ERR_INVALID_ARGUMENT;
    }
    if (n < 0 || (n > 0 && !ok_ptrs)) {
        set_null_ctx_error("n must be >= 0 and the arrays not NULL");
        return PISCO_ERR_INVALID_ARGUMENT;
    }
    return PISCO_OK;
}

pisco_status hpx_finish(cudaError_t e, unsigned int* bad, cudaStream_t st, const char* what)
{
    unsigned int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(bad);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_null_ctx_error((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
        return PISCO_ERR_CUDA;
    }
    if (h) {
        set_null_ctx_error((std::string(what) + ": an input lies outside the valid range").c_str());
        return PISCO_ERR_INVALID_ARGUMENT;
    }
    return PISCO_OK;
}

int hpx_grid(long long n)
{
    const long long b = (n + 255) / 256;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

namespace pisco {

cudaError_t launch_dump_tuned(const FwdArgs& a, const PairDump& d, int sm_count, cudaStream_t st)
{
    if (a.n <= 0) return cudaSuccess;
    const int threads = kTW * 32;
    const long long need = (a.n + kTW - 1) / kTW;
    if (a.interp == 1) {
        long long blocks = (long long)sm_count * resident_blocks(tuned_dump_kernel<true>, threads);
        tuned_dump_kernel<true><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, d);
    } else {
        long long blocks = (long long)sm_count * resident_blocks(tuned_dump_kernel<false>, threads);
        tuned_dump_kernel<false><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, d);
    }
    return cudaGetLastError();
}

}  // namespace pisco

extern "C" {

pisco_status pisco_debug_pairs(pisco_ctx* c, pisco_form form, long begin, long n,
                               const pisco_pair_dump* out, long long* npairs)
{
    if (!c || !npairs) return PISCO_ERR_INVALID_ARGUMENT;
    if (!c->sky32 || !c->nside_sky || !c->beam32 || !c->nside_beam)
        return fail(c, PISCO_ERR_NOT_READY, "sky and beam required");
    if (c->nsamples < 0 || (!c->ra && c->nsamples > 0)) return fail(c, PISCO_ERR_NOT_READY, "no scan set");
    if (begin < 0 || n < 0 || begin + n > c->nsamples)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sample range outside the scan");
    if (form != PISCO_FORM_PLAIN && form != PISCO_FORM_TUNED && form != PISCO_FORM_FP64)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad form");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = c->stream;
    Scratch scr;
    long long* sizes = nullptr;
    CK(scr.get(&sizes, (size_t)n + 1), "disc sizes");
    if (n > 0) {
        disc_sizes_kernel<<<(int)std::min<long long>((n + 7) / 8, 4096), 256, 0, s>>>(
            c->nside_sky, c->rho_max, begin, n, c->ra, c->dec, sizes);
        CK(cudaGetLastError(), "disc sizes");
    }
    std::vector<long long> off((size_t)n + 1, 0);
    CK(cudaMemcpyAsync(off.data() + 1, sizes, sizeof(long long) * n, cudaMemcpyDeviceToHost, s),
       "disc sizes D2H");
    CK(cudaStreamSynchronize(s), "disc sizes");
    for (long j = 0; j < n; ++j) off[j + 1] += off[j];
    const long long total = off[n];
    *npairs = total;
    if (!out) return PISCO_OK;  // size query
    if (out->capacity < total)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT,
                    "pair record capacity " + std::to_string(out->capacity) + " below the " +
                        std::to_string(total) + " disc pairs of the range");
    PairDump d{};
    long long* d_off = nullptr;
    CK(scr.get(&d_off, (size_t)n + 1), "pair record");
    CK(scr.get(&d.fill, (size_t)n), "pair record");
    CK(scr.get(&d.sample, (size_t)total), "pair record");
    CK(scr.get(&d.sky_pix, (size_t)total), "pair record");
    CK(scr.get(&d.beam_pix, (size_t)total), "pair record");
    CK(scr.get(&d.c2, (size_t)total), "pair record");
    CK(scr.get(&d.s2, (size_t)total), "pair record");
    CK(scr.get(&d.chi, (size_t)total), "pair record");
    CK(scr.get(&d.flags, (size_t)total), "pair record");
    CK(scr.get(&d.st_pix, 4 * (size_t)total), "pair record");
    CK(scr.get(&d.st_w, 4 * (size_t)total), "pair record");
    d.offset = d_off;
    CK(cudaMemcpyAsync(d_off, off.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, s),
       "offsets H2D");
    CK(cudaMemsetAsync(d.fill, 0, sizeof(unsigned int) * (n > 0 ? n : 1), s), "fill");
    CK(cudaMemsetAsync(d.sample, 0xff, sizeof(int) * (total > 0 ? total : 1), s), "record init");
    CK(cudaMemsetAsync(d.st_pix, 0xff, 4 * sizeof(int) * (total > 0 ? total : 1), s), "record init");
    CK(cudaMemsetAsync(d.st_w, 0, 4 * sizeof(double) * (total > 0 ? total : 1), s), "record init");
    FwdArgs a{};
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
    a.interp = (int)c->interp;
    a.err = c->d_err;
    a.fallbacks = c->d_fallbacks;
    cudaError_t e;
    if (form == PISCO_FORM_TUNED && tuned_supported(c->nside_beam, (int)c->npix_beam, c->rho_max))
        e = launch_dump_tuned(a, d, c->sm_count, s);
    else  // PLAIN and FP64 take the same per-pair decisions
        e = launch_dump_plain(a, d, c->sm_count, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "pair record launch");
    auto back = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        if (!dst || bytes == 0) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
    };
    const size_t T = (size_t)total;
    CK(back(out->sample, d.sample, sizeof(int) * T), "record D2H");
    CK(back(out->sky_pix, d.sky_pix, sizeof(int) * T), "record D2H");
    CK(back(out->beam_pix, d.beam_pix, sizeof(int) * T), "record D2H");
    CK(back(out->c2chi, d.c2, sizeof(float) * T), "record D2H");
    CK(back(out->s2chi, d.s2, sizeof(float) * T), "record D2H");
    CK(back(out->chi, d.chi, sizeof(double) * T), "record D2H");
    CK(back(out->flags, d.flags, sizeof(int) * T), "record D2H");
    CK(back(out->stencil_pix, d.st_pix, 4 * sizeof(int) * T), "record D2H");
    CK(back(out->stencil_w, d.st_w, 4 * sizeof(double) * T), "record D2H");
    CK(cudaStreamSynchronize(s), "pair record");
    return c->check_device();
}

pisco_status pisco_hpx_pix2ang_device(int nside, long long n, const long long* d_pix,
                                      double* d_theta, double* d_phi, void* stream)
{
    set_null_ctx_error("");
    pisco_status st = hpx_args(nside, n, d_pix && d_theta && d_phi);
    if (st != PISCO_OK || n == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int* bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, sizeof(unsigned int));
    if (e != cudaSuccess) return hpx_finish(e, nullptr, s, "pix2ang");
    e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        pix2ang_kernel<<<hpx_grid(n), 256, 0, s>>>(nside, n, d_pix, d_theta, d_phi, bad);
        e = cudaGetLastError();
    }
    return hpx_finish(e, bad, s, "pix2ang");
}

pisco_status pisco_hpx_ang2pix_device(int nside, long long n, const double* d_theta,
                                      const double* d_phi, long long* d_pix, void* stream)
{
    set_null_ctx_error("");
    pisco_status st = hpx_args(nside, n, d_pix && d_theta && d_phi);
    if (st != PISCO_OK || n == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int* bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, sizeof(unsigned int));
    if (e != cudaSuccess) return hpx_finish(e, nullptr, s, "ang2pix");
    e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        ang2pix_kernel<<<hpx_grid(n), 256, 0, s>>>(nside, n, d_theta, d_phi, d_pix, bad);
        e = cudaGetLastError();
    }
    return hpx_finish(e, bad, s, "ang2pix");
}

pisco_status pisco_hpx_get_interpol_device(int nside, long long n, const double* d_theta,
                                           const double* d_phi, long long* d_pix4, double* d_w4,
                                           void* stream)
{
    set_null_ctx_error("");
    pisco_status st = hpx_args(nside, n, d_pix4 && d_theta && d_phi && d_w4);
    if (st != PISCO_OK || n == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int* bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, sizeof(unsigned int));
    if (e != cudaSuccess) return hpx_finish(e, nullptr, s, "get_interpol");
    e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
        get_interpol_kernel<<<hpx_grid(n), 256, 0, s>>>(nside, n, d_theta, d_phi, d_pix4, d_w4, bad);
        e = cudaGetLastError();
    }
    return hpx_finish(e, bad, s, "get_interpol");
}

}  // extern "C"
