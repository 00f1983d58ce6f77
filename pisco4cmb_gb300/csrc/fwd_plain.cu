// fwd_plain.cu -- PLAIN and FP64 forward kernels, plus small helpers.
//
// PLAIN reproduces the reference per-pair chain on the GPU
// (src/Convolver/convolver.cpp:112-221; the GPU pair of kernels
// src/GpuConvolver/cuda/cudaConv2.cu:59-240 fused into one): for each
// sample, the disc of sky pixels within rhoMax (HEALPix query_disc, here on
// the device instead of the host OpenMP loop at gpuconvolver.cu:392-425),
// and for each disc pixel: pix2ang -> rho/sigma/chi -> nearest (or
// bilinear) beam pixel -> polarized multiply-accumulate of sky IQUV with
// the beam a and b IQUV.  Geometry is FP64, the sky x beam products FP32
// (float beams and c2chi/s2chi as in convolver.cpp:122-123,150-165) and the
// accumulation FP64.  FP64 makes every input, product and sum FP64.
//
// Work split: one warp per sample (no atomics, no host disc lists, no
// padded pair matrices).  The warp evaluates 32 disc rings at a time, one
// per lane, flattens their pixel ranges with a warp scan and strides the
// pairs across lanes; the per-lane sums are combined by a fixed shuffle
// tree, so every output is bit-for-bit reproducible.
#include <math_constants.h>

#include "hpx.cuh"
#include "internal.h"

namespace pisco {
namespace {

constexpr int kWarps = 8;
constexpr unsigned kFull = 0xffffffffu;

struct RingBatch {
    int incl[32];
    int cnt[32];
    int n1[32];
    long long s1[32];
    long long s2[32];
};

__device__ __forceinline__ void record(unsigned int* err, unsigned int code)
{
    if (err) atomicCAS(err, 0u, code);
}

// Pixel at flattened position t of a ring batch: the first lane whose
// inclusive count exceeds t owns it.
__device__ __forceinline__ long long batch_pixel(const RingBatch& w, int t)
{
    int lo = 0, hi = 31;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (w.incl[mid] > t) hi = mid;
        else lo = mid + 1;
    }
    int u = t - (w.incl[lo] - w.cnt[lo]);
    return (u < w.n1[lo]) ? w.s1[lo] + u : w.s2[lo] + (u - w.n1[lo]);
}

// Renormalised 4-point bilinear beam value (weights of stencil pixels that
// lie outside the stored partial beam map are dropped).
template <class LoadA>
__device__ __forceinline__ bool bilinear(const Hpx& hb, int npb, double rho, double sig,
                                         LoadA load, double va[4], double vb[4])
{
    int64_t px[4];
    double w[4];
    get_interpol(hb, rho, sig, px, w);
    double ws = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) va[k] = vb[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (px[i] < 0 || px[i] >= npb) continue;
        ws += w[i];
        double a[4], b[4];
        load(px[i], a, b);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            va[k] += a[k] * w[i];
            vb[k] += b[k] * w[i];
        }
    }
    if (!(ws > 0.0)) return false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        va[k] /= ws;
        vb[k] /= ws;
    }
    return true;
}

template <bool F64>
__device__ __forceinline__ void pair_accumulate(const FwdArgs& a, const Hpx& hs, const Hpx& hb,
                                                long long pix, double ra, double dec,
                                                double psi, double& acc_a, double& acc_b)
{
    double rho, sig, chi;
    double va[4], vb[4];
    if (a.interp == 0) {
        long long bp = pair_beam_pixel(hs, hb, pix, ra, dec, psi, &rho, &sig, &chi);
        if (bp >= a.npix_beam) return;
        if (bp < 0) {
            record(a.err, kCheckBeamIndex);
            return;
        }
        if (F64) {
            const D8 B = a.beam64[bp];
            va[0] = B.a.x; va[1] = B.a.y; va[2] = B.a.z; va[3] = B.a.w;
            vb[0] = B.b.x; vb[1] = B.b.y; vb[2] = B.b.z; vb[3] = B.b.w;
        } else {
            const F8 B = a.beam32[bp];
            va[0] = B.a.x; va[1] = B.a.y; va[2] = B.a.z; va[3] = B.a.w;
            vb[0] = B.b.x; vb[1] = B.b.y; vb[2] = B.b.z; vb[3] = B.b.w;
        }
    } else {
        double th, ph;
        pix2ang(hs, pix, &th, &ph);
        rho_sigma_chi(ra, dec, psi, ph, PD_SUB(PD_DIV(kPi, 2.0), th), &rho, &sig, &chi);
        bool ok;
        if (F64) {
            ok = bilinear(hb, a.npix_beam, rho, sig,
                          [&](int64_t p, double* x, double* y) {
                              const D8 B = a.beam64[p];
                              x[0] = B.a.x; x[1] = B.a.y; x[2] = B.a.z; x[3] = B.a.w;
                              y[0] = B.b.x; y[1] = B.b.y; y[2] = B.b.z; y[3] = B.b.w;
                          },
                          va, vb);
        } else {
            ok = bilinear(hb, a.npix_beam, rho, sig,
                          [&](int64_t p, double* x, double* y) {
                              const F8 B = a.beam32[p];
                              x[0] = B.a.x; x[1] = B.a.y; x[2] = B.a.z; x[3] = B.a.w;
                              y[0] = B.b.x; y[1] = B.b.y; y[2] = B.b.z; y[3] = B.b.w;
                          },
                          va, vb);
            if (ok) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {  // the interpolated beam is stored as float
                    va[k] = (double)(float)va[k];
                    vb[k] = (double)(float)vb[k];
                }
            }
        }
        if (!ok) return;
    }
    if (F64) {
        const D4 S = a.sky64[pix];
        double c2 = cos(2.0 * chi), s2 = sin(2.0 * chi);
        acc_a += S.x * va[0] + S.y * (va[1] * c2 - va[2] * s2) +
                 S.z * (va[2] * c2 + va[1] * s2) + S.w * va[3];
        acc_b += S.x * vb[0] + S.y * (-vb[1] * c2 + vb[2] * s2) +
                 S.z * (-vb[2] * c2 - vb[1] * s2) + S.w * vb[3];
    } else {
        const float4 S = a.sky32[pix];
        float c2 = (float)cos(2.0 * chi), s2 = (float)sin(2.0 * chi);
        float a0 = (float)va[0], a1 = (float)va[1], a2 = (float)va[2], a3 = (float)va[3];
        float b0 = (float)vb[0], b1 = (float)vb[1], b2 = (float)vb[2], b3 = (float)vb[3];
        float ta = S.x * a0 + S.y * (a1 * c2 - a2 * s2) + S.z * (a2 * c2 + a1 * s2) + S.w * a3;
        float tb = S.x * b0 + S.y * (-b1 * c2 + b2 * s2) + S.z * (-b2 * c2 - b1 * s2) + S.w * b3;
        acc_a += (double)ta;
        acc_b += (double)tb;
    }
}

// The disc of one sample: 32 rings per step, one per lane (HEALPix
// query_disc's FP64 edge formula), flattened by a warp scan, the pairs
// strided across lanes; f(pix) for every disc pixel.
template <class F>
__device__ __forceinline__ void walk_disc(const Hpx& hs, const DiscPlan& P, RingBatch& W, int lane,
                                          unsigned int* err, F&& f)
{
    for (long long r0 = P.full_lo; r0 <= P.full_hi; r0 += 32) {
        const long long ring = r0 + lane;
        RingSpan sp = {0, 0, 0, 0};
        if (ring <= P.full_hi) sp = disc_ring(hs, P, ring);
        const int cnt = (int)(sp.n1 + sp.n2);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        W.incl[lane] = incl;
        W.cnt[lane] = cnt;
        W.n1[lane] = (int)sp.n1;
        W.s1[lane] = sp.start1;
        W.s2[lane] = sp.start2;
        __syncwarp();
        for (int t = lane; t < total; t += 32) {
            const long long pix = batch_pixel(W, t);
            if (pix < 0 || pix >= hs.npix) {
                record(err, kCheckSkyIndex);
                continue;
            }
            f(pix);
        }
        __syncwarp();
    }
}

template <bool F64>
__global__ void __launch_bounds__(kWarps * 32) plain_kernel(FwdArgs a)
{
    __shared__ RingBatch sh[kWarps];
    const int lane = threadIdx.x & 31;
    RingBatch& W = sh[threadIdx.x >> 5];
    const Hpx hs = hpx_make(a.nside_sky);
    const Hpx hb = hpx_make(a.nside_beam);
    const long long gw = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kWarps;
    for (long long i = gw; i < a.n; i += nw) {
        const long long j = a.order ? (long long)a.order[i] : i;  // sample of position i
        const long long s = a.begin + j;
        const double ra = a.ra[s], dec = a.dec[s], psi = -a.pa[s];
        if (!(isfinite(ra) && isfinite(dec) && isfinite(psi))) {
            // non-finite pointing: NaN out (never let it reach the ring loop bounds)
            if (lane == 0) {
                if (a.out_f64) {
                    if (a.out_a) ((double*)a.out_a)[j] = CUDART_NAN;
                    if (a.out_b) ((double*)a.out_b)[j] = CUDART_NAN;
                } else {
                    if (a.out_a) ((float*)a.out_a)[j] = CUDART_NAN_F;
                    if (a.out_b) ((float*)a.out_b)[j] = CUDART_NAN_F;
                }
            }
            continue;
        }
        const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, dec), ra, a.rho_max);
        double acc_a = 0.0, acc_b = 0.0;
        walk_disc(hs, P, W, lane, a.err, [&](long long pix) {
            pair_accumulate<F64>(a, hs, hb, pix, ra, dec, psi, acc_a, acc_b);
        });
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc_a += __shfl_xor_sync(kFull, acc_a, o);
            acc_b += __shfl_xor_sync(kFull, acc_b, o);
        }
        if (lane == 0) {
            if (a.out_f64) {
                if (a.out_a) ((double*)a.out_a)[j] = acc_a;
                if (a.out_b) ((double*)a.out_b)[j] = acc_b;
            } else {
                if (a.out_a) ((float*)a.out_a)[j] = (float)acc_a;
                if (a.out_b) ((float*)a.out_b)[j] = (float)acc_b;
            }
        }
    }
}

// Record of the PLAIN form's decisions (pisco_debug_pairs): the same disc
// walk and per-pair functions as plain_kernel, each pair written to its
// sample's entries instead of accumulated.
__global__ void __launch_bounds__(kWarps * 32) plain_dump_kernel(FwdArgs a, PairDump d)
{
    __shared__ RingBatch sh[kWarps];
    const int lane = threadIdx.x & 31;
    RingBatch& W = sh[threadIdx.x >> 5];
    const Hpx hs = hpx_make(a.nside_sky);
    const Hpx hb = hpx_make(a.nside_beam);
    const long long gw = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kWarps;
    for (long long j = gw; j < a.n; j += nw) {
        const long long s = a.begin + j;
        const double ra = a.ra[s], dec = a.dec[s], psi = -a.pa[s];
        if (!(isfinite(ra) && isfinite(dec) && isfinite(psi))) continue;
        const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, dec), ra, a.rho_max);
        walk_disc(hs, P, W, lane, a.err, [&](long long pix) {
            const long long k = d.offset[j] + (long long)atomicAdd(&d.fill[j], 1u);
            if (k >= d.offset[j + 1]) {
                record(a.err, kCheckDump);
                return;
            }
            double rho, sig, chi;
            int flags = 0;
            if (a.interp == 0) {
                const long long bp = pair_beam_pixel(hs, hb, pix, ra, dec, psi, &rho, &sig, &chi);
                d.beam_pix[k] = (int)bp;
                if (bp < 0 || bp >= a.npix_beam) flags |= kPairOutside;
            } else {
                double th, ph;
                pix2ang(hs, pix, &th, &ph);
                rho_sigma_chi(ra, dec, psi, ph, PD_SUB(PD_DIV(kPi, 2.0), th), &rho, &sig, &chi);
                int64_t px[4];
                double w[4];
                get_interpol(hb, rho, sig, px, w);
                bool any = false;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    d.st_pix[4 * k + i] = (int)px[i];
                    d.st_w[4 * k + i] = w[i];
                    any |= px[i] >= 0 && px[i] < a.npix_beam;
                }
                d.beam_pix[k] = -1;
                if (!any) flags |= kPairOutside;
            }
            d.sample[k] = (int)j;
            d.sky_pix[k] = (int)pix;
            d.chi[k] = chi;
            d.c2[k] = (float)cos(2.0 * chi);
            d.s2[k] = (float)sin(2.0 * chi);
            d.flags[k] = flags;
        });
    }
}

__global__ void __launch_bounds__(256) count_kernel(int nside_sky, double rho_max, long long n,
                                                    const double* ra, const double* dec,
                                                    unsigned long long* total)
{
    const int lane = threadIdx.x & 31;
    const Hpx hs = hpx_make(nside_sky);
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long mine = 0;
    for (long long s = gw; s < n; s += nw) {
        if (!(isfinite(ra[s]) && isfinite(dec[s]))) continue;
        const DiscPlan P = disc_plan(hs, PD_SUB(kHalfPi, dec[s]), ra[s], rho_max);
        for (long long r0 = P.full_lo; r0 <= P.full_hi; r0 += 32) {
            const long long ring = r0 + lane;
            if (ring <= P.full_hi) {
                RingSpan sp = disc_ring(hs, P, ring);
                mine += (unsigned long long)(sp.n1 + sp.n2);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(kFull, mine, o);
    if (lane == 0 && mine) atomicAdd(total, mine);
}

__global__ void widen_sky_kernel(const float4* in, D4* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float4 v = in[i];
        out[i] = D4{v.x, v.y, v.z, v.w};
    }
}

__global__ void widen_beam_kernel(const F8* in, D8* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        F8 v = in[i];
        out[i] = D8{D4{v.a.x, v.a.y, v.a.z, v.a.w}, D4{v.b.x, v.b.y, v.b.z, v.b.w}};
    }
}

__global__ void narrow_sky_kernel(const D4* in, float4* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        D4 v = in[i];
        out[i] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
    }
}

__global__ void f32_to_f64_kernel(const float* in, double* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
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

}  // namespace

cudaError_t launch_forward_plain(const FwdArgs& a, bool f64, int sm_count, cudaStream_t st)
{
    if (a.n <= 0) return cudaSuccess;
    const int threads = kWarps * 32;
    if (f64) {
        long long blocks = (long long)sm_count * resident_blocks(plain_kernel<true>, threads);
        long long need = (a.n + kWarps - 1) / kWarps;
        plain_kernel<true><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a);
    } else {
        long long blocks = (long long)sm_count * resident_blocks(plain_kernel<false>, threads);
        long long need = (a.n + kWarps - 1) / kWarps;
        plain_kernel<false><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_dump_plain(const FwdArgs& a, const PairDump& d, int sm_count, cudaStream_t st)
{
    if (a.n <= 0) return cudaSuccess;
    const int threads = kWarps * 32;
    long long blocks = (long long)sm_count * resident_blocks(plain_dump_kernel, threads);
    long long need = (a.n + kWarps - 1) / kWarps;
    plain_dump_kernel<<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, d);
    return cudaGetLastError();
}

cudaError_t launch_count_pairs(int nside_sky, double rho_max, long long n, const double* ra,
                               const double* dec, unsigned long long* total, int sm_count,
                               cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    long long blocks = (long long)sm_count * resident_blocks(count_kernel, 256);
    long long need = (n + 7) / 8;
    count_kernel<<<(int)(blocks < need ? blocks : need), 256, 0, st>>>(nside_sky, rho_max, n, ra,
                                                                        dec, total);
    return cudaGetLastError();
}

cudaError_t launch_widen_sky(const float4* in, D4* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    widen_sky_kernel<<<1024, 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_widen_beam(const F8* in, D8* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    widen_beam_kernel<<<256, 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_narrow_sky(const D4* in, float4* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    narrow_sky_kernel<<<1024, 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float* in, double* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    f32_to_f64_kernel<<<1024, 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace pisco
