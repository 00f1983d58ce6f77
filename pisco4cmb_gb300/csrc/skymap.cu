// skymap.cu -- the binned map-maker on the GPU: TOD back to I, Q, U maps.
//
// Replaces SkyMap (src/SkyMap/skymap.hpp, skymap.cpp:68-231), the consumer
// of the convolver's TOD.  For every TOD value d of detector `det` at sample
// s, with pixel p = ang2pix(pi/2 - dec, ra) and psi = -(pol[det] + pa):
//   AtD[p] += (d, c d, s d),  AtA[p] += [1 c s; c cc cs; s cs ss],
// c = cos 2psi, s = sin 2psi (skymap.cpp:85-122); then per pixel
// AtA x = AtD is solved for (I, Q, U) with LAPACK's dgesv when the pixel has
// at least 3 hits (skymap.cpp:134-231).
//
// GB300 layout of the work.  Per call: one thread per TOD value computes its
// pixel (the FP64 HEALPix ang2pix of hpx.cuh) and (c, s, d) in FP64; a stable
// radix sort by pixel (CUB) groups the values of a pixel while keeping them
// in the reference's (detector, sample) order; one thread per occupied pixel
// then adds them sequentially, in FP64 without contraction, onto the
// pixel's running totals.  Each total therefore receives exactly the
// reference's additions in the reference's order (bit-identical up to the
// last-ulp differences of CUDA's and the host's cos/sin), with no atomics
// and run-to-run determinism.  The solve restates the reference LAPACK
// dgesv (dgetf2 + dgetrs) per pixel in non-contracted FP64.
//
// Deliberate difference: the reference's constructor leaves AtA and AtD
// uninitialised (the zeroing loop at skymap.cpp:25-36 is commented out);
// here they start at zero.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <new>
#include <cstring>
#include <string>

#include "../../include/pisco_gb300.h"
#include "hpx.cuh"

using namespace pisco;

// Per-pixel running totals, structure of arrays (9 x npix doubles): the six
// distinct entries of the symmetric AtA and the three of AtD.
enum MapAcc { kN = 0, kC, kS, kCC, kCS, kSS, kD, kCD, kSD, kAcc };

struct pisco_map {
    int device = 0;
    int nside = 0;
    long long npix = 0;
    cudaStream_t stream = nullptr;
    std::string error;
    double* acc = nullptr;  // kAcc x npix
    float* iqu = nullptr;   // 3 x npix
    int* hits = nullptr;
    bool solved = false;
    // per-call scratch, grown as needed
    void* buf[10] = {};
    size_t cap[10] = {};
    ~pisco_map();
};

namespace {

enum Scratch { kKeys = 0, kKeys2, kPos, kPos2, kRec, kUniq, kCount, kOff, kRuns, kTmp };

// (c, s, d) of one TOD value.
struct alignas(8) MapRec {
    double c, s, d;
};

pisco_status map_fail(pisco_map* m, pisco_status s, const std::string& msg)
{
    if (m) m->error = msg;
    return s;
}

#define MCK(call, what)                                                                           \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            cudaGetLastError();                                                                   \
            return map_fail(m, e_ == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY          \
                                                               : PISCO_ERR_CUDA,                  \
                            std::string(what) + ": " + cudaGetErrorString(e_));                   \
        }                                                                                         \
    } while (0)

pisco_status grow(pisco_map* m, int k, size_t bytes)
{
    if (m->cap[k] >= bytes && m->buf[k]) return PISCO_OK;
    if (m->buf[k]) {
        MCK(cudaStreamSynchronize(m->stream), "sync before realloc");
        cudaFree(m->buf[k]);
        m->buf[k] = nullptr;
        m->cap[k] = 0;
    }
    MCK(cudaMalloc(&m->buf[k], bytes), "map scratch");
    m->cap[k] = bytes;
    return PISCO_OK;
}

template <class T>
__global__ void map_keys_kernel(long long total, long long ns, int nside, const T* ra, const T* dec,
                                const T* pa, const T* data, const float* pol, int* keys,
                                int* pos, MapRec* rec, unsigned int* bad)
{
    const Hpx h = hpx_make(nside);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int det = (int)(e / ns);
        const double r = (double)ra[e], dc = (double)dec[e];
        // the reference's arithmetic (skymap.cpp:85-101), FP64, no contraction
        const double psi = -PD_ADD((double)pol[det], (double)pa[e]);
        const double twopsi = PD_MUL(2.0, psi);
        double s, c;
        sincos(twopsi, &s, &c);
        const double theta = PD_SUB(kHalfPi, dc);
        long long p = h.npix;  // sentinel: sorted last, never accumulated
        if (isfinite(r) && isfinite(theta) && theta >= 0.0 && theta <= kPi) p = ang2pix(h, theta, r);
        if (p < 0 || p >= h.npix) {
            atomicOr(bad, 1u);  // non-finite pointing or |dec| > pi/2
            p = h.npix;
        }
        keys[e] = (int)p;
        pos[e] = (int)e;
        rec[e] = MapRec{c, s, (double)data[e]};
    }
}

// One thread per occupied pixel: the pixel's values in sorted (= reference)
// order, added one by one onto its totals.
__global__ void map_reduce_kernel(const int* runs, const int* uniq, const int* count,
                                  const int* off, const int* pos, const MapRec* rec, double* acc,
                                  long long npix)
{
    const int nr = *runs;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        const long long p = uniq[r];
        if (p < 0 || p >= npix) continue;  // the sentinel run of rejected values
        double t[kAcc];
#pragma unroll
        for (int k = 0; k < kAcc; ++k) t[k] = acc[k * npix + p];
        const int b = off[r], n = count[r];
        for (int i = b; i < b + n; ++i) {
            const MapRec v = rec[pos[i]];
            t[kD] = PD_ADD(t[kD], PD_MUL(1.0, v.d));
            t[kCD] = PD_ADD(t[kCD], PD_MUL(v.c, v.d));
            t[kSD] = PD_ADD(t[kSD], PD_MUL(v.s, v.d));
            t[kN] = PD_ADD(t[kN], 1.0);
            t[kC] = PD_ADD(t[kC], v.c);
            t[kS] = PD_ADD(t[kS], v.s);
            t[kCC] = PD_ADD(t[kCC], PD_MUL(v.c, v.c));
            t[kCS] = PD_ADD(t[kCS], PD_MUL(v.c, v.s));
            t[kSS] = PD_ADD(t[kSS], PD_MUL(v.s, v.s));
        }
#pragma unroll
        for (int k = 0; k < kAcc; ++k) acc[k * npix + p] = t[k];
    }
}

// LAPACK dgesv for one 3 x 3 system (the reference's dgesv_ call,
// skymap.cpp:186-193), restated from the published reference LAPACK/BLAS
// algorithm: dgetf2 (pivot = first largest |a| of the column, multipliers by
// the pivot's reciprocal when |pivot| >= the safe minimum, rank-1 update
// a + l (-u) skipped where u is zero), then -- only when no pivot is exactly
// zero -- dgetrs (row interchanges, unit-lower then upper column-oriented
// triangular solves, as the reference dtrsm).  a column-major; b becomes
// the solution.  Returns LAPACK's info.
__device__ __forceinline__ int dgesv3(double a[9], double b[3])
{
    const double sfmin = 2.2250738585072014e-308;
    int ipiv[3];
    int info = 0;
#define A_(r, c) a[(c) * 3 + (r)]
    for (int j = 0; j < 3; ++j) {
        int jp = j;
        double amax = fabs(A_(j, j));
        for (int i = j + 1; i < 3; ++i)
            if (fabs(A_(i, j)) > amax) {
                amax = fabs(A_(i, j));
                jp = i;
            }
        ipiv[j] = jp;
        if (A_(jp, j) != 0.0) {
            if (jp != j)
                for (int c = 0; c < 3; ++c) {
                    const double t = A_(j, c);
                    A_(j, c) = A_(jp, c);
                    A_(jp, c) = t;
                }
            if (fabs(A_(j, j)) >= sfmin) {
                const double r = PD_DIV(1.0, A_(j, j));
                for (int i = j + 1; i < 3; ++i) A_(i, j) = PD_MUL(A_(i, j), r);
            } else {
                for (int i = j + 1; i < 3; ++i) A_(i, j) = PD_DIV(A_(i, j), A_(j, j));
            }
        } else if (info == 0) {
            info = j + 1;
        }
        for (int c = j + 1; c < 3; ++c)
            if (A_(j, c) != 0.0) {
                const double t = -A_(j, c);
                for (int i = j + 1; i < 3; ++i) A_(i, c) = PD_ADD(A_(i, c), PD_MUL(A_(i, j), t));
            }
    }
    if (info != 0) return info;
    for (int i = 0; i < 3; ++i)
        if (ipiv[i] != i) {
            const double t = b[i];
            b[i] = b[ipiv[i]];
            b[ipiv[i]] = t;
        }
    for (int k = 0; k < 3; ++k)
        if (b[k] != 0.0)
            for (int i = k + 1; i < 3; ++i) b[i] = PD_SUB(b[i], PD_MUL(b[k], A_(i, k)));
    for (int k = 2; k >= 0; --k)
        if (b[k] != 0.0) {
            b[k] = PD_DIV(b[k], A_(k, k));
            for (int i = 0; i < k; ++i) b[i] = PD_SUB(b[i], PD_MUL(b[k], A_(i, k)));
        }
#undef A_
    return 0;
}

// SkyMap::solve_map (skymap.cpp:134-231), one thread per pixel.
__global__ void map_solve_kernel(const double* acc, long long npix, float* iqu, int* hits)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const double n = acc[kN * npix + p], c = acc[kC * npix + p], s = acc[kS * npix + p];
        const double cc = acc[kCC * npix + p], cs = acc[kCS * npix + p];
        const double ss = acc[kSS * npix + p];
        double a[9] = {n, c, s, c, cc, cs, s, cs, ss};  // symmetric: row or column order alike
        double b[3] = {acc[kD * npix + p], acc[kCD * npix + p], acc[kSD * npix + p]};
        int h = (int)n;
        double ii = 0.0, qq = 0.0, uu = 0.0;  // INSUFFCOV
        if (h >= 3) {
            const int info = dgesv3(a, b);
            ii = b[0];
            qq = b[1];
            uu = b[2];
            if (info != 0) h = 0;  // unsolvable: AtD kept as the values, hits 0
        }
        iqu[p] = (float)ii;
        iqu[npix + p] = (float)qq;
        iqu[2 * npix + p] = (float)uu;
        hits[p] = h;
    }
}

int bits_for(long long v)
{
    int b = 1;
    while ((1LL << b) <= v) ++b;
    return b;
}

// The device work of one accumulate call on device arrays.
template <class T>
pisco_status accumulate(pisco_map* m, long long ns, int ndet, const T* ra, const T* dec,
                        const T* pa, const T* data, const float* h_pol, cudaStream_t st)
{
    const long long total = ns * (long long)ndet;
    if (total <= 0) return PISCO_OK;
    if (total > 0x7fffffffLL)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "more than 2^31 - 1 TOD values in one call");
    const int n = (int)total;
    pisco_status s = grow(m, kKeys, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kKeys2, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kPos, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kPos2, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kRec, sizeof(MapRec) * n + sizeof(float) * ndet + 16);
    if (s == PISCO_OK) s = grow(m, kUniq, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kCount, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kOff, sizeof(int) * n);
    if (s == PISCO_OK) s = grow(m, kRuns, 16);
    if (s != PISCO_OK) return s;
    int* keys = (int*)m->buf[kKeys];
    int* keys2 = (int*)m->buf[kKeys2];
    int* pos = (int*)m->buf[kPos];
    int* pos2 = (int*)m->buf[kPos2];
    MapRec* rec = (MapRec*)m->buf[kRec];
    float* pol = (float*)(rec + n);
    int* uniq = (int*)m->buf[kUniq];
    int* count = (int*)m->buf[kCount];
    int* off = (int*)m->buf[kOff];
    int* runs = (int*)m->buf[kRuns];
    unsigned int* bad = (unsigned int*)(runs + 2);
    const int bits = bits_for(m->npix);
    size_t t1 = 0, t2 = 0, t3 = 0;
    MCK(cub::DeviceRadixSort::SortPairs(nullptr, t1, keys, keys2, pos, pos2, n, 0, bits, st),
        "sort size");
    MCK(cub::DeviceRunLengthEncode::Encode(nullptr, t2, keys2, uniq, count, runs, n, st), "rle size");
    MCK(cub::DeviceScan::ExclusiveSum(nullptr, t3, count, off, n, st), "scan size");
    s = grow(m, kTmp, std::max(std::max(t1, t2), std::max(t3, (size_t)16)));
    if (s != PISCO_OK) return s;
    void* tmp = m->buf[kTmp];
    MCK(cudaMemcpyAsync(pol, h_pol, sizeof(float) * ndet, cudaMemcpyHostToDevice, st), "pol H2D");
    MCK(cudaMemsetAsync(bad, 0, sizeof(unsigned int), st), "reset check");
    const long long blocks = std::min<long long>((total + 255) / 256, 8192);
    map_keys_kernel<T><<<(int)blocks, 256, 0, st>>>(total, ns, m->nside, ra, dec, pa, data, pol,
                                                   keys, pos, rec, bad);
    MCK(cudaGetLastError(), "map keys");
    size_t tb = m->cap[kTmp];
    MCK(cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, pos, pos2, n, 0, bits, st), "sort");
    tb = m->cap[kTmp];
    MCK(cub::DeviceRunLengthEncode::Encode(tmp, tb, keys2, uniq, count, runs, n, st), "rle");
    tb = m->cap[kTmp];
    MCK(cub::DeviceScan::ExclusiveSum(tmp, tb, count, off, n, st), "scan");
    map_reduce_kernel<<<(int)blocks, 256, 0, st>>>(runs, uniq, count, off, pos2, rec, m->acc,
                                                  m->npix);
    MCK(cudaGetLastError(), "map reduce");
    unsigned int hb = 0;
    MCK(cudaMemcpyAsync(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, st), "check D2H");
    MCK(cudaStreamSynchronize(st), "accumulate");
    m->solved = false;
    if (hb)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT,
                        "some pointings are non-finite or have |dec| > pi/2; they were skipped");
    return PISCO_OK;
}

}  // namespace

pisco_map::~pisco_map()
{
    cudaSetDevice(device);
    for (void* p : {(void*)acc, (void*)iqu, (void*)hits})
        if (p) cudaFree(p);
    for (void* p : buf)
        if (p) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
}

extern "C" {

pisco_status pisco_map_create(int nside, int device, pisco_map** out)
{
    if (!out) return PISCO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (nside < 1 || nside > 8192) return PISCO_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return PISCO_ERR_INVALID_CONFIG;
    }
    pisco_map* m = new (std::nothrow) pisco_map;
    if (!m) return PISCO_ERR_OUT_OF_MEMORY;
    m->device = device;
    m->nside = nside;
    m->npix = 12LL * nside * nside;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&m->acc, sizeof(double) * kAcc * m->npix);
    if (e == cudaSuccess) e = cudaMalloc(&m->iqu, sizeof(float) * 3 * m->npix);
    if (e == cudaSuccess) e = cudaMalloc(&m->hits, sizeof(int) * m->npix);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->acc, 0, sizeof(double) * kAcc * m->npix, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete m;
        return e == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY : PISCO_ERR_CUDA;
    }
    *out = m;
    return PISCO_OK;
}

void pisco_map_destroy(pisco_map* m) { delete m; }

const char* pisco_map_last_error(const pisco_map* m) { return m ? m->error.c_str() : ""; }

pisco_status pisco_map_reset(pisco_map* m)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    MCK(cudaMemsetAsync(m->acc, 0, sizeof(double) * kAcc * m->npix, m->stream), "reset");
    MCK(cudaStreamSynchronize(m->stream), "reset");
    m->solved = false;
    return PISCO_OK;
}

pisco_status pisco_map_accumulate_device(pisco_map* m, long nsamples, const void* d_ra,
                                         const void* d_dec, const void* d_pa, int ndet,
                                         const float* det_pol_angles, const void* d_data,
                                         pisco_dtype dtype, void* stream)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    if (nsamples < 0 || ndet < 0) return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "negative size");
    if (nsamples == 0 || ndet == 0) return PISCO_OK;
    if (!d_ra || !d_dec || !d_pa || !d_data || !det_pol_angles)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "NULL array");
    if (dtype != PISCO_FLOAT32 && dtype != PISCO_FLOAT64)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : m->stream;
    if (dtype == PISCO_FLOAT32)
        return accumulate<float>(m, nsamples, ndet, (const float*)d_ra, (const float*)d_dec,
                                 (const float*)d_pa, (const float*)d_data, det_pol_angles, st);
    return accumulate<double>(m, nsamples, ndet, (const double*)d_ra, (const double*)d_dec,
                              (const double*)d_pa, (const double*)d_data, det_pol_angles, st);
}

pisco_status pisco_map_accumulate(pisco_map* m, long nsamples, const void* ra, const void* dec,
                                  const void* pa, int ndet, const float* det_pol_angles,
                                  const void* data, pisco_dtype dtype)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    if (nsamples < 0 || ndet < 0) return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "negative size");
    if (nsamples == 0 || ndet == 0) return PISCO_OK;
    if (!ra || !dec || !pa || !data || !det_pol_angles)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "NULL array");
    if (dtype != PISCO_FLOAT32 && dtype != PISCO_FLOAT64)
        return map_fail(m, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    const size_t esz = dtype == PISCO_FLOAT64 ? 8 : 4;
    const size_t bytes = esz * (size_t)nsamples * (size_t)ndet;
    void* d = nullptr;
    MCK(cudaMalloc(&d, 4 * bytes), "map input staging");
    const void* src[4] = {ra, dec, pa, data};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync((char*)d + k * bytes, src[k], bytes, cudaMemcpyHostToDevice, m->stream);
    pisco_status s = PISCO_OK;
    if (e != cudaSuccess) {
        cudaGetLastError();
        s = map_fail(m, PISCO_ERR_CUDA, std::string("map input H2D: ") + cudaGetErrorString(e));
    } else {
        s = pisco_map_accumulate_device(m, nsamples, d, (char*)d + bytes, (char*)d + 2 * bytes,
                                        ndet, det_pol_angles, (char*)d + 3 * bytes, dtype,
                                        m->stream);
    }
    cudaStreamSynchronize(m->stream);
    cudaFree(d);
    return s;
}

pisco_status pisco_map_solve(pisco_map* m)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    const long long blocks = std::min<long long>((m->npix + 255) / 256, 16384);
    map_solve_kernel<<<(int)blocks, 256, 0, m->stream>>>(m->acc, m->npix, m->iqu, m->hits);
    MCK(cudaGetLastError(), "map solve");
    MCK(cudaStreamSynchronize(m->stream), "map solve");
    m->solved = true;
    return PISCO_OK;
}

pisco_status pisco_map_get(pisco_map* m, float* I, float* Q, float* U, int* hits)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    if (!m->solved) return map_fail(m, PISCO_ERR_NOT_READY, "call pisco_map_solve first");
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    float* out[3] = {I, Q, U};
    for (int k = 0; k < 3; ++k)
        if (out[k])
            MCK(cudaMemcpyAsync(out[k], m->iqu + k * m->npix, sizeof(float) * m->npix,
                                cudaMemcpyDeviceToHost, m->stream),
                "map D2H");
    if (hits)
        MCK(cudaMemcpyAsync(hits, m->hits, sizeof(int) * m->npix, cudaMemcpyDeviceToHost, m->stream),
            "hits D2H");
    MCK(cudaStreamSynchronize(m->stream), "map D2H");
    return PISCO_OK;
}

pisco_status pisco_map_get_normal(pisco_map* m, double* ata, double* atd)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    MCK(cudaSetDevice(m->device), "cudaSetDevice");
    const long long n = m->npix;
    double* h = nullptr;
    MCK(cudaMallocHost(&h, sizeof(double) * kAcc * n), "host staging");
    cudaError_t e = cudaMemcpyAsync(h, m->acc, sizeof(double) * kAcc * n, cudaMemcpyDeviceToHost,
                                    m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) {
        // AtA[p] = [n c s; c cc cs; s cs ss], AtD[p] = (d, cd, sd)
        static const int ata_of[9] = {kN, kC, kS, kC, kCC, kCS, kS, kCS, kSS};
        for (long long p = 0; p < n; ++p) {
            if (ata)
                for (int k = 0; k < 9; ++k) ata[9 * p + k] = h[ata_of[k] * n + p];
            if (atd)
                for (int k = 0; k < 3; ++k) atd[3 * p + k] = h[(kD + k) * n + p];
        }
    }
    cudaFreeHost(h);
    MCK(e, "normal equations D2H");
    return PISCO_OK;
}

pisco_status pisco_map_device_arrays(pisco_map* m, const float** d_iqu, const int** d_hits,
                                     const double** d_normal)
{
    if (!m) return PISCO_ERR_INVALID_ARGUMENT;
    if (d_iqu) *d_iqu = m->iqu;
    if (d_hits) *d_hits = m->hits;
    if (d_normal) *d_normal = m->acc;
    return PISCO_OK;
}

}  // extern "C"
