// noalloc.cu -- pisco_forward_batched_noalloc: the batched TUNED forward for
// callers that must not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not
// wanted -- inside a host callback or a real-time acquisition loop that may
// not block on the allocator, inside a framework whose memory pool owns
// every byte of the GPU (it hands out buffers but forbids side allocations),
// or a long-running service that must never fail mid-run with
// out-of-memory.  Such callers own every input and output buffer; this entry
// point takes them as device pointers and keeps its own working memory (the
// work queue of the batched kernel) in a fixed array compiled into the
// library.
//
// The working memory is g_noalloc_scratch below: a file-scope
// static __device__ array of kScratchBytes (about 2.6 MB).  Every GPU that
// loads the library holds it until the process exits.  It holds the sky
// ring table (2.1 MB, sized for nside 8192), the
// detector descriptors (at most PISCO_NOALLOC_MAX_DETS), the work items (at
// most PISCO_NOALLOC_MAX_ITEMS), the queue counter, the device error word
// and the FP64-fallback counter.  All calls share it and it keeps the last
// call's contents; each call rewrites the descriptors and items and clears
// the counters before its kernel runs.  Two calls whose GPU work overlaps
// (different host threads, or different streams of one device) race on it:
// serialise them.
//
// In host code the name g_noalloc_scratch stands for a host-side shadow, not
// a device address; the device address is obtained once per device with
// cudaGetSymbolAddress (with that device current) by the first call on that
// device, and passed to the kernels.  That first call should therefore come
// before any CUDA stream capture on the device.  The address is cached for
// the life of the process: a cudaDeviceReset of that device invalidates it,
// so a process that resets a device must not call this entry point on it
// afterwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <mutex>

#include "../../include/pisco_gb300.h"
#include "internal.h"

namespace pisco {

void set_null_ctx_error(const char* msg);  // capi.cu

namespace {

constexpr int kMaxDets = PISCO_NOALLOC_MAX_DETS;
constexpr int kMaxItems = PISCO_NOALLOC_MAX_ITEMS;
constexpr int kMaxDevices = 64;

struct Scratch {
    RingT rings[kMaxRings];  // sky ring table, rebuilt by every call
    BatchDet dets[kMaxDets];
    BatchItem items[kMaxItems];
    unsigned int queue;
    unsigned int err;
    unsigned long long fallbacks;
};
constexpr size_t kScratchBytes = sizeof(Scratch);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Descriptors travel to the device as a kernel parameter (no staging copy).
struct SetupParams {
    BatchDet dets[kMaxDets];
    long long first_item[kMaxDets + 1];
    int ndet;
    int chunk;
};

__global__ void noalloc_setup_kernel(SetupParams p, Scratch* s)
{
    for (int d = threadIdx.x; d < p.ndet; d += blockDim.x) s->dets[d] = p.dets[d];
    for (int d = 0; d < p.ndet; ++d) {
        const long long n = p.dets[d].n;
        const long long base = p.first_item[d];
        const long long cnt = p.first_item[d + 1] - base;
        for (long long k = threadIdx.x; k < cnt; k += blockDim.x) {
            const long long b = k * p.chunk;
            s->items[base + k] = BatchItem{d, (int)(n - b < p.chunk ? n - b : p.chunk), b};
        }
    }
    if (threadIdx.x == 0) {
        s->queue = 0u;
        s->err = 0u;
        s->fallbacks = 0ull;
    }
}

std::mutex g_setup_mutex;

pisco_status reject(pisco_status s, const char* msg)
{
    set_null_ctx_error(msg);
    return s;
}
Scratch* g_scratch_ptr[kMaxDevices] = {};

}  // namespace
}  // namespace pisco

using namespace pisco;

extern "C" pisco_status pisco_forward_batched_noalloc(int device, int nside_sky,
                                                      const float* d_sky_iquv,
                                                      const pisco_noalloc_det* dets, int ndet,
                                                      int chunk, void* stream)
{
    // ---- argument checks (no GPU work yet)
    set_null_ctx_error("");
    if (device < 0 || device >= kMaxDevices)
        return reject(PISCO_ERR_INVALID_ARGUMENT, "noalloc: device index out of range");
    if (nside_sky < 1 || nside_sky > 8192 || !d_sky_iquv || ((uintptr_t)d_sky_iquv & 15))
        return reject(PISCO_ERR_INVALID_ARGUMENT,
                      "noalloc: sky must be a 16-byte aligned device array, nside in [1, 8192]");
    if (!dets || ndet < 1)
        return reject(PISCO_ERR_INVALID_ARGUMENT, "noalloc: need at least one detector pair");
    if (ndet > kMaxDets)
        return reject(PISCO_ERR_INVALID_ARGUMENT,
                      "noalloc: more than PISCO_NOALLOC_MAX_DETS (128) detector pairs; split the call");
    if (chunk == 0) chunk = 256;
    if (chunk < 1) return reject(PISCO_ERR_INVALID_ARGUMENT, "noalloc: chunk must be >= 0");
    SetupParams p;
    std::pair<double, int> order[kMaxDets];
    long long nitems = 0;
    for (int d = 0; d < ndet; ++d) {
        const pisco_noalloc_det& x = dets[d];
        if (x.nside_beam < 1 || x.nside_beam > 8192 || x.npix_beam < 1 ||
            x.npix_beam >= 12L * x.nside_beam * x.nside_beam || !x.beam_ab ||
            ((uintptr_t)x.beam_ab & 31) || x.nsamples < 0 ||
            (x.nsamples > 0 && (!x.ra || !x.dec || !x.pa)))
            return reject(PISCO_ERR_INVALID_ARGUMENT,
                          "noalloc: bad detector descriptor (beam size, 32-byte alignment or NULL pointing)");
        // same bound as the context-based batched forward; it also keeps the
        // item count below from overflowing
        if (x.nsamples > (1LL << 40))
            return reject(PISCO_ERR_INVALID_ARGUMENT,
                          "noalloc: more than 2^40 samples in one detector pair");
        const double rho = pisco_beam_rho_max(x.nside_beam, x.npix_beam);
        if (!tuned_supported(x.nside_beam, (int)x.npix_beam, rho))
            return reject(PISCO_ERR_UNSUPPORTED, "noalloc: a beam lies outside the TUNED form's domain");
        nitems += (x.nsamples + chunk - 1) / chunk;
        // longest (estimated pairs) first, as the context-based batched forward
        order[d] = {-(double)x.nsamples * (1.0 - std::cos(rho)), d};
    }
    if (nitems > kMaxItems)
        return reject(PISCO_ERR_INVALID_ARGUMENT,
                      "noalloc: more than PISCO_NOALLOC_MAX_ITEMS (32768) work items; raise chunk");
    std::stable_sort(order, order + ndet);
    p.ndet = ndet;
    p.chunk = chunk;
    p.first_item[0] = 0;
    for (int k = 0; k < ndet; ++k) {
        const pisco_noalloc_det& x = dets[order[k].second];
        const double rho = pisco_beam_rho_max(x.nside_beam, x.npix_beam);
        p.dets[k] = BatchDet{(const F8*)x.beam_ab, x.nside_beam, (int)x.npix_beam, rho,
                             (float)(1.7320508075688772 * x.nside_beam), x.nsamples, x.ra, x.dec,
                             x.pa, x.tod_a, x.tod_b};
        p.first_item[k + 1] = p.first_item[k] + (x.nsamples + chunk - 1) / chunk;
    }

    // ---- once per device: the device address of the static scratch array
    int prev = -1;
    cudaError_t es = cudaGetDevice(&prev);
    if (es != cudaSuccess) {
        cudaGetLastError();
        return reject(PISCO_ERR_CUDA, cudaGetErrorString(es));
    }
    es = cudaSetDevice(device);
    if (es != cudaSuccess) {
        cudaGetLastError();
        return reject(PISCO_ERR_CUDA, cudaGetErrorString(es));
    }
    Scratch* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[device]) {
            void* ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                cudaGetLastError();
                cudaSetDevice(prev);
                return reject(PISCO_ERR_CUDA, "noalloc: cudaGetSymbolAddress of the scratch array failed");
            }
            g_scratch_ptr[device] = (Scratch*)ptr;
        }
        scratch = g_scratch_ptr[device];
    }
    int sms = 0;
    es = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (es != cudaSuccess) {
        cudaGetLastError();
        cudaSetDevice(prev);
        return reject(PISCO_ERR_CUDA, cudaGetErrorString(es));
    }
    cudaStream_t st = (cudaStream_t)stream;
    noalloc_setup_kernel<<<1, 256, 0, st>>>(p, scratch);
    cudaError_t e0 = cudaGetLastError();
    if (e0 == cudaSuccess) e0 = launch_ring_table(nside_sky, scratch->rings, st);
    BatchArgs a;
    a.nside_sky = nside_sky;
    a.rings = scratch->rings;
    a.sky32 = (const float4*)d_sky_iquv;
    a.dets = scratch->dets;
    a.ndet = ndet;
    a.items = scratch->items;
    a.nitems = (int)nitems;
    a.queue = &scratch->queue;
    a.out_f64 = 0;
    a.err = &scratch->err;
    a.fallbacks = &scratch->fallbacks;
    cudaError_t e = e0;
    if (e == cudaSuccess) e = launch_batched(a, sms, st);
    // synchronous: read the device error word back
    unsigned int code = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&code, &scratch->err, sizeof(code), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return reject(PISCO_ERR_CUDA, cudaGetErrorString(e));
    }
    return code ? reject(PISCO_ERR_DEVICE_CHECK, "noalloc: device-side check failed") : PISCO_OK;
}
