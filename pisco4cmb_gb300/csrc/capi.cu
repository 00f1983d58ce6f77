// capi.cu -- the C ABI of libpisco_gb300 (include/pisco_gb300.h): context,
// device-resident inputs and the forward entry points.
//
// Replaces the host orchestration of GPUConvolver
// (src/GpuConvolver/gpuconvolver.cu:34-505): instead of a host OpenMP
// query_disc per chunk, three padded ptgPerConv x pixelsPerDisc transfers
// and two synchronising kernels, the sky, beam and scan are made resident
// once and one kernel computes every sample from its pointing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/pisco_gb300.h"
#include "ctx.h"
#include "hpx.cuh"
#include "internal.h"

using namespace pisco;

namespace {

thread_local std::string g_create_error;

pisco_status fail(pisco_ctx* c, pisco_status s, const std::string& msg)
{
    if (c) c->error = msg;
    return s;
}

pisco_status cuda_fail(pisco_ctx* c, cudaError_t e, const char* what)
{
    cudaGetLastError();  // clear sticky-free errors
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY : PISCO_ERR_CUDA, m);
}

#define CK(call, what)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

}  // namespace

namespace pisco {
// Message for pisco_last_error(NULL) from entry points that have no context.
void set_null_ctx_error(const char* msg) { g_create_error = msg; }
}  // namespace pisco

pisco_ctx::~pisco_ctx()
{
    cudaSetDevice(device);
    for (void* p : {(void*)sky32, (void*)sky64, (void*)beam32, (void*)beam64, (void*)ra,
                    (void*)dec, (void*)pa, (void*)d_err, (void*)d_count, (void*)d_fallbacks,
                    (void*)out_dev})
        if (p) cudaFree(p);
    for (auto& s : slots)
        if (s.beam) cudaFree(s.beam);
    for (void* p : {(void*)d_dets, (void*)d_items, (void*)d_queue, (void*)adj_sky32,
                    (void*)adj_beam32, (void*)adj_sky_fx, (void*)adj_beam_fx, (void*)red,
                    (void*)adj_ptab, (void*)adj_ppart,
                    (void*)rings, (void*)ord, (void*)ord_keys, (void*)ord_keys2,
                    (void*)ord_pos, ord_tmp, (void*)beam_scr, plans})
        if (p) cudaFree(p);
    for (int* p : det_ord)
        if (p) cudaFree(p);
    if (ord_event) cudaEventDestroy(ord_event);
    if (plan_event) cudaEventDestroy(plan_event);
    if (batch_event) cudaEventDestroy(batch_event);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (stream) cudaStreamDestroy(stream);
}

pisco_status pisco_ctx::activate()
{
    pisco_ctx* c = this;
    CK(cudaSetDevice(device), "cudaSetDevice");
    return PISCO_OK;
}

pisco_status pisco_ctx::ensure(void** p, size_t* cap, size_t bytes, const char* what)
{
    pisco_ctx* c = this;
    if (*cap >= bytes && *p) return PISCO_OK;
    size_t grow = bytes - (*p ? *cap : 0);
    if (cfg.maxMemUsage && mem_used + grow > cfg.maxMemUsage) {
        // the sample-plan scratch yields to every other buffer: freed when
        // that makes room (the forward then plans again within what is left)
        if (p != &plans && plans && mem_used - plans_cap + grow <= cfg.maxMemUsage) {
            CK(cudaDeviceSynchronize(), "sync before freeing the plan scratch");
            cudaFree(plans);
            mem_used -= plans_cap;
            plans = nullptr;
            plans_cap = 0;
        } else {
            return fail(this, PISCO_ERR_OUT_OF_MEMORY,
                        std::string(what) + ": maxMemUsage of the RunConfig exceeded");
        }
    }
    if (*p) {
        CK(cudaStreamSynchronize(stream), "sync before realloc");
        cudaFree(*p);
        mem_used -= *cap;
        *p = nullptr;
        *cap = 0;
    }
    CK(cudaMalloc(p, bytes), what);
    *cap = bytes;
    mem_used += bytes;
    return PISCO_OK;
}

pisco_status pisco_ctx::ensure_rings(cudaStream_t s)
{
    pisco_ctx* c = this;
    if (rings && rings_nside == nside_sky) return PISCO_OK;
    pisco_status st = ensure((void**)&rings, &rings_cap, sizeof(pisco::RingT) * pisco::kMaxRings,
                             "ring table");
    if (st != PISCO_OK) return st;
    CK(pisco::launch_ring_table(nside_sky, rings, s), "ring table");
    rings_nside = nside_sky;
    return PISCO_OK;
}

pisco_status pisco_ctx::make_order(const double* pra, const double* pdec, long long n, int** buf,
                                   size_t* cap, cudaStream_t s)
{
    pisco_ctx* c = this;
    size_t tmp_bytes = 0;
    CK(pisco::sky_order(n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &tmp_bytes,
                        s),
       "sky order size");
    const size_t nb = sizeof(int) * (size_t)n;
    pisco_status st = ensure((void**)&ord_keys, &ord_keys_cap, nb, "order keys");
    if (st == PISCO_OK) st = ensure((void**)&ord_keys2, &ord_keys2_cap, nb, "order keys");
    if (st == PISCO_OK) st = ensure((void**)&ord_pos, &ord_pos_cap, nb, "order positions");
    if (st == PISCO_OK) st = ensure(&ord_tmp, &ord_tmp_cap, tmp_bytes > 0 ? tmp_bytes : 16, "order sort");
    if (st == PISCO_OK) st = ensure((void**)buf, cap, nb, "sample order");
    if (st != PISCO_OK) return st;
    tmp_bytes = ord_tmp_cap;
    CK(pisco::sky_order(n, pra, pdec, ord_keys, ord_keys2, ord_pos, *buf, ord_tmp, &tmp_bytes, s),
       "sky order");
    return PISCO_OK;
}

pisco_status pisco_ctx::range_order(long long begin, long long n, cudaStream_t s, const int** out)
{
    pisco_ctx* c = this;
    *out = nullptr;
    if (sample_order != PISCO_ORDER_SKY || n < 2 || n > 0x7fffffffLL) return PISCO_OK;
    if (!ord_event) CK(cudaEventCreateWithFlags(&ord_event, cudaEventDisableTiming), "order event");
    else CK(cudaStreamWaitEvent(s, ord_event, 0), "order wait");
    if (!(ord && ord_begin == begin && ord_n == n && ord_version == scan_version)) {
        ord_n = -1;
        pisco_status st = make_order(ra + begin, dec + begin, n, &ord, &ord_cap, s);
        if (st != PISCO_OK) return st;
        ord_begin = begin;
        ord_n = n;
        ord_version = scan_version;
    }
    *out = ord;
    return PISCO_OK;
}

void pisco_ctx::order_used(cudaStream_t s)
{
    if (ord_event) cudaEventRecord(ord_event, s);
}

// Sample plans built by the plan kernel (1) or by each warp (0).
#ifndef PISCO_FWD_PLANS
#define PISCO_FWD_PLANS 1
#endif
// At most max_plans sample plans (4M: 384 MB of scratch, for the forward's
// chunks); fewer when maxMemUsage leaves less room (the forward then runs in
// more chunks), none below kMinPlans.
constexpr long long kMinPlans = 1024;

void pisco_ctx::plan_scratch(long long n, cudaStream_t s, void** p, long long* cap,
                             long long max_plans)
{
    *p = nullptr;
    *cap = 0;
    const long long want = std::min(n, max_plans);
    long long fit = want;
    if (cfg.maxMemUsage) {
        const size_t room = (cfg.maxMemUsage > mem_used ? cfg.maxMemUsage - mem_used : 0) + plans_cap;
        fit = std::min<long long>(want, (long long)(room / pisco::kSamplePlanBytes));
    }
    const long long need = std::min(n, kMinPlans);
    if (fit >= need && plans_cap < pisco::kSamplePlanBytes * (size_t)fit) {
        // growing frees the old scratch: wait for its last reader, on any stream
        if (plans && plan_event && cudaEventSynchronize(plan_event) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        const std::string keep = error;
        if (ensure(&plans, &plans_cap, pisco::kSamplePlanBytes * (size_t)fit, "sample plans") !=
            PISCO_OK)
            error = keep;
    }
    const long long have = plans ? (long long)(plans_cap / pisco::kSamplePlanBytes) : 0;
    if (have < need) return;
    if (!plan_event) {
        if (cudaEventCreateWithFlags(&plan_event, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            plan_event = nullptr;
            return;
        }
    } else if (cudaStreamWaitEvent(s, plan_event, 0) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    *p = plans;
    *cap = std::min(have, want);
}

void pisco_ctx::plans_used(cudaStream_t s)
{
    if (plan_event) cudaEventRecord(plan_event, s);
}

pisco_status pisco_ctx::check_device()
{
    pisco_ctx* c = this;
    unsigned int code = 0;
    CK(cudaMemcpyAsync(&code, d_err, sizeof(code), cudaMemcpyDeviceToHost, stream), "read error word");
    CK(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    if (code != kCheckOk) {
        CK(cudaMemsetAsync(d_err, 0, sizeof(unsigned int), stream), "reset error word");
        static const char* names[] = {"ok", "sky index out of range", "beam index out of range",
                                      "fallback queue overflow", "work queue", "adjoint index"};
        return fail(this, PISCO_ERR_DEVICE_CHECK,
                    std::string("device check failed: ") + (code < 6 ? names[code] : "unknown"));
    }
    return PISCO_OK;
}

extern "C" {

int pisco_abi_version(void) { return PISCO_ABI_VERSION; }

const char* pisco_status_string(pisco_status s)
{
    switch (s) {
    case PISCO_OK: return "ok";
    case PISCO_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PISCO_ERR_INVALID_CONFIG: return "invalid configuration";
    case PISCO_ERR_NOT_READY: return "sky, beam or scan not set";
    case PISCO_ERR_CUDA: return "CUDA error";
    case PISCO_ERR_OUT_OF_MEMORY: return "out of memory";
    case PISCO_ERR_UNSUPPORTED: return "unsupported";
    case PISCO_ERR_DEVICE_CHECK: return "device-side check failed";
    }
    return "unknown status";
}

const char* pisco_last_error(const pisco_ctx* c)
{
    if (!c) return g_create_error.c_str();
    return c->error.c_str();
}

pisco_status pisco_create(const pisco_run_config* cfg, pisco_ctx** out)
{
    g_create_error.clear();
    if (!out) {
        g_create_error = "pisco_create: out is NULL";
        return PISCO_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    pisco_run_config cf;
    if (cfg) cf = *cfg;
    else {
        std::memset(&cf, 0, sizeof(cf));
        cf.nStreams = 1;
        cf.ptgPerConv = 1 << 20;
    }
    // The reference rejects a configuration whose buffers exceed maxMemUsage
    // or with no stream (gpuconvolver.cu:58-70); here the per-chunk buffers
    // are only the TOD staging, so the check is on nStreams, ptgPerConv and
    // the minimum working set (outputs of one chunk).
    if (cf.nStreams < 1 || cf.ptgPerConv < 1 || cf.pixelsPerDisc < 0) {
        g_create_error = "FATAL: GPUConvolver has an invalid configuration (nStreams >= 1, "
                         "ptgPerConv >= 1 required).";
        return PISCO_ERR_INVALID_CONFIG;
    }
    if (cf.maxMemUsage && cf.maxMemUsage < (size_t)cf.ptgPerConv * 2 * sizeof(double)) {
        g_create_error = "FATAL: GPUConvolver has an invalid configuration (maxMemUsage below "
                         "the output buffers of one chunk).";
        return PISCO_ERR_INVALID_CONFIG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return PISCO_ERR_CUDA;
    }
    if (cf.deviceId < 0 || cf.deviceId >= ndev) {
        g_create_error = "deviceId out of range";
        return PISCO_ERR_INVALID_CONFIG;
    }
    pisco_ctx* c = new (std::nothrow) pisco_ctx();
    if (!c) return PISCO_ERR_OUT_OF_MEMORY;
    c->cfg = cf;
    c->device = cf.deviceId;
    pisco_status st = c->activate();
    if (st != PISCO_OK) {
        g_create_error = c->error;
        delete c;
        return st;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_count, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_fallbacks, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(c->d_fallbacks, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        g_create_error = std::string("context setup: ") + cudaGetErrorString(e);
        cudaGetLastError();
        delete c;
        return e == cudaErrorMemoryAllocation ? PISCO_ERR_OUT_OF_MEMORY : PISCO_ERR_CUDA;
    }
    c->sm_count = prop.multiProcessorCount;
    *out = c;
    return PISCO_OK;
}

pisco_status pisco_destroy(pisco_ctx* c)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    delete c;
    return PISCO_OK;
}

pisco_status pisco_set_interp(pisco_ctx* c, pisco_interp interp)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (interp != PISCO_BEAM_NEAREST && interp != PISCO_BEAM_BILINEAR)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "interp must be NEAREST or BILINEAR");
    c->interp = interp;
    return PISCO_OK;
}

pisco_status pisco_set_sample_order(pisco_ctx* c, pisco_order order)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (order != PISCO_ORDER_SCAN && order != PISCO_ORDER_SKY)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "order must be SCAN or SKY");
    c->sample_order = order;
    return PISCO_OK;
}

static bool valid_nside(int nside) { return nside >= 1 && nside <= 8192; }

pisco_status pisco_set_sky(pisco_ctx* c, int nside, const void* I, const void* Q, const void* U,
                           const void* V, pisco_dtype dt)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!valid_nside(nside)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky nside must be in [1, 8192]");
    if (!I || !Q || !U) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky I, Q and U must not be NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    const long long npix = 12LL * nside * nside;
    // transpose the four planes into interleaved IQUV (gpuconvolver.cu:248-254)
    std::vector<float> t32;
    std::vector<double> t64;
    try {
        t32.resize(4 * npix);
        if (dt == PISCO_FLOAT64) t64.resize(4 * npix);
    } catch (const std::bad_alloc&) {
        return fail(c, PISCO_ERR_OUT_OF_MEMORY, "host transpose buffer");
    }
    const void* planes[4] = {I, Q, U, V};
    for (int k = 0; k < 4; ++k) {
        if (!planes[k]) {
            for (long long i = 0; i < npix; ++i) t32[4 * i + k] = 0.0f;
            if (dt == PISCO_FLOAT64)
                for (long long i = 0; i < npix; ++i) t64[4 * i + k] = 0.0;
            continue;
        }
        if (dt == PISCO_FLOAT32) {
            const float* p = (const float*)planes[k];
            for (long long i = 0; i < npix; ++i) t32[4 * i + k] = p[i];
        } else {
            const double* p = (const double*)planes[k];
            for (long long i = 0; i < npix; ++i) {
                t64[4 * i + k] = p[i];
                t32[4 * i + k] = (float)p[i];
            }
        }
    }
    // A failure of the first allocation leaves the previous sky in place (the
    // maxMemUsage check) or no sky (cudaMalloc failed after the old buffer
    // was freed); past it the device sky is being replaced, so the context
    // reports NOT_READY until this call completes.
    st = c->ensure((void**)&c->sky32, &c->sky32_cap, sizeof(float4) * npix, "sky buffer");
    if (st != PISCO_OK) return st;
    c->nside_sky = 0;
    CK(cudaMemcpyAsync(c->sky32, t32.data(), sizeof(float4) * npix, cudaMemcpyHostToDevice, c->stream),
       "sky H2D");
    c->sky64_valid = false;
    if (dt == PISCO_FLOAT64) {
        st = c->ensure((void**)&c->sky64, &c->sky64_cap, sizeof(D4) * npix, "sky64 buffer");
        if (st != PISCO_OK) return st;
        CK(cudaMemcpyAsync(c->sky64, t64.data(), sizeof(D4) * npix, cudaMemcpyHostToDevice, c->stream),
           "sky64 H2D");
        c->sky64_valid = true;
    }
    c->nside_sky = nside;
    c->pairs_valid = false;
    st = c->ensure_rings(c->stream);
    if (st != PISCO_OK) return st;
    CK(cudaStreamSynchronize(c->stream), "sky upload");
    return PISCO_OK;
}

pisco_status pisco_set_sky_device(pisco_ctx* c, int nside, const void* d_iquv, pisco_dtype dt,
                                  void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!valid_nside(nside)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky nside must be in [1, 8192]");
    if (!d_iquv) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sky pointer is NULL");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const long long npix = 12LL * nside * nside;
    st = c->ensure((void**)&c->sky32, &c->sky32_cap, sizeof(float4) * npix, "sky buffer");
    if (st != PISCO_OK) return st;
    c->nside_sky = 0;  // replaced from here on (see pisco_set_sky)
    if (dt == PISCO_FLOAT32) {
        CK(cudaMemcpyAsync(c->sky32, d_iquv, sizeof(float4) * npix, cudaMemcpyDeviceToDevice, s), "sky D2D");
        c->sky64_valid = false;
    } else if (dt == PISCO_FLOAT64) {
        st = c->ensure((void**)&c->sky64, &c->sky64_cap, sizeof(D4) * npix, "sky64 buffer");
        if (st != PISCO_OK) return st;
        CK(cudaMemcpyAsync(c->sky64, d_iquv, sizeof(D4) * npix, cudaMemcpyDeviceToDevice, s), "sky64 D2D");
        CK(launch_narrow_sky(c->sky64, c->sky32, npix, s), "narrow sky");
        c->sky64_valid = true;
    } else {
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    }
    c->nside_sky = nside;
    c->pairs_valid = false;
    st = c->ensure_rings(s);
    if (st != PISCO_OK) return st;
    if (s != c->stream) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(c->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    return PISCO_OK;
}

pisco_status pisco_set_beam(pisco_ctx* c, int nside, long npix, const void* const a[4],
                            const void* const b[4], pisco_dtype dt)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!valid_nside(nside)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nside must be in [1, 8192]");
    if (npix < 1 || npix >= 12LL * nside * nside)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nPixels must be in [1, 12 nside^2)");
    if (!a || !b) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam plane arrays are NULL");
    for (int k = 0; k < 4; ++k)
        if (!a[k] || !b[k]) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam plane is NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    std::vector<F8> t32(npix);
    std::vector<D8> t64;
    if (dt == PISCO_FLOAT64) t64.resize(npix);
    for (long i = 0; i < npix; ++i) {
        float fa[4], fb[4];
        double da[4], db[4];
        for (int k = 0; k < 4; ++k) {
            if (dt == PISCO_FLOAT32) {
                fa[k] = ((const float*)a[k])[i];
                fb[k] = ((const float*)b[k])[i];
            } else {
                da[k] = ((const double*)a[k])[i];
                db[k] = ((const double*)b[k])[i];
                fa[k] = (float)da[k];
                fb[k] = (float)db[k];
            }
        }
        t32[i].a = make_float4(fa[0], fa[1], fa[2], fa[3]);
        t32[i].b = make_float4(fb[0], fb[1], fb[2], fb[3]);
        if (dt == PISCO_FLOAT64) t64[i] = D8{D4{da[0], da[1], da[2], da[3]}, D4{db[0], db[1], db[2], db[3]}};
    }
    st = c->ensure((void**)&c->beam32, &c->beam32_cap, sizeof(F8) * npix, "beam buffer");
    if (st != PISCO_OK) return st;
    CK(cudaMemcpyAsync(c->beam32, t32.data(), sizeof(F8) * npix, cudaMemcpyHostToDevice, c->stream),
       "beam H2D");
    c->beam64_valid = false;
    if (dt == PISCO_FLOAT64) {
        st = c->ensure((void**)&c->beam64, &c->beam64_cap, sizeof(D8) * npix, "beam64 buffer");
        if (st != PISCO_OK) return st;
        CK(cudaMemcpyAsync(c->beam64, t64.data(), sizeof(D8) * npix, cudaMemcpyHostToDevice, c->stream),
           "beam64 H2D");
        c->beam64_valid = true;
    }
    CK(cudaStreamSynchronize(c->stream), "beam upload");
    c->nside_beam = nside;
    c->npix_beam = npix;
    c->rho_max = pisco_beam_rho_max(nside, npix);
    c->pairs_valid = false;
    return PISCO_OK;
}

pisco_status pisco_set_scan(pisco_ctx* c, long n, const void* ra, const void* dec, const void* pa,
                            pisco_dtype dt)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (n < 0) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "nsamples must be >= 0");
    if (n > 0 && (!ra || !dec || !pa)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "scan arrays are NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    const size_t bytes = sizeof(double) * (size_t)std::max<long>(n, 1);
    st = c->ensure((void**)&c->ra, &c->ra_cap, bytes, "scan ra");
    if (st == PISCO_OK) st = c->ensure((void**)&c->dec, &c->dec_cap, bytes, "scan dec");
    if (st == PISCO_OK) st = c->ensure((void**)&c->pa, &c->pa_cap, bytes, "scan pa");
    if (st != PISCO_OK) return st;
    if (n > 0) {
        if (dt == PISCO_FLOAT64) {
            CK(cudaMemcpyAsync(c->ra, ra, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "ra H2D");
            CK(cudaMemcpyAsync(c->dec, dec, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "dec H2D");
            CK(cudaMemcpyAsync(c->pa, pa, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "pa H2D");
        } else {
            // float pointing (the reference Scan API): widen on the host
            std::vector<double> w;
            try {
                w.resize((size_t)n);
            } catch (const std::bad_alloc&) {
                return fail(c, PISCO_ERR_OUT_OF_MEMORY, "host widening buffer");
            }
            const void* src[3] = {ra, dec, pa};
            double* dst[3] = {c->ra, c->dec, c->pa};
            for (int k = 0; k < 3; ++k) {
                const float* f = (const float*)src[k];
                for (long i = 0; i < n; ++i) w[i] = (double)f[i];
                CK(cudaMemcpy(dst[k], w.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "scan H2D");
            }
        }
    }
    CK(cudaStreamSynchronize(c->stream), "scan upload");
    c->nsamples = n;
    c->pairs_valid = false;
    ++c->scan_version;
    return PISCO_OK;
}

pisco_status pisco_set_scan_device(pisco_ctx* c, long n, const double* d_ra, const double* d_dec,
                                   const double* d_pa, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (n < 0) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "nsamples must be >= 0");
    if (n > 0 && (!d_ra || !d_dec || !d_pa)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "scan arrays are NULL");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const size_t bytes = sizeof(double) * (size_t)std::max<long>(n, 1);
    st = c->ensure((void**)&c->ra, &c->ra_cap, bytes, "scan ra");
    if (st == PISCO_OK) st = c->ensure((void**)&c->dec, &c->dec_cap, bytes, "scan dec");
    if (st == PISCO_OK) st = c->ensure((void**)&c->pa, &c->pa_cap, bytes, "scan pa");
    if (st != PISCO_OK) return st;
    if (n > 0) {
        CK(cudaMemcpyAsync(c->ra, d_ra, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "ra D2D");
        CK(cudaMemcpyAsync(c->dec, d_dec, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "dec D2D");
        CK(cudaMemcpyAsync(c->pa, d_pa, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "pa D2D");
    }
    if (s != c->stream) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(c->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    c->nsamples = n;
    c->pairs_valid = false;
    ++c->scan_version;
    return PISCO_OK;
}

pisco_status pisco_forward_device(pisco_ctx* c, pisco_form form, long begin, long n, void* d_a,
                                  void* d_b, pisco_dtype out_dtype, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (!c->sky32 || !c->nside_sky) return fail(c, PISCO_ERR_NOT_READY, "no sky set");
    if (!c->beam32 || !c->nside_beam) return fail(c, PISCO_ERR_NOT_READY, "no beam set");
    if (c->nsamples < 0 || (!c->ra && c->nsamples > 0)) return fail(c, PISCO_ERR_NOT_READY, "no scan set");
    if (begin < 0 || n < 0 || begin + n > c->nsamples)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sample range outside the scan");
    if (out_dtype != PISCO_FLOAT32 && out_dtype != PISCO_FLOAT64)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad output dtype");
    if (form != PISCO_FORM_PLAIN && form != PISCO_FORM_TUNED && form != PISCO_FORM_FP64)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad form");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    FwdArgs a{};
    a.nside_sky = c->nside_sky;
    a.sky32 = c->sky32;
    a.rings = c->rings;
    a.sky64 = nullptr;
    a.nside_beam = c->nside_beam;
    a.npix_beam = (int)c->npix_beam;
    a.beam32 = c->beam32;
    a.beam64 = nullptr;
    a.rho_max = c->rho_max;
    a.begin = begin;
    a.n = n;
    a.ra = c->ra;
    a.dec = c->dec;
    a.pa = c->pa;
    a.out_a = d_a;
    a.out_b = d_b;
    st = c->range_order(begin, n, s, &a.order);
    if (st != PISCO_OK) return st;
    a.out_f64 = out_dtype == PISCO_FLOAT64;
    a.interp = (int)c->interp;
    a.err = c->d_err;
    a.fallbacks = c->d_fallbacks;
    cudaError_t e;
    if (form == PISCO_FORM_FP64) {
        const long long npix = 12LL * c->nside_sky * c->nside_sky;
        if (!c->sky64_valid) {
            st = c->ensure((void**)&c->sky64, &c->sky64_cap, sizeof(D4) * npix, "sky64 buffer");
            if (st != PISCO_OK) return st;
            CK(launch_widen_sky(c->sky32, c->sky64, npix, s), "widen sky");
            c->sky64_valid = true;
        }
        if (!c->beam64_valid) {
            st = c->ensure((void**)&c->beam64, &c->beam64_cap, sizeof(D8) * c->npix_beam, "beam64 buffer");
            if (st != PISCO_OK) return st;
            CK(launch_widen_beam(c->beam32, c->beam64, c->npix_beam, s), "widen beam");
            c->beam64_valid = true;
        }
        a.sky64 = c->sky64;
        a.beam64 = c->beam64;
        e = launch_forward_plain(a, true, c->sm_count, s);
    } else if (form == PISCO_FORM_TUNED &&
               tuned_supported(c->nside_beam, (int)c->npix_beam, c->rho_max)) {
        CK(cudaMemsetAsync(c->d_fallbacks, 0, sizeof(unsigned long long), s), "reset fallbacks");
        void* plans = nullptr;
        long long plan_cap = 0;
#if PISCO_FWD_PLANS
        c->plan_scratch(n, s, &plans, &plan_cap);
#endif
        e = launch_forward_tuned(a, c->sm_count, s, plans, plan_cap);
        if (plans) c->plans_used(s);
    } else {
        // PLAIN, and TUNED outside the tuned geometry's domain (a beam
        // reaching beyond the polar cap of its grid).
        e = launch_forward_plain(a, false, c->sm_count, s);
    }
    if (a.order) c->order_used(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "forward launch");
    if (s != c->stream) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(c->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    return PISCO_OK;
}

pisco_status pisco_memory_used(const pisco_ctx* c, size_t* bytes)
{
    if (!c || !bytes) return PISCO_ERR_INVALID_ARGUMENT;
    *bytes = c->mem_used;
    return PISCO_OK;
}

pisco_status pisco_sync(pisco_ctx* c)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    return c->check_device();
}

pisco_status pisco_forward(pisco_ctx* c, char polFlag, void* a, void* b, pisco_dtype out_dtype,
                           pisco_form form)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (polFlag != 'a' && polFlag != 'b' && polFlag != 'p')
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "valid polFlags are 'a', 'b' and 'p'");
    const bool wa = polFlag == 'a' || polFlag == 'p';
    const bool wb = polFlag == 'b' || polFlag == 'p';
    if ((wa && !a) || (wb && !b)) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "output array is NULL");
    if (out_dtype != PISCO_FLOAT32 && out_dtype != PISCO_FLOAT64)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad output dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    const long n = c->nsamples;
    if (n == 0) return PISCO_OK;
    const size_t esz = out_dtype == PISCO_FLOAT64 ? sizeof(double) : sizeof(float);
    // Outputs are produced in ptgPerConv chunks; each chunk's copy back
    // overlaps the next chunk's kernel on the same in-order stream pair.
    const long chunk = std::max<long>(1, std::min<long>(c->cfg.ptgPerConv, n));
    st = c->ensure(&c->out_dev, &c->out_cap, 2 * esz * (size_t)std::min<long>(n, 2 * chunk), "output buffer");
    if (st != PISCO_OK) return st;
    char* base = (char*)c->out_dev;
    const long slots = std::min<long>(n, 2 * chunk) / chunk >= 2 ? 2 : 1;
    for (long b0 = 0, k = 0; b0 < n; b0 += chunk, ++k) {
        const long m = std::min(chunk, n - b0);
        char* slot = base + (size_t)(k % slots) * 2 * esz * chunk;
        void* da = wa ? slot : nullptr;
        void* db = wb ? slot + esz * chunk : nullptr;
        st = pisco_forward_device(c, form, b0, m, da, db, out_dtype, c->stream);
        if (st != PISCO_OK) return st;
        if (wa) CK(cudaMemcpyAsync((char*)a + esz * b0, da, esz * m, cudaMemcpyDeviceToHost, c->stream), "TOD a D2H");
        if (wb) CK(cudaMemcpyAsync((char*)b + esz * b0, db, esz * m, cudaMemcpyDeviceToHost, c->stream), "TOD b D2H");
    }
    return c->check_device();
}

pisco_status pisco_count_pairs(pisco_ctx* c, long long* pairs)
{
    if (!c || !pairs) return PISCO_ERR_INVALID_ARGUMENT;
    if (!c->nside_sky || !c->nside_beam) return fail(c, PISCO_ERR_NOT_READY, "sky and beam required");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    if (!c->pairs_valid) {
        CK(cudaMemsetAsync(c->d_count, 0, sizeof(unsigned long long), c->stream), "reset count");
        CK(launch_count_pairs(c->nside_sky, c->rho_max, c->nsamples, c->ra, c->dec, c->d_count,
                              c->sm_count, c->stream),
           "count launch");
        unsigned long long v = 0;
        CK(cudaMemcpyAsync(&v, c->d_count, sizeof(v), cudaMemcpyDeviceToHost, c->stream), "count D2H");
        CK(cudaStreamSynchronize(c->stream), "count sync");
        c->pairs = (long long)v;
        c->pairs_valid = true;
    }
    *pairs = c->pairs;
    return PISCO_OK;
}

pisco_status pisco_last_fallbacks(pisco_ctx* c, long long* fallbacks)
{
    if (!c || !fallbacks) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, c->d_fallbacks, sizeof(v), cudaMemcpyDeviceToHost, c->stream), "fallbacks D2H");
    CK(cudaStreamSynchronize(c->stream), "fallbacks sync");
    *fallbacks = (long long)v;
    return PISCO_OK;
}

pisco_status pisco_tuned_calibrate(pisco_ctx* c, long begin, long n, double* worst,
                                   long long* tuned_pairs)
{
    if (!c || !worst) return PISCO_ERR_INVALID_ARGUMENT;
    if (!c->sky32 || !c->nside_sky || !c->beam32)
        return fail(c, PISCO_ERR_NOT_READY, "sky and beam required");
    if (begin < 0 || n < 0 || begin + n > c->nsamples)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "sample range outside the scan");
    if (!tuned_supported(c->nside_beam, (int)c->npix_beam, c->rho_max))
        return fail(c, PISCO_ERR_UNSUPPORTED, "beam outside the tuned form's domain");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    float* d = nullptr;  // {worst fraction, pad, u64 disc pairs of the TUNED disc}
    CK(cudaMalloc(&d, 16), "calib buffer");
    cudaMemsetAsync(d, 0, 16, c->stream);
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
    a.err = c->d_err;
    a.fallbacks = c->d_fallbacks;
    cudaError_t e = launch_tuned_calibrate(a, c->sm_count, c->stream, d);
    float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, d, 16, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(c, e, "calibration");
    *worst = v[0];
    unsigned long long pairs = 0;
    std::memcpy(&pairs, &v[2], sizeof(pairs));
    if (tuned_pairs) *tuned_pairs = (long long)pairs;
    return c->check_device();
}

}  // extern "C"
