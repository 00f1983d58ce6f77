// capi_batched.cu -- C ABI of the batched multi-detector forward and its
// autotuner (include/pisco_gb300.h: pisco_set_beam_slot,
// pisco_forward_batched, pisco_autotune_batched).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/pisco_gb300.h"
#include "ctx.h"
#include "internal.h"

using namespace pisco;

namespace {

constexpr int kMaxSlots = 1024;
constexpr int kMaxDets = 65536;

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

// Estimated pairs per sample of a detector: disc area / pixel area.
double disc_pairs(int nside_sky, double rho_max)
{
    return 12.0 * nside_sky * nside_sky * (1.0 - std::cos(rho_max)) / 2.0;
}

pisco_status validate(pisco_ctx* c, const pisco_det_desc* dets, int ndet, pisco_dtype out_dtype)
{
    if (!dets || ndet < 1 || ndet > kMaxDets)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "need 1..65536 detector descriptors");
    if (out_dtype != PISCO_FLOAT32 && out_dtype != PISCO_FLOAT64)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad output dtype");
    if (!c->sky32 || !c->nside_sky) return fail(c, PISCO_ERR_NOT_READY, "no sky set");
    for (int d = 0; d < ndet; ++d) {
        const pisco_det_desc& x = dets[d];
        if (x.beam_slot < 0 || x.beam_slot >= (int)c->slots.size() || !c->slots[x.beam_slot].beam)
            return fail(c, PISCO_ERR_NOT_READY, "detector " + std::to_string(d) + ": beam slot not set");
        if (x.nsamples < 0 || x.nsamples > (1LL << 40))
            return fail(c, PISCO_ERR_INVALID_ARGUMENT, "detector " + std::to_string(d) + ": bad nsamples");
        if (x.nsamples > 0 && (!x.ra || !x.dec || !x.pa))
            return fail(c, PISCO_ERR_INVALID_ARGUMENT, "detector " + std::to_string(d) + ": NULL pointing");
        if (x.flags & ~PISCO_DET_SKY_ORDER)
            return fail(c, PISCO_ERR_INVALID_ARGUMENT, "detector " + std::to_string(d) + ": unknown flags");
        const auto& s = c->slots[x.beam_slot];
        if (!tuned_supported(s.nside, (int)s.npix, s.rho_max))
            return fail(c, PISCO_ERR_UNSUPPORTED,
                        "detector " + std::to_string(d) + ": beam outside the TUNED domain");
    }
    return PISCO_OK;
}

std::string launch_key(pisco_ctx* c, const pisco_det_desc* dets, int ndet, pisco_dtype out_dtype,
                       int chunk, int warps, const void* plans)
{
    std::string k((const char*)dets, sizeof(pisco_det_desc) * (size_t)ndet);
    char tail[160];
    std::snprintf(tail, sizeof tail, "|%d|%d|%d|%p|%d|%d|%p", chunk, warps, (int)out_dtype,
                  (void*)c->sky32, c->nside_sky, (int)c->interp, plans);
    return k + tail;
}

// Sample plans of a batched launch: all its detectors' samples at once, up
// to 16M (1.5 GB of scratch); a larger launch plans in its warps.
constexpr long long kBatchPlans = 1LL << 24;

// One autotuned choice: chunk, warps per block, time.
struct Tuned {
    int chunk;
    int warps;
    double ms;
};

// ---- a flat JSON object {"key": [chunk, ms, warps], ...} -------------------
std::map<std::string, Tuned> read_cache(const char* path)
{
    std::map<std::string, Tuned> m;
    std::ifstream f(path);
    if (!f) return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    size_t p = 0;
    while ((p = s.find('"', p)) != std::string::npos) {
        const size_t q = s.find('"', p + 1);
        if (q == std::string::npos) break;
        const std::string key = s.substr(p + 1, q - p - 1);
        const size_t lb = s.find('[', q), rb = s.find(']', q);
        if (lb == std::string::npos || rb == std::string::npos || lb > rb) break;
        int chunk = 0, warps = 8;
        double ms = 0.0;
        const int got = std::sscanf(s.c_str() + lb + 1, "%d , %lf , %d", &chunk, &ms, &warps);
        if (got >= 2 && chunk > 0)
            m[key] = Tuned{chunk, got == 3 && batched_warps_valid(warps) ? warps : 8, ms};
        p = rb + 1;
    }
    return m;
}

bool write_cache(const char* path, const std::map<std::string, Tuned>& m)
{
    const std::string tmp = std::string(path) + ".tmp";
    std::ofstream f(tmp);
    if (!f) return false;
    f << "{\n";
    size_t i = 0;
    for (const auto& kv : m)
        f << "  \"" << kv.first << "\": [" << kv.second.chunk << ", " << kv.second.ms << ", "
          << kv.second.warps << "]"
          << (++i < m.size() ? ",\n" : "\n");
    f << "}\n";
    f.close();
    return std::rename(tmp.c_str(), path) == 0;
}

}  // namespace

extern "C" {

pisco_status pisco_set_beam_slot(pisco_ctx* c, int slot, int nside, long npix, const void* const a[4],
                                 const void* const b[4], pisco_dtype dt)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (slot < 0 || slot >= kMaxSlots) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "slot must be in [0, 1024)");
    if (nside < 1 || nside > 8192) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nside must be in [1, 8192]");
    if (npix < 1 || npix >= 12L * nside * nside)
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam nPixels must be in [1, 12 nside^2)");
    if (!a || !b) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam plane arrays are NULL");
    for (int k = 0; k < 4; ++k)
        if (!a[k] || !b[k]) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "beam plane is NULL");
    if (dt != PISCO_FLOAT32 && dt != PISCO_FLOAT64) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "bad dtype");
    pisco_status st = c->activate();
    if (st != PISCO_OK) return st;
    std::vector<F8> t(npix);
    for (long i = 0; i < npix; ++i) {
        float fa[4], fb[4];
        for (int k = 0; k < 4; ++k) {
            fa[k] = dt == PISCO_FLOAT32 ? ((const float*)a[k])[i] : (float)((const double*)a[k])[i];
            fb[k] = dt == PISCO_FLOAT32 ? ((const float*)b[k])[i] : (float)((const double*)b[k])[i];
        }
        t[i].a = make_float4(fa[0], fa[1], fa[2], fa[3]);
        t[i].b = make_float4(fb[0], fb[1], fb[2], fb[3]);
    }
    if ((int)c->slots.size() <= slot) c->slots.resize(slot + 1);
    auto& s = c->slots[slot];
    st = c->ensure((void**)&s.beam, &s.cap, sizeof(F8) * npix, "beam slot");
    if (st != PISCO_OK) return st;
    CK(cudaMemcpyAsync(s.beam, t.data(), sizeof(F8) * npix, cudaMemcpyHostToDevice, c->stream), "beam slot H2D");
    CK(cudaStreamSynchronize(c->stream), "beam slot upload");
    s.nside = nside;
    s.npix = npix;
    s.rho_max = pisco_beam_rho_max(nside, npix);
    c->graph_key.clear();
    return PISCO_OK;
}

pisco_status pisco_forward_batched(pisco_ctx* c, const pisco_det_desc* dets, int ndet,
                                   pisco_dtype out_dtype, int chunk, void* stream)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = validate(c, dets, ndet, out_dtype);
    if (st != PISCO_OK) return st;
    if (chunk < 0) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "chunk must be >= 0");
    if (chunk == 0) chunk = c->batched_chunk > 0 ? c->batched_chunk : 256;
    const int warps = c->batched_warps;
    st = c->activate();
    if (st != PISCO_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    // every detector's sample plans in one scratch (planned launch), if it
    // fits: the graph below holds its address, so the key names it
    long long total = 0;
    for (int d = 0; d < ndet; ++d) total += dets[d].nsamples;
    void* plans = nullptr;
    auto take_plans = [&]() {
        long long plan_cap = 0;
        plans = nullptr;
        if (total > 0) c->plan_scratch(total, s, &plans, &plan_cap, kBatchPlans);
        if (plan_cap < total) plans = nullptr;
    };
    take_plans();
    std::string key = launch_key(c, dets, ndet, out_dtype, chunk, warps, plans);
    if (!(c->graph_exec && key == c->graph_key)) {
        // the descriptors, items and orders below may still be read by the
        // previous launch (on another stream)
        if (c->batch_event) CK(cudaStreamWaitEvent(c->stream, c->batch_event, 0), "batch wait");
        std::vector<BatchDet> bd(ndet);
        std::vector<double> cost(ndet);
        if ((int)c->det_ord.size() < ndet) {
            c->det_ord.resize(ndet, nullptr);
            c->det_ord_cap.resize(ndet, 0);
        }
        for (int d = 0; d < ndet; ++d) {
            const auto& sl = c->slots[dets[d].beam_slot];
            const int* order = nullptr;
            if ((dets[d].flags & PISCO_DET_SKY_ORDER) && dets[d].nsamples >= 2 &&
                dets[d].nsamples <= 0x7fffffffLL) {
                st = c->make_order(dets[d].ra, dets[d].dec, dets[d].nsamples, &c->det_ord[d],
                                   &c->det_ord_cap[d], c->stream);
                if (st != PISCO_OK) return st;
                order = c->det_ord[d];
            }
            bd[d] = BatchDet{sl.beam, sl.nside, (int)sl.npix, sl.rho_max,
                             (float)(1.7320508075688772 * sl.nside), dets[d].nsamples,
                             dets[d].ra, dets[d].dec, dets[d].pa, dets[d].tod_a, dets[d].tod_b,
                             order};
            cost[d] = disc_pairs(c->nside_sky, sl.rho_max);
        }
        long long base = 0;
        for (int d = 0; d < ndet; ++d) {
            bd[d].plan_base = base;
            base += dets[d].nsamples;
        }
        const std::vector<BatchItem> items = make_items(bd, cost, chunk);
        if (items.size() > (size_t)0x7fffffff) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "too many queue items");
        st = c->ensure((void**)&c->d_dets, &c->d_dets_cap, sizeof(BatchDet) * ndet, "batch descriptors");
        if (st == PISCO_OK)
            st = c->ensure((void**)&c->d_items, &c->d_items_cap,
                           sizeof(BatchItem) * std::max<size_t>(items.size(), 1), "batch items");
        size_t qcap = c->d_queue ? sizeof(unsigned int) : 0;
        if (st == PISCO_OK) st = c->ensure((void**)&c->d_queue, &qcap, sizeof(unsigned int), "batch queue");
        if (st != PISCO_OK) return st;
        // the buffers above may have freed the plan scratch (it yields to
        // them): take it again, after them, and key the graph on it
        take_plans();
        key = launch_key(c, dets, ndet, out_dtype, chunk, warps, plans);
        CK(cudaMemcpyAsync(c->d_dets, bd.data(), sizeof(BatchDet) * ndet, cudaMemcpyHostToDevice, c->stream),
           "descriptors H2D");
        if (!items.empty())
            CK(cudaMemcpyAsync(c->d_items, items.data(), sizeof(BatchItem) * items.size(),
                               cudaMemcpyHostToDevice, c->stream),
               "items H2D");
        CK(cudaStreamSynchronize(c->stream), "batch upload");
        BatchArgs a;
        a.nside_sky = c->nside_sky;
        a.sky32 = c->sky32;
        a.rings = c->rings;
        a.dets = c->d_dets;
        a.ndet = ndet;
        a.items = c->d_items;
        a.nitems = (int)items.size();
        a.queue = c->d_queue;
        a.out_f64 = out_dtype == PISCO_FLOAT64;
        a.err = c->d_err;
        a.fallbacks = c->d_fallbacks;
        a.interp = (int)c->interp;
        a.plans = static_cast<tuned::SamplePlan*>(plans);
        a.nplans = plans ? total : 0;
        // capture (queue reset + plan kernel + kernel) once; replays reuse it
        if (c->graph_exec) {
            cudaGraphExecDestroy(c->graph_exec);
            c->graph_exec = nullptr;
            c->graph_key.clear();
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        cudaError_t e1 = cudaMemsetAsync(c->d_queue, 0, sizeof(unsigned int), c->stream);
        cudaError_t e2 = e1 == cudaSuccess
                             ? launch_batched(a, c->sm_count, c->stream, warps)
                             : e1;
        cudaError_t e3 = cudaStreamEndCapture(c->stream, &g);
        if (e2 != cudaSuccess || e3 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(c, e2 != cudaSuccess ? e2 : e3, "batched capture");
        }
        cudaError_t e4 = cudaGraphInstantiate(&c->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e4 != cudaSuccess) {
            c->graph_exec = nullptr;
            return cuda_fail(c, e4, "graph instantiate");
        }
        c->graph_key = key;
    }
    CK(cudaGraphLaunch(c->graph_exec, s), "graph launch");
    if (plans) c->plans_used(s);
    if (!c->batch_event) CK(cudaEventCreateWithFlags(&c->batch_event, cudaEventDisableTiming), "event");
    CK(cudaEventRecord(c->batch_event, s), "batch event");
    return PISCO_OK;
}

pisco_status pisco_batched_config(pisco_ctx* c, int* chunk, int* warps_per_block)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (chunk) *chunk = c->batched_chunk > 0 ? c->batched_chunk : 256;
    if (warps_per_block) *warps_per_block = c->batched_warps;
    return PISCO_OK;
}

pisco_status pisco_set_batched_config(pisco_ctx* c, int chunk, int warps_per_block)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    if (chunk < 0) return fail(c, PISCO_ERR_INVALID_ARGUMENT, "chunk must be >= 0");
    if (!batched_warps_valid(warps_per_block))
        return fail(c, PISCO_ERR_INVALID_ARGUMENT, "warps per block must be 4, 8 or 16");
    if (chunk > 0) c->batched_chunk = chunk;
    c->batched_warps = warps_per_block;
    return PISCO_OK;
}

pisco_status pisco_autotune_batched(pisco_ctx* c, const pisco_det_desc* dets, int ndet,
                                    pisco_dtype out_dtype, const char* cache_path, int* chunk_out,
                                    double* ms_out)
{
    if (!c) return PISCO_ERR_INVALID_ARGUMENT;
    pisco_status st = validate(c, dets, ndet, out_dtype);
    if (st != PISCO_OK) return st;
    st = c->activate();
    if (st != PISCO_OK) return st;
    // workload key: device, sky nside, sorted beam geometries, sample scale, form
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, c->device), "device properties");
    std::vector<std::pair<int, long>> beams;
    long long total = 0;
    for (int d = 0; d < ndet; ++d) {
        beams.emplace_back(c->slots[dets[d].beam_slot].nside, c->slots[dets[d].beam_slot].npix);
        total += dets[d].nsamples;
    }
    std::sort(beams.begin(), beams.end());
    unsigned long long h = 1469598103934665603ULL;  // FNV-1a of the beam set
    for (auto& b : beams) {
        for (unsigned long long v : {(unsigned long long)b.first, (unsigned long long)b.second}) {
            h ^= v;
            h *= 1099511628211ULL;
        }
    }
    char key[512];
    std::snprintf(key, sizeof key, "%s|nside_sky=%d|ndet=%d|beams=%016llx|log2n=%d|%s|%s|tuned",
                  prop.name, c->nside_sky, ndet, h, (int)std::log2((double)std::max<long long>(total, 1)),
                  out_dtype == PISCO_FLOAT64 ? "f64" : "f32",
                  c->interp == PISCO_BEAM_BILINEAR ? "bilinear" : "nearest");
    std::map<std::string, Tuned> cache;
    if (cache_path) {
        cache = read_cache(cache_path);
        auto it = cache.find(key);
        if (it != cache.end()) {
            c->batched_chunk = it->second.chunk;
            c->batched_warps = it->second.warps;
            if (chunk_out) *chunk_out = it->second.chunk;
            if (ms_out) *ms_out = it->second.ms;
            return PISCO_OK;
        }
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    int best = 256, best_w = 8;
    double best_ms = 1e300;
    const int keep_w = c->batched_warps;
    for (int warps : {8, 16, 4}) {
        c->batched_warps = warps;
        for (int chunk : {32, 64, 128, 256, 512, 1024, 2048, 4096, 8192}) {
            st = pisco_forward_batched(c, dets, ndet, out_dtype, chunk, c->stream);  // warm-up + capture
            if (st != PISCO_OK) break;
            double ms = 1e300;
            for (int rep = 0; rep < 2 && st == PISCO_OK; ++rep) {
                cudaEventRecord(e0, c->stream);
                st = pisco_forward_batched(c, dets, ndet, out_dtype, chunk, c->stream);
                cudaEventRecord(e1, c->stream);
                cudaEventSynchronize(e1);
                float t = 0.0f;
                cudaEventElapsedTime(&t, e0, e1);
                ms = std::min(ms, (double)t);
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = chunk;
                best_w = warps;
            }
        }
        if (st != PISCO_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != PISCO_OK) {
        c->batched_warps = keep_w;
        return st;
    }
    st = c->check_device();
    if (st != PISCO_OK) return st;
    c->batched_chunk = best;
    c->batched_warps = best_w;
    if (cache_path) {
        cache[key] = Tuned{best, best_w, best_ms};
        if (!write_cache(cache_path, cache))
            return fail(c, PISCO_ERR_INVALID_ARGUMENT, std::string("cannot write ") + cache_path);
    }
    if (chunk_out) *chunk_out = best;
    if (ms_out) *ms_out = best_ms;
    return PISCO_OK;
}

}  // extern "C"
