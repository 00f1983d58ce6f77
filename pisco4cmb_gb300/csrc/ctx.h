// ctx.h -- the context behind the opaque pisco_ctx handle.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pisco_gb300.h"
#include "internal.h"

namespace pisco {
std::vector<BatchItem> make_items(const std::vector<BatchDet>& dets, const std::vector<double>& cost,
                                  long long chunk);
}

struct pisco_ctx {
    pisco_run_config cfg{};
    int device = 0;
    int sm_count = 1;
    cudaStream_t stream = nullptr;
    std::string error;
    size_t mem_used = 0;

    // sky (RING, interleaved IQUV)
    int nside_sky = 0;
    float4* sky32 = nullptr;
    size_t sky32_cap = 0;
    pisco::D4* sky64 = nullptr;
    size_t sky64_cap = 0;
    bool sky64_valid = false;
    // ring table of the sky grid (allocated once for the largest nside, so
    // its address never changes; rebuilt when nside changes)
    pisco::RingT* rings = nullptr;
    size_t rings_cap = 0;
    int rings_nside = 0;

    // beam (partial RING map around the north pole, a|b interleaved)
    int nside_beam = 0;
    long npix_beam = 0;
    double rho_max = 0.0;
    pisco::F8* beam32 = nullptr;
    size_t beam32_cap = 0;
    pisco::D8* beam64 = nullptr;
    size_t beam64_cap = 0;
    bool beam64_valid = false;
    pisco_interp interp = PISCO_BEAM_NEAREST;

    // scan (FP64 structure of arrays)
    long nsamples = 0;
    double* ra = nullptr;
    double* dec = nullptr;
    double* pa = nullptr;
    size_t ra_cap = 0, dec_cap = 0, pa_cap = 0;

    // sample order (pisco_set_sample_order): the sky order of the last
    // forward/adjoint range, cached until the scan or the range changes
    int sample_order = 0;  // pisco_order
    long long scan_version = 0;
    int* ord = nullptr;
    size_t ord_cap = 0;
    long long ord_begin = -1, ord_n = -1, ord_version = -1;
    cudaEvent_t ord_event = nullptr;  // recorded after the last write or read of ord
    unsigned* ord_keys = nullptr;
    size_t ord_keys_cap = 0;
    unsigned* ord_keys2 = nullptr;
    size_t ord_keys2_cap = 0;
    int* ord_pos = nullptr;
    size_t ord_pos_cap = 0;
    void* ord_tmp = nullptr;
    size_t ord_tmp_cap = 0;
    std::vector<int*> det_ord;  // batched: per-descriptor orders
    std::vector<size_t> det_ord_cap;
    cudaEvent_t batch_event = nullptr;  // recorded after the last batched launch

    // per-sample plans of the TUNED forward (scratch of the plan kernel) and
    // the event recorded after their last use
    void* plans = nullptr;
    size_t plans_cap = 0;
    cudaEvent_t plan_event = nullptr;

    // staging and bookkeeping
    void* out_dev = nullptr;
    size_t out_cap = 0;
    unsigned int* d_err = nullptr;
    unsigned long long* d_count = nullptr;
    unsigned long long* d_fallbacks = nullptr;
    long long pairs = 0;
    bool pairs_valid = false;

    // batched multi-detector forward
    struct BeamSlot {
        pisco::F8* beam = nullptr;
        size_t cap = 0;
        int nside = 0;
        long npix = 0;
        double rho_max = 0.0;
    };
    std::vector<BeamSlot> slots;
    pisco::BatchDet* d_dets = nullptr;
    size_t d_dets_cap = 0;
    pisco::BatchItem* d_items = nullptr;
    size_t d_items_cap = 0;
    unsigned int* d_queue = nullptr;
    // graph of the last batched launch (queue reset + kernel) and its key
    cudaGraphExec_t graph_exec = nullptr;
    std::string graph_key;
    int batched_chunk = 0;  // last autotuned chunk (0 = not tuned)
    int batched_warps = 8;  // warps per block of the batched kernel (autotuned)

    // adjoint scratch
    float* adj_sky32 = nullptr;
    size_t adj_sky32_cap = 0;
    float* adj_beam32 = nullptr;
    size_t adj_beam32_cap = 0;
    unsigned long long* adj_sky_fx = nullptr;
    size_t adj_sky_fx_cap = 0;
    unsigned long long* adj_beam_fx = nullptr;
    size_t adj_beam_fx_cap = 0;
    double* red = nullptr;
    size_t red_cap = 0;
    // fused Gaussian beam-parameter gradient: model table, partial sums
    float* adj_ptab = nullptr;
    size_t adj_ptab_cap = 0;
    double* adj_ppart = nullptr;
    size_t adj_ppart_cap = 0;

    // device beam construction scratch (block partials, results, weights)
    double* beam_scr = nullptr;
    size_t beam_scr_cap = 0;

    ~pisco_ctx();
    pisco_status activate();
    pisco_status ensure(void** p, size_t* cap, size_t bytes, const char* what);
    // ring table for nside_sky, built on stream s if nside changed
    pisco_status ensure_rings(cudaStream_t s);
    // sky order of n pointings into *buf (n ints, grown as needed), on s
    pisco_status make_order(const double* ra, const double* dec, long long n, int** buf,
                            size_t* cap, cudaStream_t s);
    // order of samples [begin, begin + n) of the scan for a launch on s:
    // null in scan order (or n < 2 or n >= 2^31), else the cached or new
    // sky order.  Stream s first waits for the previous access to the order
    // buffer; a launch that reads it calls order_used(s) afterwards.
    pisco_status range_order(long long begin, long long n, cudaStream_t s, const int** out);
    void order_used(cudaStream_t s);
    // Scratch for the TUNED forward's sample plans, for up to n samples (at
    // most kPlanChunk at a time), ordered after their last use on stream s;
    // *p = null when it does not fit within maxMemUsage or the device (the
    // warps then build their own plans).  A launch that reads them calls
    // plans_used(s) afterwards.
    void plan_scratch(long long n, cudaStream_t s, void** p, long long* cap,
                      long long max_plans = 1LL << 22);
    void plans_used(cudaStream_t s);
    pisco_status check_device();
};
