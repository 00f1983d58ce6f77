// ctx.h -- the context behind the opaque pisco_ctx handle.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/pisco_gb300.h"
#include "internal.h"

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

    // staging and bookkeeping
    void* out_dev = nullptr;
    size_t out_cap = 0;
    unsigned int* d_err = nullptr;
    unsigned long long* d_count = nullptr;
    unsigned long long* d_fallbacks = nullptr;
    long long pairs = 0;
    bool pairs_valid = false;

    ~pisco_ctx();
    pisco_status activate();
    pisco_status ensure(void** p, size_t* cap, size_t bytes, const char* what);
    pisco_status check_device();
};
