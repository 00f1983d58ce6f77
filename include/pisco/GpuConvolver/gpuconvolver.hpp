// GPUConvolver -- the reference's GPU drop-in interface
// (src/GpuConvolver/gpuconvolver.hpp:17-82) on libpisco_gb300 (sm_103a).
//
// Same calls and order: construct with a RunConfig, configure_execution(),
// update_beam/update_sky/update_scan (each copies to the device),
// exec_convolution(data_a, data_b) computes both detectors.  Differences on
// purpose: every sample is computed (the reference drops the tail,
// gpuconvolver.cu:386); CUDA failures throw std::runtime_error instead of
// exit(-1); the default form is TUNED (FP32 per-pair geometry with FP64
// pointing and an FP64 re-evaluation of every near-edge pixel decision; a
// beam outside its domain is convolved by the PLAIN chain automatically);
// set_form() selects PLAIN (the reference's per-pair chain), TUNED or FP64.
#ifndef PISCO_GPUCONVOLVER_HPP
#define PISCO_GPUCONVOLVER_HPP

#include <cstring>
#include <stdexcept>

#include "../Polbeam/polbeam.hpp"
#include "../Scan/scan.hpp"
#include "../Sky/sky.hpp"
#include "../pisco_detail.hpp"
#include "cuda/cudaConv2.h"

class GPUConvolver {
  public:
    explicit GPUConvolver(CUDACONV::RunConfig cfg_) : ctx(nullptr), nsamples(0), form(PISCO_FORM_TUNED)
    {
        std::memcpy(&cfg, &cfg_, sizeof(cfg));
    }
    ~GPUConvolver()
    {
        if (ctx) pisco_destroy(ctx);
    }
    GPUConvolver(const GPUConvolver&) = delete;
    GPUConvolver& operator=(const GPUConvolver&) = delete;

    void configure_execution(void)
    {
        if (ctx) return;
        pisco_detail::check(pisco_create(&cfg, &ctx), nullptr, "GPUConvolver::configure_execution");
    }
    void update_beam(PolBeam* beam)
    {
        need_ctx();
        const void* a[4] = {beam->aBeams[0], beam->aBeams[1], beam->aBeams[2], beam->aBeams[3]};
        const void* b[4] = {beam->bBeams[0], beam->bBeams[1], beam->bBeams[2], beam->bBeams[3]};
        pisco_detail::check(pisco_set_beam(ctx, beam->get_nside(), (long)beam->size(), a, b, PISCO_FLOAT32),
                            ctx, "GPUConvolver::update_beam");
    }
    void update_sky(Sky* sky)
    {
        need_ctx();
        pisco_detail::check(pisco_set_sky(ctx, sky->get_nside(), sky->sI, sky->sQ, sky->sU, sky->sV,
                                          PISCO_FLOAT32),
                            ctx, "GPUConvolver::update_sky");
    }
    void update_scan(Scan* scan)
    {
        need_ctx();
        nsamples = scan->get_nsamples();
        pisco_detail::check(pisco_set_scan(ctx, nsamples, scan->get_ra_ptr(), scan->get_dec_ptr(),
                                           scan->get_pa_ptr(), PISCO_FLOAT32),
                            ctx, "GPUConvolver::update_scan");
    }
    void exec_convolution(float* data_a, float* data_b)
    {
        need_ctx();
        pisco_detail::check(pisco_forward(ctx, 'p', data_a, data_b, PISCO_FLOAT32, form), ctx,
                            "GPUConvolver::exec_convolution");
    }
    void set_form(pisco_form f) { form = f; }
    // PISCO_ORDER_SKY: each launch processes its samples sorted by sky cell
    // (TOD unchanged, still in scan order); after configure_execution().
    void set_sample_order(pisco_order order)
    {
        need_ctx();
        pisco_detail::check(pisco_set_sample_order(ctx, order), ctx, "GPUConvolver::set_sample_order");
    }
    pisco_ctx* handle() { return ctx; }

  private:
    void need_ctx()
    {
        if (!ctx) throw std::invalid_argument("GPUConvolver: call configure_execution() first");
    }
    pisco_run_config cfg;
    pisco_ctx* ctx;
    long nsamples;
    pisco_form form;
};

#endif
