// Convolver -- the reference's convolution interface
// (src/Convolver/convolver.hpp:14-36).  exec_convolution(polFlag, a, b) runs
// on the GPU (PLAIN form) through libpisco_gb300; a bad polFlag throws
// std::invalid_argument("valid polFlags are 'a', 'b' and 'p'") as the
// reference does (convolver.cpp:66-70), before any work starts.
#ifndef PISCO_CONVOLVER_HPP
#define PISCO_CONVOLVER_HPP

#include <stdexcept>

#include "../Polbeam/polbeam.hpp"
#include "../Scan/scan.hpp"
#include "../Sky/sky.hpp"
#include "../pisco_detail.hpp"

class Convolver {
  public:
    Convolver(Scan* scan_, Sky* sky_, PolBeam* beam_) : scan(scan_), sky(sky_), beam(beam_) {}
    ~Convolver() {}

    void exec_convolution(char polFlag, float* data_a, float* data_b)
    {
        if (polFlag != 'a' && polFlag != 'b' && polFlag != 'p')
            throw std::invalid_argument("valid polFlags are 'a', 'b' and 'p'");
        pisco_ctx* ctx = nullptr;
        pisco_detail::check(pisco_create(nullptr, &ctx), nullptr, "Convolver");
        struct Guard {
            pisco_ctx* c;
            ~Guard() { pisco_destroy(c); }
        } guard{ctx};
        pisco_detail::check(pisco_set_sky(ctx, sky->get_nside(), sky->sI, sky->sQ, sky->sU, sky->sV,
                                          PISCO_FLOAT32),
                            ctx, "Convolver::update_sky");
        const void* a[4] = {beam->aBeams[0], beam->aBeams[1], beam->aBeams[2], beam->aBeams[3]};
        const void* b[4] = {beam->bBeams[0], beam->bBeams[1], beam->bBeams[2], beam->bBeams[3]};
        pisco_detail::check(pisco_set_beam(ctx, beam->get_nside(), (long)beam->size(), a, b, PISCO_FLOAT32),
                            ctx, "Convolver::update_beam");
        pisco_detail::check(pisco_set_scan(ctx, scan->get_nsamples(), scan->get_ra_ptr(),
                                           scan->get_dec_ptr(), scan->get_pa_ptr(), PISCO_FLOAT32),
                            ctx, "Convolver::update_scan");
        pisco_detail::check(pisco_forward(ctx, polFlag, data_a, data_b, PISCO_FLOAT32, PISCO_FORM_PLAIN),
                            ctx, "Convolver::exec_convolution");
    }

  private:
    Scan* scan;
    Sky* sky;
    PolBeam* beam;
};

#endif
