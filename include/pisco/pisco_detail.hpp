// pisco_detail.hpp -- shared helpers of the header-only C++ drop-in classes
// (Scan, Sky, PolBeam, Convolver, GPUConvolver) over the C ABI of
// libpisco_gb300.so.  C-ABI status codes become the exceptions the
// reference throws: std::invalid_argument for argument/config errors,
// std::runtime_error for CUDA failures (the reference exits instead).
#ifndef PISCO_DETAIL_HPP
#define PISCO_DETAIL_HPP

#include <stdexcept>
#include <string>

#include "../pisco_gb300.h"

namespace pisco_detail {

inline void check(pisco_status s, const pisco_ctx* ctx, const char* what)
{
    if (s == PISCO_OK) return;
    std::string msg = std::string(what) + ": " + pisco_last_error(ctx) + " (" +
                      pisco_status_string(s) + ")";
    if (s == PISCO_ERR_INVALID_ARGUMENT || s == PISCO_ERR_INVALID_CONFIG)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

}  // namespace pisco_detail

// Minimal stand-ins for the Healpix C++ types the reference exposes as
// public members (Sky::hpxBase, PolBeam::hpxBase), RING scheme only.
struct pisco_pointing {
    double theta, phi;
};

class PiscoHealpixBase {
    int nside_;

  public:
    explicit PiscoHealpixBase(int nside = 1) : nside_(nside) {}
    int Nside() const { return nside_; }
    long Npix() const { return 12L * nside_ * nside_; }
    pisco_pointing pix2ang(long pix) const
    {
        pisco_pointing p;
        pisco_detail::check(pisco_hpx_pix2ang(nside_, 1, &pix, &p.theta, &p.phi), nullptr, "pix2ang");
        return p;
    }
    long ang2pix(const pisco_pointing& p) const
    {
        long pix = 0;
        pisco_detail::check(pisco_hpx_ang2pix(nside_, 1, &p.theta, &p.phi, &pix), nullptr, "ang2pix");
        return pix;
    }
};

#endif
