/* HEALPix C++ compatibility shim (TEST INFRASTRUCTURE ONLY).
 * Healpix_Base (RING scheme only) implemented on the oracle's C
 * restatement of the HEALPix algorithms (oracle/oracle.c). */
#ifndef PISCO_SHIM_HEALPIX_BASE_H
#define PISCO_SHIM_HEALPIX_BASE_H
#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <vector>
#include "arr.h"
#include "pointing.h"
#include "rangeset.h"
#include "oracle.h"

enum Healpix_Ordering_Scheme { RING, NEST };
enum nside_dummy { SET_NSIDE };

class Healpix_Base {
    orc_hpx h;
  public:
    Healpix_Base() { orc_hpx_init(&h, 1); }
    Healpix_Base(int nside, Healpix_Ordering_Scheme s, const nside_dummy) {
        if (s != RING) throw std::invalid_argument("shim supports RING only");
        orc_hpx_init(&h, nside);
    }
    int Nside() const { return (int)h.nside; }
    int Npix() const { return (int)h.npix; }
    pointing pix2ang(int pix) const {
        pointing p;
        orc_pix2ang(&h, pix, &p.theta, &p.phi);
        return p;
    }
    int ang2pix(const pointing& p) const { return (int)orc_ang2pix(&h, p.theta, p.phi); }
    void query_disc(pointing p, double radius, rangeset<int>& out) const {
        std::vector<int64_t> rg(2 * (8 * h.nside + 8));
        int64_t n = orc_query_disc(&h, p.theta, p.phi, radius, rg.data(), (int64_t)rg.size() / 2);
        out.clear();
        for (int64_t i = 0; i < n; ++i) out.append((int)rg[2 * i], (int)rg[2 * i + 1]);
    }
    void get_interpol(const pointing& p, fix_arr<int, 4>& pix, fix_arr<double, 4>& wgt) const {
        int64_t px[4];
        double w[4];
        orc_get_interpol(&h, p.theta, p.phi, px, w);
        for (int i = 0; i < 4; ++i) {
            pix[i] = (int)px[i];
            wgt[i] = w[i];
        }
    }
};
#endif
