// PolBeam -- polarized beam of a detector pair as partial RING maps around
// the north pole; same interface as the reference (src/Polbeam/polbeam.hpp:23-93).
// Owns its buffers.  The construction arithmetic runs in libpisco_gb300
// (pisco_beam_* entry points) and is bit-identical to the reference's.
#ifndef PISCO_POLBEAM_HPP
#define PISCO_POLBEAM_HPP

#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "../pisco_detail.hpp"

class PolBeam {
  public:
    PolBeam(int _nside, long _nPixels, double _epsilon, char _enabledDets)
        : nside(_nside), nPixels(_nPixels), hpxBase(_nside), enabledDets(_enabledDets),
          epsilon(_epsilon)
    {
        if (_enabledDets != 'a' && _enabledDets != 'b' && _enabledDets != 'p')
            throw std::invalid_argument("enabledDets must be 'a', 'b' or 'p'");
        rhoMax = pisco_beam_rho_max(_nside, _nPixels);
        if (rhoMax < 0.0) throw std::invalid_argument("nPixels outside the beam grid");
        store.assign(16 * (size_t)nPixels, 0.0f);
        float* p = store.data();
        for (int k = 0; k < 4; ++k) aBeams[k] = p + (size_t)k * nPixels;
        for (int k = 0; k < 4; ++k) bBeams[k] = p + (size_t)(4 + k) * nPixels;
        Ia = p + 8 * (size_t)nPixels;
        Qa = p + 9 * (size_t)nPixels;
        Ua = p + 10 * (size_t)nPixels;
        Va = p + 11 * (size_t)nPixels;
        Ib = p + 12 * (size_t)nPixels;
        Qb = p + 13 * (size_t)nPixels;
        Ub = p + 14 * (size_t)nPixels;
        Vb = p + 15 * (size_t)nPixels;
    }
    ~PolBeam() {}
    PolBeam(const PolBeam&) = delete;
    PolBeam& operator=(const PolBeam&) = delete;

    int get_nside() const { return nside; }
    unsigned long size() const { return (unsigned long)nPixels; }
    double get_rho_max() const { return rhoMax; }

    void beam_from_fields(char polFlag, double* magEco, double* phsEco, double* magEcx,
                          double* phsEcx)
    {
        float *I, *Q, *U, *V;
        if (polFlag == 'a') {
            I = Ia; Q = Qa; U = Ua; V = Va;
        } else if (polFlag == 'b') {
            I = Ib; Q = Qb; U = Ub; V = Vb;
        } else {
            throw std::invalid_argument("polFlag must be 'a' or 'b'");
        }
        pisco_detail::check(pisco_beam_from_fields(nPixels, magEco, phsEco, magEcx, phsEcx, I, Q, U, V),
                            nullptr, "PolBeam::beam_from_fields");
    }

    void build(int nsideSky)
    {
        const float* ta[4] = {Ia, Qa, Ua, Va};
        const float* tb[4] = {Ib, Qb, Ub, Vb};
        pisco_detail::check(pisco_beam_build(nside, nPixels, epsilon, enabledDets, nsideSky, ta, tb,
                                             aBeams, bBeams),
                            nullptr, "PolBeam::build");
    }

    void make_unpol_gaussian_elliptical_beams(double fwhmx, double fwhmy, double phi0)
    {
        std::vector<double> f(4 * (size_t)nPixels);
        double* m0 = f.data();
        double* p0 = m0 + nPixels;
        double* m1 = p0 + nPixels;
        double* p1 = m1 + nPixels;
        pisco_detail::check(pisco_beam_gaussian_fields(nside, nPixels, fwhmx, fwhmy, phi0, m0, p0, m1, p1),
                            nullptr, "PolBeam::make_unpol_gaussian_elliptical_beams");
        if (enabledDets == 'a' || enabledDets == 'p') beam_from_fields('a', m0, p0, m1, p1);
        if (enabledDets == 'b' || enabledDets == 'p') beam_from_fields('b', m0, p0, m1, p1);
    }

    float* aBeams[4];
    float* bBeams[4];
    int nside;
    long nPixels;
    PiscoHealpixBase hpxBase;
    char enabledDets;
    float *Ia, *Qa, *Ua, *Va;
    float *Ib, *Qb, *Ub, *Vb;

  private:
    double rhoMax;
    double epsilon;
    std::vector<float> store;
};

#endif
