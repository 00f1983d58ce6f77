// Sky -- non-owning view of I, Q, U, V RING maps, same interface as the
// reference (src/Sky/sky.hpp:12-38).  hpxBase is a RING-only stand-in for
// the Healpix_Base member.
#ifndef PISCO_SKY_HPP
#define PISCO_SKY_HPP

#include "../pisco_detail.hpp"

class Sky {
  public:
    Sky(int nside_, const float* I, const float* Q, const float* U, const float* V)
        : hpxBase(nside_), sI(I), sQ(Q), sU(U), sV(V), nside(nside_), nPixels(12 * nside_ * nside_)
    {
    }
    ~Sky() {}
    int get_nside(void) const { return nside; }
    int size(void) const { return nPixels; }

    PiscoHealpixBase hpxBase;
    const float* sI;
    const float* sQ;
    const float* sU;
    const float* sV;

  private:
    int nside;
    int nPixels;
};

#endif
