/*
 * ref_map_harness.cpp -- C entry point around the reference's binned
 * map-maker (TEST INFRASTRUCTURE ONLY; built by oracle/build_ref.sh into
 * oracle/_ref/).
 *
 * SkyMap (src/SkyMap/skymap.cpp) is compiled unmodified from the reference
 * tree against the HEALPix shim.  Two adaptations live here:
 *   - the reference links LAPACK's dgesv_ (skymap.cpp:13-19); LAPACK is not
 *     in the reference tree, so dgesv_ below is the oracle's restatement
 *     (orc_dgesv3), itself checked against LAPACK through scipy;
 *   - the constructor leaves the accumulators uninitialised (the zeroing
 *     loop at skymap.cpp:25-36 is commented out), so they are zeroed here
 *     before the first accumulate_data, and read back for comparison
 *     (private members opened by a define; the class layout is unchanged).
 */
#include <cstring>

#define private public
#include "SkyMap/skymap.hpp"
#undef private

#include "oracle.h"

extern "C" void dgesv_(int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b, int* ldb,
                       int* info)
{
    if (*n != 3 || *nrhs != 1 || *lda != 3 || *ldb != 3) {
        *info = -1;  // only the 3 x 3, one right-hand side case is called
        return;
    }
    *info = orc_dgesv3(a, ipiv, b);
}

/* SkyMap(nside); zeroed accumulators; ncalls x accumulate_data(...) on the
 * same arrays ([det * nsamples + s] layout, float as in the reference);
 * solve_map(); copies AtA (9 x npix), AtD (3 x npix), I, Q, U and hits. */
extern "C" int ref_skymap_run(int nside, int nsamples, const float* ra, const float* dec,
                              const float* pa, int ndet, const float* pol, const float* data,
                              int ncalls, double* ata, double* atd, float* I, float* Q, float* U,
                              int* hits)
{
    SkyMap m(nside);
    const long np = m.size();
    std::memset(m.AtA, 0, sizeof(double) * 9 * np);
    std::memset(m.AtD, 0, sizeof(double) * 3 * np);
    for (int c = 0; c < ncalls; ++c)
        m.accumulate_data(nsamples, const_cast<float*>(ra), const_cast<float*>(dec),
                          const_cast<float*>(pa), ndet, const_cast<float*>(pol),
                          const_cast<float*>(data));
    std::memcpy(ata, m.AtA, sizeof(double) * 9 * np);
    std::memcpy(atd, m.AtD, sizeof(double) * 3 * np);
    m.solve_map();
    std::memcpy(I, m.get_stokes_I(), sizeof(float) * np);
    std::memcpy(Q, m.get_stokes_Q(), sizeof(float) * np);
    std::memcpy(U, m.get_stokes_U(), sizeof(float) * np);
    std::memcpy(hits, m.get_hitmap(), sizeof(int) * np);
    return 0;
}
