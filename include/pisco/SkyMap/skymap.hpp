// SkyMap -- the binned map-maker, same interface as the reference
// (src/SkyMap/skymap.hpp:13-56), running on the GPU through
// libpisco_gb300.so (pisco_map_*).  accumulate_data adds TOD into per-pixel
// normal equations kept on the device; solve_map solves them for I, Q, U.
// Differences from the reference: the accumulators start at zero (the
// reference leaves them uninitialised, skymap.cpp:25-36); no LAPACK is
// linked (its dgesv is restated on the device); pointings with |dec| > pi/2
// are skipped and reported (std::invalid_argument) instead of mapped.
#ifndef PISCO_SKYMAP_HPP
#define PISCO_SKYMAP_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "../pisco_detail.hpp"

class SkyMap {
    const int INSUFFCOV = 0;

  public:
    explicit SkyMap(int _nside, int device = 0) : nside(_nside), nPixels(12L * _nside * _nside)
    {
        const pisco_status s = pisco_map_create(_nside, device, &map);
        if (s != PISCO_OK)
            throw std::invalid_argument(std::string("SkyMap: ") + pisco_status_string(s));
    }
    ~SkyMap() { pisco_map_destroy(map); }
    SkyMap(const SkyMap&) = delete;
    SkyMap& operator=(const SkyMap&) = delete;

    // ra, dec, pa, data: ndetectors x nsamples floats, [det * nsamples + s]
    void accumulate_data(int nsamples, float ra[], float dec[], float pa[], int ndetectors,
                         float detPolAngles[], float data[])
    {
        check(pisco_map_accumulate(map, nsamples, ra, dec, pa, ndetectors, detPolAngles, data,
                                   PISCO_FLOAT32),
              "SkyMap::accumulate_data");
        fresh = false;
    }
    void solve_map(void)
    {
        check(pisco_map_solve(map), "SkyMap::solve_map");
        I.resize(nPixels);
        Q.resize(nPixels);
        U.resize(nPixels);
        hits.resize(nPixels);
        check(pisco_map_get(map, I.data(), Q.data(), U.data(), hits.data()), "SkyMap::solve_map");
        fresh = true;
    }

    int get_nside(void) const { return nside; }
    int size(void) const { return (int)nPixels; }
    // valid after solve_map (as in the reference, where they are filled there)
    const float* get_stokes_I(void) { return I.data(); }
    const float* get_stokes_Q(void) { return Q.data(); }
    const float* get_stokes_U(void) { return U.data(); }
    const int* get_hitmap(void) { return hits.data(); }
    pisco_map* handle() { return map; }

  private:
    void check(pisco_status s, const char* what)
    {
        if (s == PISCO_OK) return;
        const std::string msg =
            std::string(what) + ": " + pisco_map_last_error(map) + " (" + pisco_status_string(s) + ")";
        if (s == PISCO_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
        throw std::runtime_error(msg);
    }
    int nside;
    long nPixels;
    pisco_map* map = nullptr;
    bool fresh = false;
    std::vector<float> I, Q, U;
    std::vector<int> hits;
};

#endif
