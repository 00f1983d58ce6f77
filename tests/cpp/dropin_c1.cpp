// dropin_c1.cpp -- a caller written against the reference API, compiled
// unchanged against include/pisco (header-only wrappers over the C ABI of
// libpisco_gb300.so).  Builds the c1 PolBeam, reads the sky and scan from raw
// float32 files, runs GPUConvolver and Convolver and writes both TODs; with
// an eighth argument it also maps the GPU TOD of detectors a (0 deg) and b
// (90 deg) back with SkyMap and writes I, Q, U and the hits (float32 planes).
//
// usage: dropin_c1 <nside_sky> <nsamples> sky.f32 (3 planes) scan.f32
//        (ra, dec, pa planes) out_gpuconv.f32 out_conv.f32 [out_map.f32]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "Convolver/convolver.hpp"
#include "GpuConvolver/gpuconvolver.hpp"
#include "Polbeam/polbeam.hpp"
#include "Scan/scan.hpp"
#include "Sky/sky.hpp"
#include "SkyMap/skymap.hpp"

static std::vector<float> read_f32(const char* path, size_t n)
{
    std::vector<float> v(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(float), n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

static void write_f32(const char* path, const std::vector<float>& v)
{
    FILE* f = std::fopen(path, "wb");
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv)
{
    if (argc != 7 && argc != 8) return 2;
    const int nsideSky = std::atoi(argv[1]);
    const long ns = std::atol(argv[2]);
    const long npix = 12L * nsideSky * nsideSky;
    std::vector<float> sky = read_f32(argv[3], 3 * npix);
    std::vector<float> scan = read_f32(argv[4], 3 * ns);
    std::vector<float> V(npix, 0.0f);

    // beam: nside 256, radius 5 deg, circular FWHM 2 deg, epsilon 0.01
    const int nsideBeam = 256;
    const long nPixels = pisco_beam_npix_for_radius(nsideBeam, 5.0 * M_PI / 180.0);
    PolBeam beam(nsideBeam, nPixels, 0.01, 'p');
    beam.make_unpol_gaussian_elliptical_beams(2.0, 2.0, 0.0);
    beam.build(nsideSky);

    Sky skyv(nsideSky, sky.data(), sky.data() + npix, sky.data() + 2 * npix, V.data());
    Scan scanv(ns, scan.data(), scan.data() + ns, scan.data() + 2 * ns);

    CUDACONV::RunConfig cfg;
    cfg.nStreams = 1;
    cfg.maxMemUsage = size_t(1) << 30;
    cfg.deviceId = 0;
    cfg.gridSizeX = cfg.gridSizeY = cfg.blockSizeX = cfg.blockSizeY = 0;
    cfg.ptgPerConv = 6000;  // does not divide nsamples: every sample still computed
    cfg.pixelsPerDisc = 2000;
    GPUConvolver gconv(cfg);
    gconv.configure_execution();
    gconv.update_beam(&beam);
    gconv.update_sky(&skyv);
    gconv.update_scan(&scanv);
    std::vector<float> ga(ns), gb(ns);
    gconv.exec_convolution(ga.data(), gb.data());

    Convolver conv(&scanv, &skyv, &beam);
    std::vector<float> ca(ns), cb(ns);
    conv.exec_convolution('p', ca.data(), cb.data());
    bool threw = false;
    try {
        conv.exec_convolution('x', ca.data(), cb.data());
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    if (!threw) return 3;

    std::vector<float> out1(2 * ns), out2(2 * ns);
    for (long i = 0; i < ns; ++i) {
        out1[i] = ga[i];
        out1[ns + i] = gb[i];
        out2[i] = ca[i];
        out2[ns + i] = cb[i];
    }
    write_f32(argv[5], out1);
    write_f32(argv[6], out2);

    if (argc == 8) {
        // two detectors of one pair: same pointing, angles 0 and 90 deg
        std::vector<float> ra2(2 * ns), dec2(2 * ns), pa2(2 * ns), d2(2 * ns);
        for (long i = 0; i < ns; ++i)
            for (int det = 0; det < 2; ++det) {
                ra2[det * ns + i] = scan[i];
                dec2[det * ns + i] = scan[ns + i];
                pa2[det * ns + i] = scan[2 * ns + i];
                d2[det * ns + i] = det == 0 ? ga[i] : gb[i];
            }
        float pol[2] = {0.0f, (float)(M_PI / 2.0)};
        SkyMap smap(nsideSky);
        smap.accumulate_data((int)ns, ra2.data(), dec2.data(), pa2.data(), 2, pol, d2.data());
        smap.solve_map();
        std::vector<float> m(4 * npix);
        for (long p = 0; p < npix; ++p) {
            m[p] = smap.get_stokes_I()[p];
            m[npix + p] = smap.get_stokes_Q()[p];
            m[2 * npix + p] = smap.get_stokes_U()[p];
            m[3 * npix + p] = (float)smap.get_hitmap()[p];
        }
        write_f32(argv[7], m);
    }
    std::printf("dropin ok\n");
    return 0;
}
