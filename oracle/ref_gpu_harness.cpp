// ref_gpu_harness.cpp -- TEST INFRASTRUCTURE ONLY (a baseline, never the
// product).  Runs the reference's own GPU kernels -- K1
// fill_pixel_matching_matrix and K2 partial_polarized_convolution
// (src/GpuConvolver/cuda/cudaConv2.cu:59-240), compiled unmodified from the
// reference tree into oracle/_ref/refconv.cubin by build_ref.sh -- with the
// host orchestration of GPUConvolver (src/GpuConvolver/gpuconvolver.cu):
//   update_sky   (:225-270)  sky transposed to float4 IQUV;
//   update_beam  (:271-345)  beams transposed to float4 per detector;
//   update_scan  (:347-380)  pointing float4 (ra, dec, -pa, 0) in pinned memory;
//   exec_convolution (:382-505) per chunk of ptgPerConv samples: host
//     query_disc (OpenMP) into a ptgPerConv x pixPerDisc int buffer, three
//     host-to-device copies, K1, memset, K2, two device-to-host copies; the
//     nsamples % ptgPerConv tail is dropped as in the reference.
// Healpix C++'s query_disc is absent; the oracle's restatement stands in (it
// gives the same disc: pinned in tests/test_oracle_healpix.py).  Kernels are
// launched with the reference's geometry (16 x 128 blocks of 16 x 16,
// cudaConv2.h:6-9).  K2 calls __syncthreads inside its loop over pointings,
// which is uniform across a block only when ptgPerConv is a multiple of
// 16 x 128; the harness refuses other values instead of launching.  A disc
// larger than pixPerDisc is an error here (the reference writes past its
// buffer).  The driver API loads the cubin at run time (the reference's .cu
// sources are not needed where this runs).
#include <cuda.h>
#include <omp.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

extern "C" {
#include "oracle.h"
}

namespace {

// Itanium-mangled names of the two kernels (file-scope __global__ functions).
const char* kK1 = "_Z26fill_pixel_matching_matrixiPfiiiPiS0_S0_S_";
const char* kK2 = "_Z29partial_polarized_convolutioniiPfiiS_S_iiPiS0_S0_S_S_S_";
constexpr int kBX = 16, kBY = 16, kGX = 16, kGY = 128;  // cudaConv2.h:6-9

std::string g_err;

bool ck(CUresult r, const char* what)
{
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return false;
}

struct Dev {
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction k1 = nullptr, k2 = nullptr;
};

bool open_dev(const char* cubin, Dev* d)
{
    if (!ck(cuInit(0), "cuInit")) return false;
    if (!ck(cuDeviceGet(&d->dev, 0), "cuDeviceGet")) return false;
    if (!ck(cuDevicePrimaryCtxRetain(&d->ctx, d->dev), "primary context")) return false;
    if (!ck(cuCtxPushCurrent(d->ctx), "push context")) return false;
    if (!ck(cuModuleLoad(&d->mod, cubin), "cuModuleLoad")) return false;
    if (!ck(cuModuleGetFunction(&d->k1, d->mod, kK1), "K1 lookup")) return false;
    if (!ck(cuModuleGetFunction(&d->k2, d->mod, kK2), "K2 lookup")) return false;
    return true;
}

void close_dev(Dev* d)
{
    if (d->mod) cuModuleUnload(d->mod);
    if (d->ctx) {
        CUcontext c;
        cuCtxPopCurrent(&c);
        cuDevicePrimaryCtxRelease(d->dev);
    }
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err.c_str(); }

// 0 when the cubin loads and both kernels are found.
int refgpu_probe(const char* cubin)
{
    Dev d;
    const bool ok = open_dev(cubin, &d);
    close_dev(&d);
    return ok ? 0 : -1;
}

// The reference GPUConvolver pipeline over nsamples pointings (float, as the
// reference's Scan).  sky: npix x 4 float IQUV (already transposed); beam_a,
// beam_b: npix_beam x 4 float.  out_a/out_b receive the first
// nsamples - nsamples % ptg_per_conv samples.  Times (seconds): t[0] whole
// exec_convolution, t[1] K1 + K2 device time, t[2] host query_disc, t[3] copies.
// Returns the number of samples computed, or -1 (refgpu_last_error()).
long refgpu_convolve(const char* cubin, int nside_sky, const float* sky, int nside_beam,
                     long npix_beam, const float* beam_a, const float* beam_b, long nsamples,
                     const float* ra, const float* dec, const float* pa, int ptg_per_conv,
                     int pix_per_disc, int nthreads, float* out_a, float* out_b, double t[4])
{
    if (ptg_per_conv <= 0 || ptg_per_conv % (kGY * kBY) != 0) {
        g_err = "ptgPerConv must be a positive multiple of 2048 (uniform barriers in K2)";
        return -1;
    }
    if (pix_per_disc <= 0 || nside_sky < 1 || nside_beam < 1 || npix_beam < 1 || nsamples < 0) {
        g_err = "bad arguments";
        return -1;
    }
    Dev d;
    if (!open_dev(cubin, &d)) {
        close_dev(&d);
        return -1;
    }
    const long npix_sky = 12L * nside_sky * nside_sky;
    const size_t ptg_bytes = sizeof(float) * 4 * (size_t)ptg_per_conv;
    const size_t disc_bytes = sizeof(int) * (size_t)ptg_per_conv * pix_per_disc;
    const size_t cnt_bytes = sizeof(int) * (size_t)ptg_per_conv;
    const size_t res_bytes = sizeof(float) * (size_t)ptg_per_conv;
    CUdeviceptr d_sky = 0, d_ba = 0, d_bb = 0, d_ptg = 0, d_disc = 0, d_cnt = 0, d_mbp = 0,
                d_chi = 0, d_res = 0;
    float* h_ptg = nullptr;
    int* h_disc = nullptr;
    int* h_cnt = nullptr;
    CUevent e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
    long done = -1;
    double t_disc = 0, t_copy = 0, t_kern = 0;
    bool ok = ck(cuMemAlloc(&d_sky, sizeof(float) * 4 * npix_sky), "alloc sky") &&
              ck(cuMemAlloc(&d_ba, sizeof(float) * 4 * npix_beam), "alloc beam a") &&
              ck(cuMemAlloc(&d_bb, sizeof(float) * 4 * npix_beam), "alloc beam b") &&
              ck(cuMemAlloc(&d_ptg, ptg_bytes), "alloc ptg") &&
              ck(cuMemAlloc(&d_disc, disc_bytes), "alloc disc") &&
              ck(cuMemAlloc(&d_cnt, cnt_bytes), "alloc counts") &&
              ck(cuMemAlloc(&d_mbp, disc_bytes), "alloc beam pixels") &&
              ck(cuMemAlloc(&d_chi, sizeof(float) * (size_t)ptg_per_conv * pix_per_disc), "alloc chi") &&
              ck(cuMemAlloc(&d_res, 2 * res_bytes), "alloc result") &&
              ck(cuMemAllocHost((void**)&h_ptg, sizeof(float) * 4 * (size_t)(nsamples > 0 ? nsamples : 1)), "pinned ptg") &&
              ck(cuMemAllocHost((void**)&h_disc, disc_bytes), "pinned disc") &&
              ck(cuMemAllocHost((void**)&h_cnt, cnt_bytes), "pinned counts") &&
              ck(cuMemsetD8(d_disc, 0, disc_bytes), "memset disc") &&
              ck(cuMemsetD8(d_mbp, 0, disc_bytes), "memset beam pixels") &&
              ck(cuMemcpyHtoD(d_sky, sky, sizeof(float) * 4 * npix_sky), "copy sky") &&
              ck(cuMemcpyHtoD(d_ba, beam_a, sizeof(float) * 4 * npix_beam), "copy beam a") &&
              ck(cuMemcpyHtoD(d_bb, beam_b, sizeof(float) * 4 * npix_beam), "copy beam b") &&
              ck(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event") &&
              ck(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event") &&
              ck(cuEventCreate(&e2, CU_EVENT_DEFAULT), "event") &&
              ck(cuEventCreate(&e3, CU_EVENT_DEFAULT), "event");
    if (ok) {
        // update_scan: (ra, dec, -pa, 0) per sample
        for (long i = 0; i < nsamples; ++i) {
            h_ptg[4 * i + 0] = ra[i];
            h_ptg[4 * i + 1] = dec[i];
            h_ptg[4 * i + 2] = -pa[i];
            h_ptg[4 * i + 3] = 0.0f;
        }
        // rhoMax of the beam grid (polbeam.cpp:35-36)
        const double rho_max = orc_beam_rho_max(nside_beam, npix_beam);
        const long nsamples2 = nsamples - (nsamples % ptg_per_conv);
        const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
        const double t0 = now_s();
        int overflow = 0;
        for (long samp = 0; ok && samp < nsamples2; samp += ptg_per_conv) {
            double ta = now_s();
#pragma omp parallel num_threads(nt)
            {
                std::vector<int64_t> pix(pix_per_disc);
#pragma omp for schedule(static)
                for (int k = 0; k < ptg_per_conv; ++k) {
                    const float r = h_ptg[4 * (samp + k) + 0];
                    const float de = h_ptg[4 * (samp + k) + 1];
                    const int64_t n = orc_query_disc_pixels(nside_sky, M_PI_2 - de, r, rho_max,
                                                            pix.data(), pix_per_disc);
                    if (n < 0) {
#pragma omp atomic write
                        overflow = 1;
                        h_cnt[k] = 0;
                        continue;
                    }
                    for (int64_t q = 0; q < n; ++q)
                        h_disc[(size_t)k * pix_per_disc + q] = (int)pix[q];
                    h_cnt[k] = (int)n;
                }
            }
            double tb = now_s();
            t_disc += tb - ta;
            if (overflow) {
                g_err = "a disc holds more than pixPerDisc pixels";
                ok = false;
                break;
            }
            ok = ck(cuMemcpyHtoD(d_ptg, h_ptg + 4 * samp, ptg_bytes), "copy ptg") &&
                 ck(cuMemcpyHtoD(d_cnt, h_cnt, cnt_bytes), "copy counts") &&
                 ck(cuMemcpyHtoD(d_disc, h_disc, disc_bytes), "copy disc");
            if (!ok) break;
            double tc = now_s();
            t_copy += tc - tb;
            int nptgs = ptg_per_conv, ns = nside_sky, nb = nside_beam, ppd = pix_per_disc;
            int nsp = (int)npix_sky, nbp = (int)npix_beam;
            void* a1[] = {&nptgs, &d_ptg, &ns, &nb, &ppd, &d_cnt, &d_disc, &d_mbp, &d_chi};
            ok = ck(cuEventRecord(e0, 0), "record") &&
                 ck(cuLaunchKernel(d.k1, kGX, kGY, 1, kBX, kBY, 1, 0, 0, a1, nullptr), "K1 launch") &&
                 ck(cuEventRecord(e1, 0), "record") && ck(cuCtxSynchronize(), "K1");
            if (!ok) break;
            CUdeviceptr d_res_b = d_res + res_bytes;
            void* a2[] = {&ns,    &nsp,   &d_sky,  &nb,    &nbp,   &d_ba,  &d_bb,   &nptgs,
                          &ppd,   &d_cnt, &d_disc, &d_mbp, &d_chi, &d_res, &d_res_b};
            ok = ck(cuMemsetD8(d_res, 0, 2 * res_bytes), "memset result") &&
                 ck(cuEventRecord(e2, 0), "record") &&
                 ck(cuLaunchKernel(d.k2, kGX, kGY, 1, kBX, kBY, 1, 0, 0, a2, nullptr), "K2 launch") &&
                 ck(cuEventRecord(e3, 0), "record") && ck(cuCtxSynchronize(), "K2");
            if (!ok) break;
            float ms1 = 0, ms2 = 0;
            cuEventElapsedTime(&ms1, e0, e1);
            cuEventElapsedTime(&ms2, e2, e3);
            t_kern += 1e-3 * (ms1 + ms2);
            double td = now_s();
            ok = ck(cuMemcpyDtoH(out_a + samp, d_res, res_bytes), "copy a") &&
                 ck(cuMemcpyDtoH(out_b + samp, d_res + res_bytes, res_bytes), "copy b");
            t_copy += now_s() - td;
        }
        if (ok) {
            t[0] = now_s() - t0;
            t[1] = t_kern;
            t[2] = t_disc;
            t[3] = t_copy;
            done = nsamples2;
        }
    }
    for (CUevent e : {e0, e1, e2, e3})
        if (e) cuEventDestroy(e);
    for (CUdeviceptr p : {d_sky, d_ba, d_bb, d_ptg, d_disc, d_cnt, d_mbp, d_chi, d_res})
        if (p) cuMemFree(p);
    for (void* p : {(void*)h_ptg, (void*)h_disc, (void*)h_cnt})
        if (p) cuMemFreeHost(p);
    close_dev(&d);
    return done;
}

}  // extern "C"
