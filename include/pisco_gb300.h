/*
 * pisco_gb300.h -- C ABI of libpisco_gb300.so, the GB300 (sm_103a)
 * pixel-space polarized-beam convolver.
 *
 * Plain pointers and sizes only.  Every entry point returns a status code;
 * nothing exits, throws or waits for a key press across this boundary
 * (the reference's gpuAssert exits or blocks on getchar,
 * src/GpuConvolver/gpuconvolver.cu:8-32).  Host pointers are borrowed for the
 * duration of the call.  Device buffers are owned by the context.  A context
 * is used by one host thread at a time; separate contexts may run
 * concurrently.
 *
 * Angles are radians.  Maps are HEALPix RING-ordered.  The position angle
 * `pa` is counter-clockwise on the sky and is negated internally, as the
 * reference does (convolver.cpp:87-89, gpuconvolver.cu:459-461).
 */
#ifndef PISCO_GB300_H
#define PISCO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PISCO_ABI_VERSION 1

typedef enum pisco_status {
    PISCO_OK = 0,
    PISCO_ERR_INVALID_ARGUMENT = 1, /* bad polFlag, NULL pointer, bad size */
    PISCO_ERR_INVALID_CONFIG = 2,   /* RunConfig rejected (memory limit ...) */
    PISCO_ERR_NOT_READY = 3,        /* sky, beam or scan not set yet */
    PISCO_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    PISCO_ERR_OUT_OF_MEMORY = 5,    /* device or pinned allocation failed */
    PISCO_ERR_UNSUPPORTED = 6,      /* e.g. tuned form with a beam too wide */
    PISCO_ERR_DEVICE_CHECK = 7      /* a kernel's own bounds/wait check fired */
} pisco_status;

typedef enum pisco_dtype { PISCO_FLOAT32 = 0, PISCO_FLOAT64 = 1 } pisco_dtype;

/* PLAIN: the reference's per-pair chain on the GPU (FP64 geometry, FP32
 *        sky x beam products, FP64 accumulation).
 * TUNED: FP64 per-sample frame, FP32 per-pair geometry with an FP64
 *        re-evaluation of every decision that lies near a pixel edge, FP32
 *        products with compensated (two-sum) accumulation.
 * FP64:  every input, product and sum in FP64. */
typedef enum pisco_form {
    PISCO_FORM_PLAIN = 0,
    PISCO_FORM_TUNED = 1,
    PISCO_FORM_FP64 = 2
} pisco_form;

/* Beam lookup: nearest beam pixel (the reference's live path,
 * convolver.cpp:186-203) or 4-pixel bilinear (the commented-out
 * get_interpol block, convolver.cpp:162-185). */
typedef enum pisco_interp { PISCO_BEAM_NEAREST = 0, PISCO_BEAM_BILINEAR = 1 } pisco_interp;

/* Mirrors CUDACONV::RunConfig (src/GpuConvolver/cuda/cudaConv2.h:13-26).
 * ptgPerConv is the host<->device pipelining chunk (samples); pixelsPerDisc
 * is accepted for compatibility (no disc lists are materialised);
 * maxMemUsage bounds the context's device memory; nStreams >= 1 copy/compute
 * streams (the reference forces 1, gpuconvolver.cu:39).  grid/block sizes are
 * accepted and ignored (the reference ignores them too). */
typedef struct pisco_run_config {
    int nStreams;
    size_t maxMemUsage;
    int deviceId;
    int gridSizeX;
    int gridSizeY;
    int blockSizeX;
    int blockSizeY;
    int ptgPerConv;
    int pixelsPerDisc;
} pisco_run_config;

typedef struct pisco_ctx pisco_ctx;

/* ---- context (replaces GPUConvolver::GPUConvolver / configure_execution /
 *      ~GPUConvolver, gpuconvolver.hpp:21-34, gpuconvolver.cu:34-87,172-221) */
pisco_status pisco_create(const pisco_run_config* cfg, pisco_ctx** out);
pisco_status pisco_destroy(pisco_ctx* ctx);
const char* pisco_last_error(const pisco_ctx* ctx);
const char* pisco_status_string(pisco_status s);
int pisco_abi_version(void);

/* ---- inputs ---------------------------------------------------------- */
/* GPUConvolver::update_sky (gpuconvolver.cu:223-269): four host RING maps,
 * V may be NULL (zeros).  dtype FLOAT64 keeps an FP64 copy for the FP64
 * form; FLOAT32 maps are widened on the device when the FP64 form runs. */
pisco_status pisco_set_sky(pisco_ctx* ctx, int nside, const void* I, const void* Q,
                           const void* U, const void* V, pisco_dtype dtype);
/* Same, from a device buffer of npix x 4 interleaved (I,Q,U,V) values. */
pisco_status pisco_set_sky_device(pisco_ctx* ctx, int nside, const void* d_iquv,
                                  pisco_dtype dtype, void* stream);
/* GPUConvolver::update_beam (gpuconvolver.cu:271-345): PolBeam::aBeams[4]
 * and bBeams[4] planes (polbeam.hpp:67-68), npix = PolBeam::nPixels; the
 * disc radius is rhoMax = pix2ang(nside, npix).theta (polbeam.cpp:35-36). */
pisco_status pisco_set_beam(pisco_ctx* ctx, int nside, long npix, const void* const a[4],
                            const void* const b[4], pisco_dtype dtype);
/* GPUConvolver::update_scan (gpuconvolver.cu:347-380): n samples of ra, dec,
 * pa (host arrays of dtype).  Stored on the device as FP64. */
pisco_status pisco_set_scan(pisco_ctx* ctx, long n, const void* ra, const void* dec,
                            const void* pa, pisco_dtype dtype);
/* Same, from device FP64 arrays (copied device to device). */
pisco_status pisco_set_scan_device(pisco_ctx* ctx, long n, const double* d_ra,
                                   const double* d_dec, const double* d_pa, void* stream);
pisco_status pisco_set_interp(pisco_ctx* ctx, pisco_interp interp);

/* ---- forward --------------------------------------------------------- */
/* GPUConvolver::exec_convolution (gpuconvolver.cu:382-505) and
 * Convolver::exec_convolution (convolver.cpp:22-72): polFlag 'a', 'b' or
 * 'p' selects which host outputs are written (a and/or b, each n samples of
 * out_dtype).  Every sample is computed, including the tail the reference
 * drops (gpuconvolver.cu:386).  The scan is streamed to the device in
 * ptgPerConv chunks overlapped with compute when it was set from the host. */
pisco_status pisco_forward(pisco_ctx* ctx, char polFlag, void* a, void* b,
                           pisco_dtype out_dtype, pisco_form form);
/* Inputs already resident: outputs to device arrays (either may be NULL),
 * samples [begin, begin+n) of the current scan, on `stream` (NULL = the
 * context's stream).  Asynchronous; check pisco_sync() for device errors. */
pisco_status pisco_forward_device(pisco_ctx* ctx, pisco_form form, long begin, long n,
                                  void* d_a, void* d_b, pisco_dtype out_dtype, void* stream);
/* Waits for the context's work and reports device-side check failures. */
pisco_status pisco_sync(pisco_ctx* ctx);

/* ---- statistics of the last forward (for the roofline) ---------------- */
/* Number of (sample, disc pixel) pairs of the current scan and the number of
 * pairs the TUNED form re-evaluated in FP64. */
pisco_status pisco_count_pairs(pisco_ctx* ctx, long long* pairs);
pisco_status pisco_last_fallbacks(pisco_ctx* ctx, long long* fallbacks);
/* Diagnostic (no reference counterpart): runs the TUNED form on samples
 * [begin, begin+n) with each FP32 pixel decision also evaluated in FP64 and
 * returns the worst FP32 error as a fraction of the FP64 re-evaluation
 * margin (must stay well below 1).  Outputs are discarded. */
pisco_status pisco_tuned_calibrate(pisco_ctx* ctx, long begin, long n, double* worst_fraction);

/* ---- host HEALPix / PolBeam helpers (for the C++ PolBeam wrapper) ------ */
/* Healpix_Base::pix2ang / ang2pix, RING (used by polbeam.cpp:130,441). */
pisco_status pisco_hpx_pix2ang(int nside, long n, const long* pix, double* theta, double* phi);
pisco_status pisco_hpx_ang2pix(int nside, long n, const double* theta, const double* phi,
                               long* pix);
/* Beam map size for a radius (ang2pix(nside, radius, 0), the convention of
 * scripts/fields2beams.py:102) and its rhoMax (polbeam.cpp:35-36). */
long pisco_beam_npix_for_radius(int nside, double radius_rad);
double pisco_beam_rho_max(int nside, long npix);
/* PolBeam::make_unpol_gaussian_elliptical_beams field step
 * (polbeam.cpp:290-372): co-polar magnitude sqrt(gaussian), zero phases and
 * zero cross-polar field. */
pisco_status pisco_beam_gaussian_fields(int nside, long npix, double fwhmx_deg,
                                        double fwhmy_deg, double phi0_deg, double* magEco,
                                        double* phsEco, double* magEcx, double* phsEcx);
/* PolBeam::beam_from_fields (polbeam.cpp:117-184): tilde I,Q,U,V. */
pisco_status pisco_beam_from_fields(long npix, const double* magEco, const double* phsEco,
                                    const double* magEcx, const double* phsEcx, float* I,
                                    float* Q, float* U, float* V);
/* PolBeam::build (polbeam.cpp:186-288): a = (Ia+eps Ib, Qa-eps Qb, Ua-eps Ub,
 * Va+eps Vb)/Na and likewise b; Na = sum(Ia) (nsideSky/nsideBeam)^2. */
pisco_status pisco_beam_build(int nside_beam, long npix, double epsilon, char enabledDets,
                              int nside_sky, const float* const tilde_a[4],
                              const float* const tilde_b[4], float* const out_a[4],
                              float* const out_b[4]);

#ifdef __cplusplus
}
#endif
#endif /* PISCO_GB300_H */
