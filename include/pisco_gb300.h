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
 *        products with compensated (two-sum) accumulation.  With the
 *        bilinear lookup the stencil is formed in FP32 and only pairs at the
 *        boresight are re-evaluated (its weights are continuous).  A beam
 *        whose disc reaches beyond the polar cap of its grid (rhoMax > 0.5
 *        rad or within two rings of the cap's edge) is convolved by the
 *        PLAIN chain instead.
 * FP64:  every input, product and sum in FP64. */
typedef enum pisco_form {
    PISCO_FORM_PLAIN = 0,
    PISCO_FORM_TUNED = 1,
    PISCO_FORM_FP64 = 2
} pisco_form;

/* Beam lookup: nearest beam pixel (the reference's live path,
 * convolver.cpp:186-203) or 4-pixel bilinear (the commented-out
 * get_interpol block, convolver.cpp:162-185).  The forward forms, the
 * batched launch and the adjoint all take both. */
typedef enum pisco_interp { PISCO_BEAM_NEAREST = 0, PISCO_BEAM_BILINEAR = 1 } pisco_interp;

/* Order in which a launch processes the samples of its range (no reference
 * counterpart; the reference walks the scan in time order).  SKY sorts the
 * range by a Z-order code of the pointing's sky cell so that concurrently
 * running warps gather from overlapping disc footprints; TOD is written in
 * scan order and is bit-identical in both orders. */
typedef enum pisco_order { PISCO_ORDER_SCAN = 0, PISCO_ORDER_SKY = 1 } pisco_order;

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
/* Sample order of the context's forward and adjoint launches (default
 * PISCO_ORDER_SCAN).  In SKY order the sort of a sample range runs on the
 * launch's stream the first time the range is used after pisco_set_scan*,
 * and is reused after that. */
pisco_status pisco_set_sample_order(pisco_ctx* ctx, pisco_order order);

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
/* Device bytes the context holds, the figure RunConfig.maxMemUsage bounds
 * (the reference checks its fixed buffers against it once,
 * gpuconvolver.cu:58-70; here every buffer counts as it grows).  The TUNED
 * forward keeps up to 4M sample plans of 96 bytes as scratch: fewer (the
 * forward runs in chunks) when maxMemUsage leaves less room, none when it
 * leaves room for fewer than 1024 (each warp then plans its own samples);
 * the TOD is the same bit for bit in every case. */
pisco_status pisco_memory_used(const pisco_ctx* ctx, size_t* bytes);

/* ---- statistics of the last forward (for the roofline) ---------------- */
/* Number of (sample, disc pixel) pairs of the current scan and the number of
 * pairs the TUNED form re-evaluated in FP64. */
pisco_status pisco_count_pairs(pisco_ctx* ctx, long long* pairs);
pisco_status pisco_last_fallbacks(pisco_ctx* ctx, long long* fallbacks);
/* Diagnostic (no reference counterpart): runs the TUNED form on samples
 * [begin, begin+n) with each FP32 pixel decision also evaluated in FP64 and
 * returns the worst FP32 error as a fraction of the FP64 re-evaluation
 * margin (must stay well below 1), and (if tuned_pairs is not NULL) the
 * number of disc pairs the TUNED disc evaluation produced (must equal
 * pisco_count_pairs over the same samples).  Outputs are discarded. */
pisco_status pisco_tuned_calibrate(pisco_ctx* ctx, long begin, long n, double* worst_fraction,
                                   long long* tuned_pairs);

/* ---- per-pair record of a form's decisions (diagnostic; no reference
 *      counterpart as an entry point -- the reference checks the same
 *      decisions in its device tests, tests/cudaConvolution/
 *      test_sky_to_beam_matching_kernel.cu:188-216) ---------------------- */
/* Host arrays of `capacity` entries each (4 per entry for the stencil);
 * any pointer may be NULL (that field is not returned). */
typedef struct pisco_pair_dump {
    long long capacity;
    int* sample;       /* position of the pair's sample in [0, n) */
    int* sky_pix;      /* the disc pixel (RING) */
    int* beam_pix;     /* nearest lookup: the beam pixel chosen, also when it
                          lies beyond the stored map; bilinear lookup: -1 */
    float* c2chi;      /* cos 2chi and sin 2chi as the form multiplies by them */
    float* s2chi;
    double* chi;       /* PLAIN / FP64: the FP64 chi; TUNED: NaN */
    int* flags;        /* PISCO_PAIR_REDONE | PISCO_PAIR_OUTSIDE_BEAM */
    int* stencil_pix;  /* bilinear lookup: 4 stencil pixels per pair, in
                          get_interpol's order; nearest: -1 */
    double* stencil_w; /* TUNED: the FP32 weights the kernel multiplies by
                          (renormalised over the stored map, 0 beyond it);
                          PLAIN / FP64: get_interpol's FP64 weights */
} pisco_pair_dump;
#define PISCO_PAIR_REDONE 1       /* TUNED: re-evaluated with the FP64 chain */
#define PISCO_PAIR_OUTSIDE_BEAM 2 /* beam pixel (every stencil pixel) beyond the
                                     stored map: the pair adds nothing */
/* Runs the per-sample body of `form` (with the context's beam lookup) over
 * samples [begin, begin+n) of the current scan and records every (sample,
 * disc pixel) pair it visits: each sample's pairs appear together, in no
 * particular order within the sample.  *npairs = the number of disc pairs of
 * the range (HEALPix query_disc).  out == NULL only sizes the record;
 * out->capacity below *npairs is PISCO_ERR_INVALID_ARGUMENT.  Synchronous;
 * allocates its device buffers for the call. */
pisco_status pisco_debug_pairs(pisco_ctx* ctx, pisco_form form, long begin, long n,
                               const pisco_pair_dump* out, long long* npairs);

/* ---- HEALPix RING on the device, whole arrays (the device routines every
 *      kernel uses; the reference's device port is
 *      src/GpuConvolver/cuda/cudaHealpix.cu:56-259) ---------------------
 * Device arrays of n values on `stream` (NULL: the legacy default stream)
 * of the current device; synchronous.  An out-of-range input is
 * PISCO_ERR_INVALID_ARGUMENT (its outputs are NaN / -1). */
pisco_status pisco_hpx_pix2ang_device(int nside, long long n, const long long* d_pix,
                                      double* d_theta, double* d_phi, void* stream);
pisco_status pisco_hpx_ang2pix_device(int nside, long long n, const double* d_theta,
                                      const double* d_phi, long long* d_pix, void* stream);
/* Four pixels and weights per point (n x 4 each), get_interpol's order. */
pisco_status pisco_hpx_get_interpol_device(int nside, long long n, const double* d_theta,
                                           const double* d_phi, long long* d_pix4, double* d_w4,
                                           void* stream);

/* ---- batched multi-detector forward ------------------------------------ */
/* One detector pair of a batched forward.  Device pointers: FP64 pointing
 * of nsamples samples and the two TOD outputs (out_dtype; either may be
 * NULL).  The reference handles one pair per GPUConvolver
 * (gpuconvolver.hpp:17-82); a focal plane is a loop over such objects. */
typedef struct pisco_det_desc {
    int beam_slot; /* beam set with pisco_set_beam_slot */
    int flags;     /* PISCO_DET_SKY_ORDER: process this pair's samples in sky
                      order (sorted when the launch is captured) */
    long long nsamples;
    const double* ra;
    const double* dec;
    const double* pa;
    void* tod_a;
    void* tod_b;
} pisco_det_desc;
#define PISCO_DET_SKY_ORDER 1

/* Beam of one detector pair (PolBeam::aBeams / bBeams planes), kept in slot
 * `slot` (0 <= slot < 1024) for batched launches; same arguments as
 * pisco_set_beam. */
pisco_status pisco_set_beam_slot(pisco_ctx* ctx, int slot, int nside, long npix,
                                 const void* const a[4], const void* const b[4],
                                 pisco_dtype dtype);
/* All pairs in one persistent TUNED launch over a (detector, sample-chunk)
 * work queue, longest chunks first.  chunk = samples per queue item (0 =
 * the last autotuned value, else 256).  The launch is captured in a CUDA
 * graph and replayed while the same descriptors and chunk are resubmitted.
 * Asynchronous on `stream` (NULL = context stream); pisco_sync() reports
 * device-side check failures.  Every beam must fit the TUNED form's domain
 * (PISCO_ERR_UNSUPPORTED otherwise). */
pisco_status pisco_forward_batched(pisco_ctx* ctx, const pisco_det_desc* dets, int ndet,
                                   pisco_dtype out_dtype, int chunk, void* stream);
/* Autotuner (no reference counterpart): times the batched launch on these
 * descriptors for each tile -- 4, 8 or 16 warps per block, every shape at 16
 * warps per SM -- and chunk sizes 32..8192, keeps the fastest pair in the
 * context and, if cache_path is not NULL, in a JSON object keyed by device,
 * sky nside, beam set, output type and beam lookup (read first: a cached key
 * is reused without timing).  Returns the chosen chunk and its time in ms;
 * pisco_batched_config reports the chosen tile. */
pisco_status pisco_autotune_batched(pisco_ctx* ctx, const pisco_det_desc* dets, int ndet,
                                    pisco_dtype out_dtype, const char* cache_path,
                                    int* chunk_out, double* ms_out);
/* The chunk (0 passed to pisco_forward_batched means this one) and warps per
 * block the batched launch uses now (either pointer may be NULL). */
pisco_status pisco_batched_config(pisco_ctx* ctx, int* chunk, int* warps_per_block);
/* Sets them without timing (chunk 0 keeps the current chunk; warps per block
 * 4, 8 or 16). */
pisco_status pisco_set_batched_config(pisco_ctx* ctx, int chunk, int warps_per_block);

/* ---- allocation-free batched forward (no counterpart in the reference) --
 * For callers that may not allocate device memory (real-time loops, host
 * callbacks, services whose memory pool owns the whole GPU): the batched
 * TUNED forward with every buffer supplied by the caller and its own
 * working memory (sky ring table, work queue, descriptors, counters) in a
 * fixed array of about 2.6 MB compiled into the library, shared by all calls.  No context;
 * calls no allocator.  Synchronous (returns when the TOD is written).
 * Limits: at most PISCO_NOALLOC_MAX_DETS detector pairs and at most
 * PISCO_NOALLOC_MAX_ITEMS work items, sum over pairs of
 * ceil(nsamples / chunk) -- raise chunk for long scans; beyond either limit
 * the call returns PISCO_ERR_INVALID_ARGUMENT with the reason in
 * pisco_last_error(NULL); so does a pair of more than 2^40 samples.  The
 * first call on a device looks up the array's device address and should
 * come before any stream capture on that device; the address is kept for
 * the life of the process, so do not call this entry point on a device
 * after a cudaDeviceReset of it.
 * Calls whose GPU work overlaps race on the shared array: serialise them. */
#define PISCO_NOALLOC_MAX_DETS 128
#define PISCO_NOALLOC_MAX_ITEMS 32768

typedef struct pisco_noalloc_det {
    int nside_beam;
    long npix_beam;
    const float* beam_ab; /* device, npix_beam x 8: a.I,Q,U,V, b.I,Q,U,V; 32-B aligned */
    long long nsamples;
    const double* ra; /* device FP64 pointing */
    const double* dec;
    const double* pa;
    float* tod_a; /* device outputs (either may be NULL) */
    float* tod_b;
} pisco_noalloc_det;

/* d_sky_iquv: device, 12 nside_sky^2 x 4 floats (I,Q,U,V), 16-B aligned.
 * chunk: samples per work item (0 = 256). */
pisco_status pisco_forward_batched_noalloc(int device, int nside_sky, const float* d_sky_iquv,
                                           const pisco_noalloc_det* dets, int ndet, int chunk,
                                           void* stream);

/* ---- adjoint (no reference counterpart: PISCO has no gradient) --------- */
/* ATOMIC: float atomics, fast, last bits vary run to run.
 * DETERMINISTIC: 64-bit fixed-point atomics with a scale from a rigorous
 * bound on every total; bit-identical results whatever the order. */
typedef enum pisco_adjoint_mode {
    PISCO_ADJ_ATOMIC = 0,
    PISCO_ADJ_DETERMINISTIC = 1,
    /* OR-ed with either mode: the sky gradient holds I, Q, U only (its V
     * column is written as zero and not accumulated: a quarter fewer
     * accumulations in the DETERMINISTIC mode) */
    PISCO_ADJ_SKY_IQU = 2
} pisco_adjoint_mode;

/* Beam from a device buffer of npix x 8 interleaved values (a.I,Q,U,V,
 * b.I,Q,U,V), e.g. a beam built by differentiable code on the GPU. */
pisco_status pisco_set_beam_device(pisco_ctx* ctx, int nside, long npix, const void* d_ab,
                                   pisco_dtype dtype, void* stream);
/* Transpose of the TUNED forward over samples [begin, begin+n) of the
 * current scan: d_ga, d_gb = dL/dTOD a, b (n values of g_dtype, device).
 * Writes (overwrites) d_gsky = dL/dsky as npix x 4 (I,Q,U,V interleaved) and
 * d_gbeam = dL/dbeam as npixB x 8 (a.IQUV, b.IQUV), either may be NULL, in
 * out_dtype.  The pair set and beam pixels are exactly the forward's. */
pisco_status pisco_adjoint_device(pisco_ctx* ctx, long begin, long n, const void* d_ga,
                                  const void* d_gb, pisco_dtype g_dtype, void* d_gsky,
                                  void* d_gbeam, pisco_dtype out_dtype, pisco_adjoint_mode mode,
                                  void* stream);
/* The adjoint with the beam-parameter gradient formed directly (no
 * reference counterpart): for a context whose beam is the elliptical
 * Gaussian pair model of pisco_beam_gaussian_device with these parameters,
 * d_grad (5 device doubles) = dL/d(fwhm_deg, ellipticity, phi0_deg, dx, dy),
 * the value pisco_beam_gaussian_param_grad_device gives from
 * pisco_adjoint_device's beam-map gradient, without forming that map: each
 * pair's share is weighted by the model's weight and derivatives, recomputed
 * from the parameters for every call at the beam pixel centres, and reduced
 * per warp and then in warp order (the same result on every run, in either
 * mode).  d_gsky as pisco_adjoint_device (may be NULL); the mode selects the
 * sky gradient's accumulation. */
pisco_status pisco_adjoint_gaussian_device(pisco_ctx* ctx, long begin, long n, const void* d_ga,
                                           const void* d_gb, pisco_dtype g_dtype, void* d_gsky,
                                           pisco_dtype out_dtype, pisco_adjoint_mode mode,
                                           double epsilon, int nside_sky, double fwhm_deg,
                                           double ellipticity, double phi0_deg, double dx,
                                           double dy, double* d_grad, void* stream);
/* Host arrays: g_a, g_b (nsamples each) in; sky gradient planes out (any of
 * gI, gQ, gU, gV may be NULL). */
pisco_status pisco_adjoint(pisco_ctx* ctx, const void* g_a, const void* g_b, pisco_dtype g_dtype,
                           void* gI, void* gQ, void* gU, void* gV, pisco_dtype out_dtype,
                           pisco_adjoint_mode mode);

/* Beam-parameter gradient (the dbeam_params of the adjoint; no reference
 * counterpart): dL/d(fwhm_deg, ellipticity, phi0_deg, dx, dy) of an
 * elliptical Gaussian detector-pair beam (PolBeam's
 * make_unpol_gaussian_elliptical_beams + build, polbeam.cpp:204-268, 290-372,
 * with fwhm_x,y = F sqrt((1 +- e) / (1 -+ e)) and the centre offset by
 * (dx, dy) radians in the beam plane), from gbeam = dL/dbeam (npix x 8 host
 * doubles, a.IQUV b.IQUV, e.g. pisco_adjoint_device's d_gbeam).  The beam
 * weights are recomputed and differentiated analytically, normalisation
 * included. */
pisco_status pisco_beam_gaussian_param_grad(int nside_beam, long npix, double epsilon,
                                            int nside_sky, double fwhm_deg, double ellipticity,
                                            double phi0_deg, double dx, double dy,
                                            const double* gbeam, double grad[5]);

/* ---- beams built on the device (PolBeam construction, polbeam.cpp:117-372) --
 * Outputs are d_ab = npix x 8 floats (a.I,Q,U,V, b.I,Q,U,V; device, 16-B
 * aligned), the layout pisco_set_beam_device takes; set_beam != 0 also makes
 * the result the context's beam.  Run on `stream` (NULL: the context's) and
 * return without waiting.  Sums are deterministic (fixed order). */
/* PolBeam::beam_from_fields for each enabled detector + PolBeam::build
 * (polbeam.cpp:117-288): d_fields_a / d_fields_b = 4 x npix doubles (planes
 * magEco, phsEco, magEcx, phsEcx; device); a detector's fields may be NULL when
 * enabledDets leaves it out (its tilde beams are then zero).  Per pixel the
 * host step's rounded operations; the normalisation is summed as a fixed tree
 * and cos/sin are the device's, so results match pisco_beam_from_fields +
 * pisco_beam_build to about one float ulp. */
pisco_status pisco_beam_build_device(pisco_ctx* ctx, int nside_beam, long npix, double epsilon,
                                     char enabledDets, int nside_sky, const double* d_fields_a,
                                     const double* d_fields_b, float* d_ab, int set_beam,
                                     void* stream);
/* The beam of pisco_beam_gaussian_param_grad's model (elliptical Gaussian
 * pair, fwhm_x,y = F sqrt((1 +- e) / (1 -+ e)), rotated by phi0, centre at
 * (dx, dy) radians): a = b = ((1 + eps) g, (1 - eps) g, 0, 0) / N with
 * N = (nside_sky / nside_beam)^2 sum g. */
pisco_status pisco_beam_gaussian_device(pisco_ctx* ctx, int nside_beam, long npix, double epsilon,
                                        int nside_sky, double fwhm_deg, double ellipticity,
                                        double phi0_deg, double dx, double dy, float* d_ab,
                                        int set_beam, void* stream);
/* pisco_beam_gaussian_param_grad on the device: d_gbeam = dL/dbeam (npix x 8
 * of g_dtype, device), d_grad = 5 device doubles dL/d(fwhm_deg, ellipticity,
 * phi0_deg, dx, dy) (NaN when the model's weights sum to zero). */
pisco_status pisco_beam_gaussian_param_grad_device(pisco_ctx* ctx, int nside_beam, long npix,
                                                   double epsilon, int nside_sky, double fwhm_deg,
                                                   double ellipticity, double phi0_deg, double dx,
                                                   double dy, const void* d_gbeam,
                                                   pisco_dtype g_dtype, double* d_grad,
                                                   void* stream);

/* ---- binned map-maker (replaces SkyMap, src/SkyMap/skymap.hpp:13-56) ---
 * Accumulates TOD into per-pixel normal equations (3 x 3 AtA and AtD, FP64,
 * device-resident) and solves them for I, Q, U.  Each pixel's totals
 * receive the reference's additions in the reference's order
 * (skymap.cpp:68-132), deterministically. */
typedef struct pisco_map pisco_map;
/* SkyMap::SkyMap(int nside) (skymap.cpp:21-37): RING map of 12 nside^2
 * pixels on `device`, accumulators zero (the reference leaves them
 * uninitialised). */
pisco_status pisco_map_create(int nside, int device, pisco_map** out);
void pisco_map_destroy(pisco_map* map);
const char* pisco_map_last_error(const pisco_map* map);
/* Zero the accumulators. */
pisco_status pisco_map_reset(pisco_map* map);
/* SkyMap::accumulate_data(nsamples, ra, dec, pa, ndetectors, detPolAngles,
 * data) (skymap.cpp:68-132): host arrays of ndet x nsamples values indexed
 * [det * nsamples + s], dtype FLOAT32 (the reference's type) or FLOAT64;
 * det_pol_angles: ndet host floats.  psi = -(pol + pa).  Pointings with
 * |dec| > pi/2 or non-finite values are skipped and reported
 * (PISCO_ERR_INVALID_ARGUMENT after the rest is accumulated).  Synchronous. */
pisco_status pisco_map_accumulate(pisco_map* map, long nsamples, const void* ra, const void* dec,
                                  const void* pa, int ndet, const float* det_pol_angles,
                                  const void* data, pisco_dtype dtype);
/* Same from device arrays; runs on `stream` (NULL: the map's own) and
 * returns when done.  At most 2^31 - 1 values per call. */
pisco_status pisco_map_accumulate_device(pisco_map* map, long nsamples, const void* d_ra,
                                         const void* d_dec, const void* d_pa, int ndet,
                                         const float* det_pol_angles, const void* d_data,
                                         pisco_dtype dtype, void* stream);
/* SkyMap::solve_map (skymap.cpp:134-231): per pixel, hits = (int)AtA[0][0];
 * with hits >= 3 AtA x = AtD is solved (LAPACK dgesv, restated) for
 * (I, Q, U); an exactly singular system keeps AtD as (I, Q, U) and sets
 * hits to 0; hits < 3 gives I = Q = U = 0 (INSUFFCOV). */
pisco_status pisco_map_solve(pisco_map* map);
/* get_stokes_I / _Q / _U, get_hitmap (skymap.hpp:32-35): host copies of
 * 12 nside^2 values each (any pointer may be NULL). */
pisco_status pisco_map_get(pisco_map* map, float* I, float* Q, float* U, int* hits);
/* The normal equations in the reference's layout: ata = 9 x npix doubles
 * (AtA row-major per pixel, skymap.cpp:114-122), atd = 3 x npix (either may
 * be NULL); host copies. */
pisco_status pisco_map_get_normal(pisco_map* map, double* ata, double* atd);
/* Device arrays: I, Q, U (3 x npix floats), hits (npix ints) and the normal
 * equations (9 x npix doubles: AtA[0][0], [0][1], [0][2], [1][1], [1][2],
 * [2][2], then AtD[0..2], each as one npix-long plane). */
pisco_status pisco_map_device_arrays(pisco_map* map, const float** d_iqu, const int** d_hits,
                                     const double** d_normal);

/* ---- detector pointing from the array centre (BPoint::focal_plane_to_sky,
 *      src/Bpoint/bpoint.cpp:553-674, src/Bpoint/BPoint.h:99-103) ----------
 * The geometry-only step of BPoint (its ephemeris part needs SOFA and JPL
 * tables, which the reference tree does not hold): per detector, receiver-
 * frame offsets det_dx (positive right) and det_dy (positive up) and the
 * polarization angle ccw from the receiver y axis; per sample, the array
 * centre (x_ac, y_ac) and rot_ac, the angle of the receiver's up axis from
 * the zenith (flag 0, Az/El), the celestial pole (flag 1, Ra/Dec) or the
 * source (flag 2, source-relative).  Outputs ndets x nsamples, indexed
 * [det * nsamples + s]: longitude (Ra/Az; flag 2: bearing), latitude and the
 * detector's polarization direction (position angle + polarization angle).
 * Radians; FP64 on the GPU.  Host arrays, synchronous, current device.
 * A beam model's centre offset (dx, dy) (pisco_beam_gaussian_device) is, to
 * first order, the focal-plane offset (det_dx, det_dy) = (-dy, -dx) of a
 * detector whose scan position angle is rot_ac. */
pisco_status pisco_focal_plane_to_sky(int ndets, const double* det_dx, const double* det_dy,
                                      const double* det_pol_angle, long nsamples,
                                      const double* x_ac, const double* y_ac,
                                      const double* rot_ac, int flag, double* x_det,
                                      double* y_det, double* rot_det);
/* Same with device arrays, on `stream` (NULL: the legacy default stream);
 * asynchronous. */
pisco_status pisco_focal_plane_to_sky_device(int ndets, const double* d_det_dx,
                                             const double* d_det_dy, const double* d_det_pol,
                                             long nsamples, const double* d_x_ac,
                                             const double* d_y_ac, const double* d_rot_ac, int flag,
                                             double* d_x_det, double* d_y_det, double* d_rot_det,
                                             void* stream);

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
