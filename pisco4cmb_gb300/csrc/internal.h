// internal.h -- device data layout and kernel launchers of libpisco_gb300.
//
// HBM layout (all RING-ordered, resident for the life of a context):
//   sky32  float4[npix]         I,Q,U,V interleaved, one 16-byte load per pixel
//   sky64  D4[npix]             FP64 copy for the FP64 form (32 bytes/pixel)
//   beam32 F8[npixB]            a.IQUV | b.IQUV: both detectors of one beam
//                               pixel in one 32-byte sector
//   beam64 D8[npixB]            FP64 copy (64 bytes/pixel)
//   ra/dec/pa double[n]         FP64 pointing (structure of arrays)
//   out    float|double[n]      TOD a and b
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pisco {

namespace tuned {
struct SamplePlan;  // tuned_core.cuh
}

struct alignas(32) D4 {
    double x, y, z, w;
};
struct alignas(32) F8 {
    float4 a, b;
};
struct alignas(64) D8 {
    D4 a, b;
};

// Per-ring geometry of the sky grid, built once per nside on the device
// (ring_table_kernel, fwd_tuned.cu) from hpx.cuh's ring_info and ring2z, so
// every value is the one the HEALPix formulas give: rings 1 .. 4 nside - 1
// at index ring - 1.  64 bytes, four 16-byte loads.  At most 32,767 rings
// (nside 8192): 2.1 MB.
struct alignas(16) RingT {
    double z;      // ring2z
    double omz2;   // 1 - z*z, rounded as the disc-edge formula rounds it
    double dec;    // latitude atan2(z, sqrt((1 - z)(1 + z)))
    double fr;     // npix / (2 pi), rounded as the disc-edge formula rounds it
    double dphi;   // 2 pi / npix
    float s;       // sqrt(1 - z^2)
    float dphif;   // 2 pi / npix
    float zf;      // z
    int start;     // first pixel
    int npix2;     // 2 npix + (1 if the ring is shifted by half a pixel)
};
constexpr int kMaxRings = 4 * 8192 - 1;

// Device-side check codes written to the context's error word (first one
// wins).  Kernels never trap: they record the code, skip the access and
// finish.
enum DevCheck : unsigned int {
    kCheckOk = 0,
    kCheckSkyIndex = 1,
    kCheckBeamIndex = 2,
    kCheckFallbackOverflow = 3,
    kCheckQueue = 4,
    kCheckAdjointIndex = 5,
    kCheckDump = 6,  // a pair record found its sample's entries full
};

struct FwdArgs {
    int nside_sky;
    const RingT* rings;  // sky ring table (TUNED form)
    const float4* sky32;
    const D4* sky64;
    int nside_beam;
    int npix_beam;
    const F8* beam32;
    const D8* beam64;
    double rho_max;
    long long begin, n;
    const double* ra;
    const double* dec;
    const double* pa;
    void* out_a;  // may be null
    void* out_b;  // may be null
    const int* order;  // position -> sample (sky order) or null (scan order)
    int out_f64;
    int interp;  // 0 nearest, 1 bilinear
    unsigned int* err;
    unsigned long long* fallbacks;  // tuned form: pairs re-evaluated in FP64
};

// One detector pair of a batched launch, as the device sees it.
struct BatchDet {
    const F8* beam;
    int nside_beam;
    int npix_beam;
    double rho_max;
    float rscale;  // sqrt(3) * nside_beam
    long long n;
    const double* ra;
    const double* dec;
    const double* pa;
    void* out_a;
    void* out_b;
    const int* order;  // position -> sample (sky order) or null
    long long plan_base;  // planned launch: its plans start at BatchArgs::plans[plan_base]
};

// One unit of the work queue: samples [begin, begin + count) of detector det.
struct BatchItem {
    int det;
    int count;
    long long begin;
};

struct BatchArgs {
    int nside_sky;
    const RingT* rings;  // sky ring table
    const float4* sky32;
    const BatchDet* dets;
    int ndet;
    const BatchItem* items;
    int nitems;
    unsigned int* queue;  // next item (reset to 0 before every launch)
    int out_f64;
    unsigned int* err;
    unsigned long long* fallbacks;
    int interp = 0;  // 0 nearest, 1 bilinear beam lookup
    // sample plans of every detector's positions (BatchDet::plan_base), built
    // by a plan kernel before the batched kernel; null: each warp plans its own
    tuned::SamplePlan* plans = nullptr;
    long long nplans = 0;  // sum of the detectors' samples
};

struct AdjArgs {
    int nside_sky;
    const RingT* rings;  // sky ring table
    const float4* sky32;  // needed for the beam gradient
    int nside_beam;
    int npix_beam;
    const F8* beam32;
    double rho_max;
    long long begin, n;
    const double* ra;
    const double* dec;
    const double* pa;
    const void* g_a;  // dL/dTOD a, b (n values each)
    const void* g_b;
    const int* order;  // position -> sample (sky order) or null
    int g_f64;
    int fixed;                     // 1: fixed-point int64 accumulation
    float* gsky32;                 // atomic: [npix][4] or null
    unsigned long long* gsky_fx;   // fixed: planes [4][npix] or null
    float* gbeam32;                // atomic: [npixB][8] or null
    unsigned long long* gbeam_fx;  // fixed: [npixB][8] or null
    double sky_scale, beam_scale;  // fixed-point scales 2^S
    int want_v;                    // accumulate the sky gradient's V column
    int interp;                    // 0 nearest, 1 bilinear beam lookup
    unsigned int* err;
    unsigned long long* fallbacks;
    // fused Gaussian beam-parameter gradient (no beam-map gradient): the
    // model table (npixB x 8 floats) or null, the per-warp partial sums
    // (6 doubles per warp of the grid) and the model's (1 + eps, 1 - eps)
    const float* ptab = nullptr;
    double* ppart = nullptr;
    float ceps_i = 1.0f, ceps_q = 1.0f;
    // the samples' plans (a.n of them, index: position), built by the planned
    // launch itself into this scratch; null: each warp plans its own samples
    tuned::SamplePlan* plans = nullptr;
};

// Per-pair record of a form's decisions (pisco_debug_pairs, debug.cu): the
// pairs of the sample at position j fill entries [offset[j], offset[j+1]),
// in no particular order (fill[j] counts the entries written so far).
struct PairDump {
    const long long* offset;  // n + 1 entries
    unsigned int* fill;       // n entries, zero before the launch
    int* sample;
    int* sky_pix;
    int* beam_pix;  // nearest lookup: the beam pixel; bilinear: -1
    float* c2;      // cos 2chi, sin 2chi as the form multiplies by them
    float* s2;
    double* chi;    // PLAIN / FP64 forms: the FP64 chi; TUNED: NaN
    int* flags;     // kPairRedone | kPairOutside
    int* st_pix;    // bilinear stencil: 4 per entry
    double* st_w;
};
constexpr int kPairRedone = 1;   // re-evaluated with the FP64 chain (TUNED)
constexpr int kPairOutside = 2;  // beam pixel (or every stencil pixel) beyond the stored map
// PLAIN-form record (fwd_plain.cu) and TUNED-form record (debug.cu) of
// samples [a.begin, a.begin + a.n); a.order must be null.
cudaError_t launch_dump_plain(const FwdArgs& a, const PairDump& d, int sm_count, cudaStream_t st);
cudaError_t launch_dump_tuned(const FwdArgs& a, const PairDump& d, int sm_count, cudaStream_t st);

// Fused beam-parameter gradient of the elliptical Gaussian pair model
// (beam_model.h): a table of the model's weight and its five derivatives at
// every beam pixel (npix x 8 floats) with the partial rows of its sums
// (kParamCols doubles each, gauss_table_rows(npix) rows, beam_dev.cu); the
// adjoint adds one row of beam-gradient-weighted sums (launch_fold_params);
// launch_gauss_param_finish turns nrows rows into dL/d(F, e, phi0, dx, dy).
constexpr int kParamCols = 12;
int gauss_table_rows(long npix);
cudaError_t launch_gauss_param_table(int nside_beam, long npix, double fwhm_deg, double e,
                                     double phi0_deg, double dx, double dy, float* tab,
                                     double* part, cudaStream_t st);
cudaError_t launch_gauss_param_finish(const double* part, int nrows, double oc, double* out,
                                      cudaStream_t st);
// Sums the adjoint's per-warp partials (nwarps x 6) in warp order into one
// partial row (columns 1 and 7..11; the rest zero).
cudaError_t launch_fold_params(const double* ppart, int nwarps, double* row, cudaStream_t st);

// Upper bound on the warps of an adjoint launch's grid.
int adjoint_max_warps(int sm_count);
// nwarps (optional): the warps of the launch's grid (the rows of ppart it writes).
cudaError_t launch_adjoint(const AdjArgs& a, int sm_count, cudaStream_t st, int* nwarps = nullptr);
// The same with a.plans: the plan kernel, then the planned kernels (adjoint_planned.cu).
cudaError_t launch_adjoint_planned(const AdjArgs& a, int sm_count, cudaStream_t st, int* nwarps);
cudaError_t launch_abs_sum(const void* ga, const void* gb, int f64, long long n, double* part,
                           cudaStream_t st);
cudaError_t launch_abs_max(const float* x, long long n, double* part, cudaStream_t st);
cudaError_t launch_fixed_to_float(const unsigned long long* in, void* out, int out_f64, long long n,
                                  double inv_scale, cudaStream_t st);
// The sky's fixed-point planes [4][npix] to the interleaved [npix][4] gradient.
cudaError_t launch_fixed_planes_to_float(const unsigned long long* in, void* out, int out_f64,
                                         long long npix, double inv_scale, cudaStream_t st);

// PLAIN (f64 = false) and FP64 (f64 = true) forms.
cudaError_t launch_forward_plain(const FwdArgs& a, bool f64, int sm_count, cudaStream_t st);
// Bytes of one sample's plan (tuned::SamplePlan, tuned_core.cuh).
constexpr size_t kSamplePlanBytes = 96;
// TUNED form.  plans: scratch for plan_cap sample plans (kSamplePlanBytes
// each), or null: with it the per-sample FP64 geometry is built beforehand
// by a kernel with one thread per sample, plan_cap samples at a time;
// without it each warp builds its own (the same values either way).
cudaError_t launch_forward_tuned(const FwdArgs& a, int sm_count, cudaStream_t st,
                                 void* plans = nullptr, long long plan_cap = 0);
bool tuned_supported(int nside_beam, int npix_beam, double rho_max);
// Same kernel with every FP32 decision also evaluated in FP64: writes the
// worst |FP32 - FP64| / margin seen over the non-fallback pairs to *calib.
cudaError_t launch_tuned_calibrate(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib);
// Sky order of n < 2^31 samples (order.cu).  With tmp == NULL stores the
// temporary bytes the sort needs in *tmp_bytes and does nothing else;
// otherwise writes order[0..n): the positions 0..n-1 sorted by the Z-order
// code of their pointing's sky cell (keys, keys_sorted, pos: n each).
cudaError_t sky_order(long long n, const double* ra, const double* dec, unsigned* keys,
                      unsigned* keys_sorted, int* pos, int* order, void* tmp, size_t* tmp_bytes,
                      cudaStream_t st);
// Fills the sky ring table (4 nside - 1 entries) for nside <= 8192.
cudaError_t launch_ring_table(int nside, RingT* rings, cudaStream_t st);
// Batched TUNED forward (fwd_batched.cu).
// warps: warps per block, 4, 8 or 16 (32 warps per SM for the planned nearest
// lookup, 16 otherwise, in every shape).
bool batched_warps_valid(int warps);
// The persistent grid is the instance's resident blocks on sm_count SMs.
cudaError_t launch_batched(const BatchArgs& a, int sm_count, cudaStream_t st, int warps = 8);
// Per-sample disc sizes (pairs) for the roofline byte model.
cudaError_t launch_count_pairs(int nside_sky, double rho_max, long long n, const double* ra,
                               const double* dec, unsigned long long* total, int sm_count,
                               cudaStream_t st);
// float -> double widening and scan conversion helpers.
cudaError_t launch_widen_sky(const float4* in, D4* out, long long npix, cudaStream_t st);
cudaError_t launch_widen_beam(const F8* in, D8* out, long long npix, cudaStream_t st);
cudaError_t launch_f32_to_f64(const float* in, double* out, long long n, cudaStream_t st);
cudaError_t launch_narrow_sky(const D4* in, float4* out, long long npix, cudaStream_t st);

}  // namespace pisco
