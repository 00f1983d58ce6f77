// fwd_tuned.cu -- TUNED forward, one detector pair per launch.
//
// Same result as the reference chain (convolver.cpp:112-221) pair by pair,
// with FP32 per-pair geometry; see tuned_core.cuh for the geometry and the
// FP64 re-evaluation of near-edge decisions.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so the reference's per-pair FP64
// transcendentals (about ten per pair) cannot stay on the hot path.
//
// One warp per sample, grid sized to the resident warps of the GPU and
// strided over samples; per-lane compensated FP32 sums, fixed shuffle-tree
// reduction (bit-reproducible).
#include "tuned_core.cuh"

namespace pisco {
namespace {

// Launch shape: the nearest lookup runs one block of 32 warps per SM
// (register cap 64).  The kernel is latency-bound, and with each sample's
// plan (WarpSmem::plan) and the grids' and beam's descriptors in shared
// memory, read where needed, its pair loop fits 64 registers with little
// spilling, so eight warps per scheduler hide what four could not (c2
// forward: 129.9 ms, against 169.7 ms for 16 warps at 128 registers; with
// the descriptors in registers 20 warps gave 162.1 ms and 24 warps, spilling
// inside the loop, 174.6 ms).  The 32 warps work on consecutive samples,
// whose discs overlap, so their sky reads share L1.  Its 169 KB of per-warp
// shared state is a static allocation, which sm_103a allows beyond 48 KB.
// The bilinear lookup, which needs more registers per pair, runs 8 x 2 with
// its descriptors in registers (296.3 ms; from shared memory 374.1 ms).  For
// the nearest lookup the beam's descriptor in registers (its pointer and size
// then come from the kernel parameters) is slower: 133.4 against 120.4 ms.
#ifndef PISCO_FWD_WARPS
#define PISCO_FWD_WARPS 32
#endif
#ifndef PISCO_BIL_WARPS
#define PISCO_BIL_WARPS 8
#endif

// kBil: bilinear beam lookup (the PLAIN form's get_interpol stencil in FP32).
// kTW: warps per block (fwd_warps_per_sm / kTW blocks per SM).
// Positions [pos0, pos1) of the launch.  kPlanned: plans holds their sample
// plans (index position - pos0); otherwise each warp builds its own.
// Warps per SM: 32 for the planned nearest lookup (register cap 64), 16 for
// the others (cap 128).
template <bool kCalib, bool kBil, bool kPlanned>
constexpr int fwd_warps_per_sm()
{
    return kPlanned && !kBil && !kCalib ? 32 : 16;
}

template <bool kCalib, bool kBil, int kTW, bool kPlanned>
__global__ void __launch_bounds__(kTW * 32, fwd_warps_per_sm<kCalib, kBil, kPlanned>() / kTW)
    tuned_kernel(FwdArgs a, float* calib, const tuned::SamplePlan* __restrict__ plans,
                 long long pos0, long long pos1)
{
    __shared__ tuned::WarpSmem sm[kTW];
    const int lane = threadIdx.x & 31;
    tuned::WarpSmem& S = sm[threadIdx.x >> 5];
    // The nearest lookup keeps the grids' and the beam's descriptors in
    // shared memory, read where needed rather than held in registers across
    // the pair loop: at its 64-register cap (32 warps per SM) that leaves the
    // registers to the pair geometry.  The bilinear lookup, which reads the
    // beam descriptor on every stencil pixel, keeps them in registers.
    constexpr bool kDescSmem = !kBil;
    __shared__ Hpx s_hs, s_hb;
    __shared__ tuned::Beam s_B;
    const Hpx rhs = hpx_make(a.nside_sky);
    const Hpx rhb = hpx_make(a.nside_beam);
    const tuned::Beam rB = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    if constexpr (kDescSmem) {
        if (threadIdx.x == 0) {
            s_hs = rhs;
            s_hb = rhb;
            s_B = rB;
        }
        __syncthreads();
    }
    const Hpx& hs = kDescSmem ? s_hs : rhs;
    const Hpx& hb = kDescSmem ? s_hb : rhb;
    const tuned::Beam& B = kDescSmem ? s_B : rB;
    const long long gw = (long long)blockIdx.x * kTW + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kTW;
    unsigned long long nfall = 0, npairs = 0;
    float cmax = 0.0f;
    tuned::Gather g;
    g.sky = a.sky32;
    tuned::Queue Q{0, 0};
    for (long long i = pos0 + gw; i < pos1; i += nw) {
        const long long j = a.order ? (long long)a.order[i] : i;  // sample of position i
        const long long s = a.begin + j;
        const tuned::Out o{a.out_a, a.out_b, j, a.out_f64};
        const double ra = a.ra[s], dec = a.dec[s], pa = a.pa[s];
        if constexpr (kPlanned)
            tuned::sample_planned<kCalib, kBil>(plans[i - pos0], hs, a.rings, hb, B, ra, dec, pa, o,
                                                S, Q, lane, a.err, g, nfall, cmax, npairs);
        else
            tuned::sample<kCalib, kBil>(hs, a.rings, hb, B, ra, dec, pa, o, S, Q, lane, a.err, g,
                                        nfall, cmax, npairs);
    }
    tuned::flush<kBil>(hs, S, Q, lane, a.err, g);
    if (lane == 0 && nfall && a.fallbacks) atomicAdd(a.fallbacks, nfall);
    if (kCalib && calib) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cmax = fmaxf(cmax, __shfl_xor_sync(tuned::kFull, cmax, o));
        if (lane == 0) {
            atomicMax((int*)calib, __float_as_int(cmax));
            atomicAdd(reinterpret_cast<unsigned long long*>(calib + 2), npairs);
        }
    }
}

// The sample plans of positions [pos0, pos1), one thread per sample.
__global__ void plan_kernel(FwdArgs a, tuned::SamplePlan* __restrict__ plans, long long pos0,
                            long long pos1)
{
    const Hpx hs = hpx_make(a.nside_sky);
    const tuned::Beam B = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    for (long long i = pos0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < pos1;
         i += (long long)gridDim.x * blockDim.x) {
        const long long j = a.order ? (long long)a.order[i] : i;
        const long long s = a.begin + j;
        plans[i - pos0] = tuned::make_plan(hs, B, a.ra[s], a.dec[s], a.pa[s]);
    }
}
static_assert(sizeof(tuned::SamplePlan) == kSamplePlanBytes, "sample plan size");

__global__ void ring_table_kernel(int nside, RingT* rings)
{
    const Hpx h = hpx_make(nside);
    const long long nr = 4LL * nside - 1;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x + 1; r <= nr;
         r += (long long)gridDim.x * blockDim.x) {
        const RingInfo ri = ring_info(h, r);
        const double z = ring2z(h, r);
        const double s = sqrt(PD_MUL(PD_SUB(1.0, z), PD_ADD(1.0, z)));
        RingT t;
        t.z = z;
        t.omz2 = PD_SUB(1.0, PD_MUL(z, z));
        t.dec = atan2(z, s);
        t.fr = PD_MUL((double)ri.npix, kInvTwoPi);
        t.dphi = PD_DIV(kTwoPi, (double)ri.npix);
        t.s = (float)s;
        t.dphif = (float)t.dphi;
        t.zf = (float)z;
        t.start = (int)ri.start;
        t.npix2 = (int)(2 * ri.npix + (ri.shifted ? 1 : 0));
        rings[r - 1] = t;
    }
}

template <class K>
int resident_blocks(K kernel, int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    return nb;
}

template <bool kCalib, bool kBil, int kTW, bool kPlanned>
void launch_shape(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib,
                  tuned::SamplePlan* plans, long long plan_cap)
{
    const int threads = kTW * 32;
    const long long resident =
        (long long)sm_count * resident_blocks(tuned_kernel<kCalib, kBil, kTW, kPlanned>, threads);
    const long long step = kPlanned ? plan_cap : a.n;
    for (long long p0 = 0; p0 < a.n; p0 += step) {
        const long long p1 = p0 + step < a.n ? p0 + step : a.n;
        if (kPlanned) {
            const long long pb = (p1 - p0 + 255) / 256;
            plan_kernel<<<(int)(pb < 65536 ? pb : 65536), 256, 0, st>>>(a, plans, p0, p1);
        }
        const long long need = (p1 - p0 + kTW - 1) / kTW;
        tuned_kernel<kCalib, kBil, kTW, kPlanned>
            <<<(int)(resident < need ? resident : need), threads, 0, st>>>(a, calib, plans, p0, p1);
    }
}

// kTW: the planned launch's block; without plans the warps build their own
// (FP64 disc plan in the loop's registers), which spills at 64 registers, so
// that launch keeps 16 warps per SM.  A planned launch of fewer than four
// samples per resident warp uses blocks of 8 warps (4 per SM), so that its
// samples spread over every SM (32-warp blocks would fill n / 32 SMs).
template <bool kBil, int kTW>
void launch_lookup(const FwdArgs& a, int sm_count, cudaStream_t st, tuned::SamplePlan* plans,
                   long long plan_cap)
{
    constexpr int kUnplanned = kTW > 16 ? 16 : kTW;
    if (plans && plan_cap > 0) {
        const long long chunk = plan_cap < a.n ? plan_cap : a.n;
        if (kTW > 8 && chunk < 4LL * sm_count * kTW)
            launch_shape<false, kBil, (kTW > 8 ? 8 : kTW), true>(a, sm_count, st, nullptr, plans, plan_cap);
        else
            launch_shape<false, kBil, kTW, true>(a, sm_count, st, nullptr, plans, plan_cap);
    } else {
        launch_shape<false, kBil, kUnplanned, false>(a, sm_count, st, nullptr, nullptr, 0);
    }
}

cudaError_t launch_tuned_impl(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib,
                              tuned::SamplePlan* plans, long long plan_cap)
{
    if (a.n <= 0) return cudaSuccess;
    // calibration measures the nearest-pixel decisions, whatever the lookup
    if (calib) launch_shape<true, false, 16, false>(a, sm_count, st, calib, nullptr, 0);
    else if (a.interp == 1) launch_lookup<true, PISCO_BIL_WARPS>(a, sm_count, st, plans, plan_cap);
    else launch_lookup<false, PISCO_FWD_WARPS>(a, sm_count, st, plans, plan_cap);
    return cudaGetLastError();
}

}  // namespace

bool tuned_supported(int nside_beam, int npix_beam, double rho_max)
{
    // The FP32 geometry uses the polar-cap branch of the beam grid's
    // ang2pix: every pair must land in a ring well inside the north cap.
    if (!(rho_max > 0.0) || rho_max > 0.5) return false;
    const double ring = nside_beam * sqrt(3.0 * (1.0 - cos(rho_max)));
    if (ring + 2.0 >= nside_beam) return false;
    const long long ncap = 2LL * nside_beam * (nside_beam - 1);
    return npix_beam <= ncap;
}

cudaError_t launch_ring_table(int nside, RingT* rings, cudaStream_t st)
{
    if (nside < 1 || nside > 8192 || !rings) return cudaErrorInvalidValue;
    const long long nr = 4LL * nside - 1;
    ring_table_kernel<<<(int)((nr + 255) / 256), 256, 0, st>>>(nside, rings);
    return cudaGetLastError();
}

cudaError_t launch_forward_tuned(const FwdArgs& a, int sm_count, cudaStream_t st, void* plans,
                                 long long plan_cap)
{
    return launch_tuned_impl(a, sm_count, st, nullptr, static_cast<tuned::SamplePlan*>(plans),
                             plan_cap);
}

cudaError_t launch_tuned_calibrate(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib)
{
    return launch_tuned_impl(a, sm_count, st, calib, nullptr, 0);
}

}  // namespace pisco
