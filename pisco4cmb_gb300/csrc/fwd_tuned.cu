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

constexpr int kTW = 8;

template <bool kCalib>
__global__ void __launch_bounds__(kTW * 32, PISCO_TUNED_MINB)
    tuned_kernel(FwdArgs a, float rscale, float* calib)
{
    __shared__ tuned::WarpSmem sm[kTW];
    const int lane = threadIdx.x & 31;
    tuned::WarpSmem& S = sm[threadIdx.x >> 5];
    const Hpx hs = hpx_make(a.nside_sky);
    const Hpx hb = hpx_make(a.nside_beam);
    const tuned::Beam B = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    (void)rscale;
    const long long gw = (long long)blockIdx.x * kTW + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kTW;
    unsigned long long nfall = 0, npairs = 0;
    float cmax = 0.0f;
    tuned::Gather g;
    g.sky = a.sky32;
    tuned::Queue Q{0, 0};
    for (long long i = gw; i < a.n; i += nw) {
        const long long s = a.begin + i;
        const tuned::Out o{a.out_a, a.out_b, i, a.out_f64};
        tuned::sample<kCalib>(hs, hb, B, a.ra[s], a.dec[s], a.pa[s], o, S, Q, lane, a.err, g, nfall,
                              cmax, npairs);
    }
    tuned::flush(hs, S, Q, lane, a.err, g);
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

template <class K>
int resident_blocks(K kernel, int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    return nb;
}

cudaError_t launch_tuned_impl(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib)
{
    if (a.n <= 0) return cudaSuccess;
    const int threads = kTW * 32;
    const float rscale = (float)(1.7320508075688772 * (double)a.nside_beam);
    const long long need = (a.n + kTW - 1) / kTW;
    if (calib) {
        long long blocks = (long long)sm_count * resident_blocks(tuned_kernel<true>, threads);
        tuned_kernel<true><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, rscale, calib);
    } else {
        long long blocks = (long long)sm_count * resident_blocks(tuned_kernel<false>, threads);
        tuned_kernel<false><<<(int)(blocks < need ? blocks : need), threads, 0, st>>>(a, rscale, nullptr);
    }
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

cudaError_t launch_forward_tuned(const FwdArgs& a, int sm_count, cudaStream_t st)
{
    return launch_tuned_impl(a, sm_count, st, nullptr);
}

cudaError_t launch_tuned_calibrate(const FwdArgs& a, int sm_count, cudaStream_t st, float* calib)
{
    return launch_tuned_impl(a, sm_count, st, calib);
}

}  // namespace pisco
