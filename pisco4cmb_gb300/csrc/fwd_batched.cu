// fwd_batched.cu -- many detector pairs (each with its own beam, scan and
// TOD) in one persistent launch fed by a (detector, sample-chunk) work queue.
//
// The reference handles one detector pair per GPUConvolver and launches two
// synchronising kernels per ptgPerConv chunk (gpuconvolver.cu:382-505); a
// focal plane of uneven detectors (beam radii 1-5 deg, 10k-1M samples) then
// leaves the GPU idle in every tail.  Here the host cuts every detector's
// samples into chunks, orders the chunks longest-first (estimated pairs),
// and one kernel whose blocks pull chunks with one atomic each runs them all
// (the warps of a block share a chunk, sample by sample).
// The launch (queue reset, the plan kernel that builds every sample's FP64
// geometry with one thread per sample, the batched kernel) is captured once
// in a CUDA graph and replayed while the same detector set is resubmitted.  The chunk size and
// the block shape (warps per block) are chosen by the autotuner
// (pisco_autotune_batched) and cached per workload key in a JSON file.
//
// Per sample the TUNED geometry of tuned_core.cuh runs unchanged, so every
// detector's TOD equals its single-detector TUNED forward bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "ctx.h"
#include "tuned_core.cuh"

using namespace pisco;

namespace pisco {
namespace {


// A block pulls one item at a time and its warps take the item's samples
// round-robin, so the warps of an SM work on neighbouring samples (whose
// discs overlap) at the same moment, as in the single-detector launch.
// The block's current item, set up once by thread 0.
struct ItemState {
    Hpx hb;
    tuned::Beam B;
    const double* ra;
    const double* dec;
    const double* pa;
    void* out_a;
    void* out_b;
    const int* order;  // position -> sample, or null
    long long begin, end;
    long long plan_base;
    int state;  // 0: queue empty, 1: run, 2: bad item (skipped)
};

// Every detector's sample plans (position p of detector d at
// plans[plan_base + p]; the bases ascend with d and end at a.nplans), one
// thread per sample over all detectors at once: the FP64 per-sample geometry
// the warps would otherwise build themselves (tuned_core.cuh make_plan).
__global__ void batched_plan_kernel(BatchArgs a)
{
    const Hpx hs = hpx_make(a.nside_sky);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < a.nplans;
         g += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = a.ndet - 1;  // the last detector whose plans start at or before g
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.dets[mid].plan_base <= g) lo = mid;
            else hi = mid - 1;
        }
        const BatchDet& det = a.dets[lo];
        const long long p = g - det.plan_base;
        if (p < 0 || p >= det.n) {
            tuned::record(a.err, kCheckQueue);
            continue;
        }
        const tuned::Beam B = tuned::make_beam(det.beam, det.nside_beam, det.npix_beam, det.rho_max);
        const long long s = det.order ? (long long)det.order[p] : p;
        a.plans[g] = tuned::make_plan(hs, B, det.ra[s], det.dec[s], det.pa[s]);
    }
}

// Warps per SM of an instance: the planned nearest lookup runs 32 (register
// cap 64: its per-sample plan and the descriptors are in shared memory, as in
// the single-detector launch), the others 16 (cap 128).
template <bool kBil, bool kPlanned>
constexpr int warps_per_sm()
{
    return kPlanned && !kBil ? 32 : 16;
}

// kBil: bilinear beam lookup (tuned_core.cuh bilinear_f32).  kW: warps per
// block, the tile the autotuner picks with the chunk size; every tile of an
// instance keeps the same warps per SM (warps_per_sm / kW blocks), so all
// compile to the same register cap and differ in how many warps share an
// item (and its samples' discs).  kPlanned: the samples' plans come from
// batched_plan_kernel.
template <bool kBil, int kW, bool kPlanned>
__global__ void __launch_bounds__(kW * 32, warps_per_sm<kBil, kPlanned>() / kW)
    batched_kernel(BatchArgs a)
{
    constexpr int kBW = kW;
    __shared__ tuned::WarpSmem sm[kBW];
    __shared__ ItemState s_item[2];
    __shared__ Hpx s_hs;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    tuned::WarpSmem& S = sm[warp];
    if (threadIdx.x == 0) s_hs = hpx_make(a.nside_sky);
    __syncthreads();
    const Hpx& hs = s_hs;
    unsigned long long nfall = 0, npairs = 0;
    float cmax = 0.0f;
    tuned::Gather g;
    g.sky = a.sky32;
    tuned::Queue Q{0, 0};
    for (int round = 0;; ++round) {
        // double-buffered: a slot is rewritten only after the next barrier,
        // which every thread reaches after it is done with the slot
        ItemState& T = s_item[round & 1];
        if (threadIdx.x == 0) {
            const int item = (int)atomicAdd(a.queue, 1u);
            T.state = 0;
            if (item < a.nitems) {
                const BatchItem it = a.items[item];
                if (it.det < 0 || it.det >= a.ndet) {
                    tuned::record(a.err, kCheckQueue);
                    T.state = 2;
                } else {
                    const BatchDet& d = a.dets[it.det];
                    T.hb = hpx_make(d.nside_beam);
                    T.B = tuned::make_beam(d.beam, d.nside_beam, d.npix_beam, d.rho_max);
                    T.ra = d.ra;
                    T.dec = d.dec;
                    T.pa = d.pa;
                    T.out_a = d.out_a;
                    T.out_b = d.out_b;
                    T.order = d.order;
                    T.plan_base = d.plan_base;
                    T.begin = it.begin;
                    T.end = it.begin + it.count;
                    T.state = 1;
                }
            }
        }
        __syncthreads();
        const int state = T.state;
        if (state == 0) break;
        if (state == 2) continue;
        for (long long p = T.begin + warp; p < T.end; p += kBW) {
            const long long s = T.order ? (long long)T.order[p] : p;  // sample of position p
            const tuned::Out o{T.out_a, T.out_b, s, a.out_f64};
            if constexpr (kPlanned)
                tuned::sample_planned<false, kBil>(a.plans[T.plan_base + p], hs, a.rings, T.hb, T.B,
                                                   T.ra[s], T.dec[s], T.pa[s], o, S, Q, lane, a.err,
                                                   g, nfall, cmax, npairs);
            else
                tuned::sample<false, kBil>(hs, a.rings, T.hb, T.B, T.ra[s], T.dec[s], T.pa[s], o,
                                           S, Q, lane, a.err, g, nfall, cmax, npairs);
        }
    }
    tuned::flush<kBil>(hs, S, Q, lane, a.err, g);
    if (lane == 0 && nfall && a.fallbacks) atomicAdd(a.fallbacks, nfall);
}

}  // namespace

namespace {

// Resident blocks of an instance on the whole GPU (its persistent grid).
template <bool kBil, int kW, bool kPlanned>
int grid_of(int sm_count)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel<kBil, kW, kPlanned>, kW * 32,
                                                      0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    return sm_count * nb;
}

template <bool kBil, int kW, bool kPlanned>
void launch_one(const BatchArgs& a, int sm_count, cudaStream_t st)
{
    batched_kernel<kBil, kW, kPlanned><<<grid_of<kBil, kW, kPlanned>(sm_count), kW * 32, 0, st>>>(a);
}

template <int kW>
void launch_shape(const BatchArgs& a, int sm_count, cudaStream_t st)
{
    if (a.plans) {
        const long long pb = (a.nplans + 255) / 256;
        batched_plan_kernel<<<(int)(pb < 65536 ? pb : 65536), 256, 0, st>>>(a);
        if (a.interp == 1) launch_one<true, kW, true>(a, sm_count, st);
        else launch_one<false, kW, true>(a, sm_count, st);
    } else {
        if (a.interp == 1) launch_one<true, kW, false>(a, sm_count, st);
        else launch_one<false, kW, false>(a, sm_count, st);
    }
}

}  // namespace

bool batched_warps_valid(int warps) { return warps == 4 || warps == 8 || warps == 16; }

cudaError_t launch_batched(const BatchArgs& a, int sm_count, cudaStream_t st, int warps)
{
    if (a.nitems <= 0) return cudaSuccess;
    if (warps == 4) launch_shape<4>(a, sm_count, st);
    else if (warps == 16) launch_shape<16>(a, sm_count, st);
    else launch_shape<8>(a, sm_count, st);
    return cudaGetLastError();
}

// Work list: every detector's samples in chunks of `chunk`, longest
// (estimated pairs = samples x disc size) first; ties by detector, begin.
std::vector<BatchItem> make_items(const std::vector<BatchDet>& dets, const std::vector<double>& cost,
                                  long long chunk)
{
    std::vector<BatchItem> items;
    for (int d = 0; d < (int)dets.size(); ++d)
        for (long long b = 0; b < dets[d].n; b += chunk)
            items.push_back(BatchItem{d, (int)std::min(chunk, dets[d].n - b), b});
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem& x, const BatchItem& y) {
        return (double)x.count * cost[x.det] > (double)y.count * cost[y.det];
    });
    return items;
}

}  // namespace pisco
