// fwd_batched.cu -- many detector pairs (each with its own beam, scan and
// TOD) in one persistent launch fed by a (detector, sample-chunk) work queue.
//
// The reference handles one detector pair per GPUConvolver and launches two
// synchronising kernels per ptgPerConv chunk (gpuconvolver.cu:382-505); a
// focal plane of uneven detectors (beam radii 1-5 deg, 10k-1M samples) then
// leaves the GPU idle in every tail.  Here the host cuts every detector's
// samples into chunks, orders the chunks longest-first (estimated pairs),
// and one kernel whose warps pull chunks with one atomic each runs them all.
// The launch (queue reset + kernel) is captured once in a CUDA graph and
// replayed while the same detector set is resubmitted.  The chunk size is
// chosen by the autotuner (pisco_autotune_batched) and cached per workload
// key in a JSON file.
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

constexpr int kBW = 8;  // warps per block

__global__ void __launch_bounds__(kBW * 32, 2) batched_kernel(BatchArgs a)
{
    __shared__ tuned::WarpSmem sm[kBW];
    const int lane = threadIdx.x & 31;
    tuned::WarpSmem& S = sm[threadIdx.x >> 5];
    const Hpx hs = hpx_make(a.nside_sky);
    unsigned long long nfall = 0;
    float cmax = 0.0f;
    tuned::Gather g;
    g.sky = a.sky32;
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(a.queue, 1u);
        item = __shfl_sync(tuned::kFull, item, 0);
        if (item >= a.nitems) break;
        const BatchItem it = a.items[item];
        if (it.det < 0 || it.det >= a.ndet) {
            tuned::record(a.err, kCheckQueue);
            continue;
        }
        const BatchDet d = a.dets[it.det];
        const Hpx hb = hpx_make(d.nside_beam);
        const tuned::Beam B = {d.beam, d.nside_beam, d.npix_beam, d.rho_max, d.rscale};
        for (long long s = it.begin; s < it.begin + it.count; ++s) {
            g.reset();
            double ta = CUDART_NAN, tb = CUDART_NAN;
            if (tuned::sample<false>(hs, hb, B, d.ra[s], d.dec[s], d.pa[s], S, lane, a.err, g,
                                     nfall, cmax))
                g.total(ta, tb);
            if (lane == 0) {
                tuned::store_out(d.out_a, a.out_f64, s, ta);
                tuned::store_out(d.out_b, a.out_f64, s, tb);
            }
        }
    }
    if (lane == 0 && nfall && a.fallbacks) atomicAdd(a.fallbacks, nfall);
}

}  // namespace

int batched_grid(int sm_count)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel, kBW * 32, 0) !=
            cudaSuccess ||
        nb < 1)
        nb = 1;
    return sm_count * nb;
}

cudaError_t launch_batched(const BatchArgs& a, int grid, cudaStream_t st)
{
    if (a.nitems <= 0) return cudaSuccess;
    batched_kernel<<<grid, kBW * 32, 0, st>>>(a);
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
