// adjoint_planned.cu -- the adjoint's kernels reading sample plans built
// beforehand: adjoint_plan_kernel builds each sample's FP64 geometry (its
// disc, frame and psi phasors; tuned_core.cuh make_plan) with one thread per
// sample, then the kernels of adjoint_kernels.cuh run with kPlanned (the
// nearest lookup at 32 warps per SM).  The plans are the values the warps
// would build, so the pairs and their values are the same: the fixed-point
// (DETERMINISTIC) sky and beam gradients are the same bit for bit, while the
// parameter gradient's per-warp partial sums follow the launch's warps.
#include <cuda_runtime.h>

#include "adjoint_kernels.cuh"

namespace pisco {
namespace {

// Positions [0, a.n): plans[i] is the plan of sample a.begin + order(i).
__global__ void adjoint_plan_kernel(AdjArgs a)
{
    const Hpx hs = hpx_make(a.nside_sky);
    const tuned::Beam B = tuned::make_beam(a.beam32, a.nside_beam, a.npix_beam, a.rho_max);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long j = a.order ? (long long)a.order[i] : i;
        const long long s = a.begin + j;
        a.plans[i] = tuned::make_plan(hs, B, a.ra[s], a.dec[s], a.pa[s]);
    }
}

}  // namespace

cudaError_t launch_adjoint_planned(const AdjArgs& a, int sm_count, cudaStream_t st, int* nwarps)
{
    if (nwarps) *nwarps = 0;
    if (a.n <= 0) return cudaSuccess;
    const long long b = (a.n + 255) / 256;
    adjoint_plan_kernel<<<(int)(b < 65536 ? b : 65536), 256, 0, st>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_adjoint_impl<true>(a, sm_count, st, nwarps);
}

}  // namespace pisco
