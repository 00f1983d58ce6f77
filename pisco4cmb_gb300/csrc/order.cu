// order.cu -- sky-ordered processing of a scan.
//
// The reference walks a scan in time order (convolver.cpp:38-70,
// gpuconvolver.cu:382-505).  A focal plane, a scan strategy that revisits
// the sky, or a shuffled data set then puts unrelated pointings side by side,
// and the warps running at one moment gather from scattered disc
// footprints.  In sky order the samples of a forward range are sorted by a
// Z-order (Morton) code of their boresight's cell on a 2^16 x 2^16 grid
// equal-area in (phi, z), so the warps resident at one moment hold
// neighbouring pointings whose footprints overlap in L2 and L1.
//
// Output stays in scan order: a kernel takes position i of the sorted order,
// reads sample order[i] and writes its TOD (or reads its TOD gradient) at
// order[i].  Every sample's result is independent of the order in which the
// samples are processed (the TUNED kernels keep their re-evaluation sums per
// sample), so both orders give bit-identical TOD.  An out-of-date order (a
// scan changed in place) costs locality only: the kernels still visit every
// position once.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include "ctx.h"
#include "internal.h"

namespace pisco {
namespace {

// Spreads the low 16 bits of x to the even bit positions.
__device__ __forceinline__ unsigned spread16(unsigned x)
{
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// Key of each sample (non-finite pointings last) and its position.
__global__ void order_keys_kernel(long long n, const double* ra, const double* dec,
                                  unsigned* keys, int* pos)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double r = ra[i], d = dec[i];
        unsigned key = 0xffffffffu;
        if (isfinite(r) && isfinite(d)) {
            float sr, cr, sd, cd;
            sincosf((float)fmod(r, 6.283185307179586), &sr, &cr);
            sincosf((float)fmod(d, 6.283185307179586), &sd, &cd);
            float phi = atan2f(cd * sr, cd * cr);
            if (phi < 0.0f) phi += 6.2831853f;
            const float fx = phi * (65536.0f / 6.2831853f);
            const float fy = (sd + 1.0f) * 32768.0f;
            const unsigned ix = fx >= 65535.0f ? 65535u : (fx > 0.0f ? (unsigned)fx : 0u);
            const unsigned iy = fy >= 65535.0f ? 65535u : (fy > 0.0f ? (unsigned)fy : 0u);
            key = spread16(ix) | (spread16(iy) << 1);
            if (key == 0xffffffffu) key = 0xfffffffeu;
        }
        keys[i] = key;
        pos[i] = (int)i;
    }
}

}  // namespace

cudaError_t sky_order(long long n, const double* ra, const double* dec, unsigned* keys,
                      unsigned* keys_sorted, int* pos, int* order, void* tmp, size_t* tmp_bytes,
                      cudaStream_t st)
{
    if (!tmp) {
        return cub::DeviceRadixSort::SortPairs(nullptr, *tmp_bytes, keys, keys_sorted, pos, order,
                                               (int)n, 0, 32, st);
    }
    if (n <= 0) return cudaSuccess;
    const long long blocks = (n + 255) / 256;
    order_keys_kernel<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(n, ra, dec, keys, pos);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cub::DeviceRadixSort::SortPairs(tmp, *tmp_bytes, keys, keys_sorted, pos, order, (int)n,
                                           0, 32, st);
}

}  // namespace pisco
