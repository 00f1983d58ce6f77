// adjoint.cu -- the adjoint's entry points into the kernels of
// adjoint_kernels.cuh (each warp planning its own samples; the planned
// kernels are in adjoint_planned.cu) and the fixed-order reductions around
// them: the bounds that set the DETERMINISTIC fixed-point scales, the
// fixed-point to float conversions and the fold of the per-warp parameter
// rows.
#include <cuda_runtime.h>

#include "adjoint_kernels.cuh"

namespace pisco {
namespace {

// Sum of the per-warp rows (6 doubles each) in warp order per thread, then a
// fixed tree: one partial row in the layout of the Gaussian model's sums
// (column 1: sum s g; columns 7..11: sum s dg/dt; the rest zero).
__global__ void __launch_bounds__(256) fold_params_kernel(const double* ppart, int nwarps,
                                                          double* row)
{
    __shared__ double sh[6][256];
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = threadIdx.x; w < nwarps; w += 256)
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] += ppart[6 * w + k];
#pragma unroll
    for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
#pragma unroll
            for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < kParamCols) {
        const int c = threadIdx.x;
        row[c] = c == 1 ? sh[0][0] : (c >= 7 ? sh[c - 6][0] : 0.0);
    }
}

// Fixed-order partial sums of |ga| + |gb| (one per block, then one block).
__global__ void abs_sum_kernel(const void* ga, const void* gb, int f64, long long n, double* part)
{
    __shared__ double sh[256];
    double v = 0.0;
    for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += 256ll * gridDim.x) {
        const double x = f64 ? ((const double*)ga)[i] : (double)((const float*)ga)[i];
        const double y = f64 ? ((const double*)gb)[i] : (double)((const float*)gb)[i];
        if (isfinite(x)) v += fabs(x);
        if (isfinite(y)) v += fabs(y);
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// max |component| of a float array, fixed order (blocks -> one block).
__global__ void abs_max_kernel(const float* x, long long n, double* part)
{
    __shared__ double sh[256];
    double v = 0.0;
    for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += 256ll * gridDim.x)
        if (isfinite(x[i])) v = fmax(v, fabs((double)x[i]));
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void fold_kernel(double* part, int nb, int is_max)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v = 0.0;
    for (int i = 0; i < nb; ++i) v = is_max ? fmax(v, part[i]) : v + part[i];
    part[0] = v;
}

__global__ void fixed_to_float_kernel(const unsigned long long* in, void* out, int out_f64,
                                      long long n, double inv_scale)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)(long long)in[i] * inv_scale;
        if (out_f64) ((double*)out)[i] = v;
        else ((float*)out)[i] = (float)v;
    }
}

// The DETERMINISTIC sky accumulator (planes [4][npix]) to the interleaved
// [npix][4] gradient.
__global__ void fixed_planes_kernel(const unsigned long long* in, void* out, int out_f64,
                                    long long npix, double inv_scale)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 4 * npix;
         i += (long long)gridDim.x * blockDim.x) {
        const long long p = i >> 2, k = i & 3;
        const double v = (double)(long long)in[k * npix + p] * inv_scale;
        if (out_f64) ((double*)out)[i] = v;
        else ((float*)out)[i] = (float)v;
    }
}

}  // namespace


constexpr int kRedBlocks = 256;

cudaError_t launch_abs_sum(const void* ga, const void* gb, int f64, long long n, double* part,
                           cudaStream_t st)
{
    abs_sum_kernel<<<kRedBlocks, 256, 0, st>>>(ga, gb, f64, n, part);
    fold_kernel<<<1, 32, 0, st>>>(part, kRedBlocks, 0);
    return cudaGetLastError();
}

cudaError_t launch_abs_max(const float* x, long long n, double* part, cudaStream_t st)
{
    abs_max_kernel<<<kRedBlocks, 256, 0, st>>>(x, n, part);
    fold_kernel<<<1, 32, 0, st>>>(part, kRedBlocks, 1);
    return cudaGetLastError();
}

cudaError_t launch_fixed_to_float(const unsigned long long* in, void* out, int out_f64, long long n,
                                  double inv_scale, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    fixed_to_float_kernel<<<1024, 256, 0, st>>>(in, out, out_f64, n, inv_scale);
    return cudaGetLastError();
}

int adjoint_max_warps(int sm_count) { return sm_count * 32 * kAW; }

cudaError_t launch_fold_params(const double* ppart, int nwarps, double* row, cudaStream_t st)
{
    fold_params_kernel<<<1, 256, 0, st>>>(ppart, nwarps, row);
    return cudaGetLastError();
}

cudaError_t launch_fixed_planes_to_float(const unsigned long long* in, void* out, int out_f64,
                                         long long npix, double inv_scale, cudaStream_t st)
{
    if (npix <= 0) return cudaSuccess;
    fixed_planes_kernel<<<1024, 256, 0, st>>>(in, out, out_f64, npix, inv_scale);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const AdjArgs& a, int sm_count, cudaStream_t st, int* nwarps)
{
    if (a.plans) return launch_adjoint_planned(a, sm_count, st, nwarps);
    return launch_adjoint_impl<false>(a, sm_count, st, nwarps);
}

}  // namespace pisco
