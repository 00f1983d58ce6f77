// ref_gpu_kernels.cu -- TEST INFRASTRUCTURE ONLY.  One translation unit made of
// the reference's own device sources (src/GpuConvolver/cuda/cudaHealpix.cu,
// cudaSphtransf.cu, cudaConv2.cu), which build_ref.sh reads in place from the
// reference tree (-I) and compiles unmodified into oracle/_ref/refconv.cubin
// for sm_103a with the reference's nvcc options (CMakeLists.txt:57-61, minus
// the sm_52 target).  oracle/ref_gpu_harness.cpp loads the cubin and runs the
// reference's kernels K1 and K2 as its GPUConvolver does.
#include "cudaHealpix.cu"
#include "cudaSphtransf.cu"
#include "cudaConv2.cu"
