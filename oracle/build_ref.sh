#!/bin/sh
# Builds oracle/_ref/ (TEST INFRASTRUCTURE ONLY) from the reference's own
# sources: the reference tree ($PISCO_REFERENCE, default the directory
# "reference" beside this repository) when it is present, else the copy of
# its src/ folder that an earlier run on a machine with the tree staged in
# oracle/_ref/src_tree/.  Everything under oracle/_ref/ is git-ignored and
# never committed: the staged copy only lets a machine without the reference
# tree (and of another architecture) compile the reference's own code
# itself.  Outputs go to oracle/_ref/ only.
#   libpisco_ref.so    : Convolver, Sky, Scan, PolBeam, Sphtrigo compiled
#                        unmodified with the reference's CPU flags
#                        (CMakeLists.txt:27,37-39) against the HEALPix shim
#                        in oracle/shim/ (Healpix C++ itself is absent).
#   libpisco_refmap.so : the binned map-maker SkyMap (skymap.cpp), same flags;
#   libpisco_refmap_exact.so: the same without floating-point contraction;
#                        LAPACK's dgesv_ is the oracle's restatement.
#   libpisco_refdev.so : the reference's device HEALPix port and device
#                        rotation (cudaHealpix.cu, cudaSphtransf.cu)
#                        compiled for the host with __device__ removed.
#   refconv.cubin      : the reference's device code (cudaHealpix.cu,
#                        cudaSphtransf.cu, cudaConv2.cu: kernels K1, K2)
#                        compiled unmodified for sm_103a, loaded at run time
#                        by oracle/ref_gpu_harness.cpp.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PISCO_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
STAGE="$OUT/src_tree"
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
if [ -f "$REF/src/Convolver/convolver.cpp" ]; then
    # only the folders this recipe compiles (about 170 KB)
    rm -rf "$STAGE"
    mkdir -p "$STAGE/src"
    for d in Convolver Sky Scan Polbeam Sphtrigo SkyMap GpuConvolver; do
        cp -R "$REF/src/$d" "$STAGE/src/$d"
    done
elif [ -f "$STAGE/src/Convolver/convolver.cpp" ]; then
    REF="$STAGE"
else
    echo "build_ref.sh: reference tree not found at $REF and no staged copy; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/obj"
gcc -O2 -fPIC -fopenmp -ffp-contract=off -c "$HERE/oracle.c" -o "$OUT/obj/oracle.o"
CXXF="-O3 -march=native -fopenmp -pthread -DCONVOLVER_OPENMPENABLED -fPIC -w -I$REF/src -I$HERE/shim -I$HERE"
for f in Convolver/convolver Sky/sky Scan/scan Polbeam/polbeam Sphtrigo/sphtrigo; do
    g++ $CXXF -c "$REF/src/$f.cpp" -o "$OUT/obj/$(basename $f).o" &
done
g++ $CXXF -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
wait
g++ -shared -fopenmp -o "$OUT/libpisco_ref.so" "$OUT"/obj/convolver.o "$OUT"/obj/sky.o \
    "$OUT"/obj/scan.o "$OUT"/obj/polbeam.o "$OUT"/obj/sphtrigo.o "$OUT"/obj/ref_harness.o \
    "$OUT"/obj/oracle.o
# binned map-maker (src/SkyMap/skymap.cpp): with the reference's flags, and
# once more without floating-point contraction (a bit-exact pin of the
# oracle's restatement); skymap.cpp uses std::cerr and malloc without their
# headers, which -include supplies.
MAPF="-include iostream -include cstdlib -include cstdio -include cmath"
g++ $CXXF $MAPF -c "$REF/src/SkyMap/skymap.cpp" -o "$OUT/obj/skymap.o"
g++ $CXXF $MAPF -ffp-contract=off -c "$REF/src/SkyMap/skymap.cpp" -o "$OUT/obj/skymap_exact.o"
g++ $CXXF -c "$HERE/ref_map_harness.cpp" -o "$OUT/obj/ref_map_harness.o"
g++ -shared -fopenmp -o "$OUT/libpisco_refmap.so" "$OUT"/obj/skymap.o "$OUT"/obj/ref_map_harness.o \
    "$OUT"/obj/oracle.o
g++ -shared -fopenmp -o "$OUT/libpisco_refmap_exact.so" "$OUT"/obj/skymap_exact.o \
    "$OUT"/obj/ref_map_harness.o "$OUT"/obj/oracle.o
DEVF="-O2 -fPIC -w -x c++ -D__device__= -include cmath -include math.h -I$REF/src -I$REF/src/GpuConvolver/cuda -I$CUDA_INC"
g++ $DEVF -c "$REF/src/GpuConvolver/cuda/cudaHealpix.cu" -o "$OUT/obj/cudaHealpix.o"
g++ $DEVF -c "$REF/src/GpuConvolver/cuda/cudaSphtransf.cu" -o "$OUT/obj/cudaSphtransf.o"
g++ -O2 -fPIC -w -I$REF/src -I$CUDA_INC -D__device__= -c "$HERE/refdev_harness.cpp" -o "$OUT/obj/refdev_harness.o"
g++ -shared -o "$OUT/libpisco_refdev.so" "$OUT"/obj/cudaHealpix.o "$OUT"/obj/cudaSphtransf.o \
    "$OUT"/obj/refdev_harness.o
NVCC=${CUDA_HOME:-/usr/local/cuda}/bin/nvcc
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I"$REF/src/GpuConvolver/cuda" \
    -o "$OUT/refconv.cubin" "$HERE/ref_gpu_kernels.cu"
echo "build_ref.sh: built $OUT/libpisco_ref.so, libpisco_refmap*.so, libpisco_refdev.so and refconv.cubin"
