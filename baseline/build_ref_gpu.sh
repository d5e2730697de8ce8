#!/usr/bin/env bash
# Builds the reference's own GPU time-block path for this GPU: its src/wh.cu
# (MVSKernel, launched by WHCudaIntegrator::integrate_particles_timeblock_cuda
# through thrust::for_each, src/wh.cu:344-395) and the host sources it links
# against, compiled unmodified from the staged copy in baseline/_ref/src with
# the reference Makefile's device flags (-O3 -lineinfo -maxrregcount 64,
# Makefile:25) for sm_103a instead of its sm_35, plus baseline/ref_gpu_driver.cu,
# a C-ABI driver that sets up the reference's device state and times one
# block.  Output: baseline/_ref/libglisser_ref_gpu.so.  Measurement only.
#
# The forced includes stand in for standard headers that the reference relies
# on transitively and that GCC 13 no longer pulls in; C++11 for the .cpp files
# avoids the make_unique clash in src/util.h; nvcc needs C++17 for CCCL.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="$HERE/_ref/src"
OUT="$HERE/_ref/gpu_build"
if [ ! -f "$SRC/wh.cu" ]; then
    echo "no staged reference sources in $SRC (run baseline/stage_ref.sh)" >&2
    exit 2
fi
mkdir -p "$OUT"
INCS="-include limits -include string -include cstring -include array -include map -include cmath -include stdexcept -include algorithm"
NVTX=""
for d in /usr/local/cuda/include/nvtx3 /usr/local/cuda/targets/*/include/nvtx3; do
    [ -d "$d" ] && NVTX="-I$d" && break
done
pids=()
for f in wh convert data interp util swift; do
    g++ -std=c++11 -O3 -fPIC -w $INCS -I"$SRC" -c "$SRC/$f.cpp" -o "$OUT/$f.o" &
    pids+=($!)
done
nvcc -std=c++17 -O3 -lineinfo -maxrregcount 64 -gencode arch=compute_103a,code=sm_103a -w -Xcompiler "-fPIC -w" \
    $NVTX -I"$SRC" $INCS -c "$SRC/wh.cu" -o "$OUT/wh_cu.o" &
pids+=($!)
nvcc -std=c++17 -O3 -gencode arch=compute_103a,code=sm_103a -w -Xcompiler "-fPIC -w" $NVTX -I"$SRC" $INCS \
    -c "$HERE/ref_gpu_driver.cu" -o "$OUT/ref_gpu_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
nvcc -shared -gencode arch=compute_103a,code=sm_103a -o "$HERE/_ref/libglisser_ref_gpu.so" "$OUT"/*.o -lpthread
echo "built $HERE/_ref/libglisser_ref_gpu.so"
