#!/usr/bin/env bash
# Test infrastructure: compiles the UNMODIFIED reference sources -- the staged
# copy in baseline/_ref/src (baseline/stage_ref.sh), or else the src/ directory
# of the reference checkout named by GLISSER_REF_DIR -- together with
# oracle/ref_driver.cu into oracle/_ref/libglisser_ref.so.  The library pins
# the oracle restatement, generates tests/golden/ and is the reference CPU
# baseline of bench.py; it is never shipped or linked by the product.
#
# The forced includes stand in for standard headers that the reference relies
# on transitively and that GCC 13 no longer pulls in.  C++11 for the .cpp files
# avoids the make_unique clash in src/util.h; nvcc needs C++17 for CCCL.
# -ffp-contract=off keeps the host arithmetic free of fused multiply-adds so
# that x86 and aarch64 builds of the oracle agree bit for bit.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$HERE/../baseline/_ref/src"
if [ ! -f "$SRC/wh.cu" ]; then
    SRC="${GLISSER_REF_DIR:?no staged reference sources: run baseline/stage_ref.sh or set GLISSER_REF_DIR}/src"
fi
if [ ! -f "$SRC/wh.cu" ]; then
    echo "reference sources not found at $SRC" >&2
    exit 2
fi
mkdir -p "$OUT"
INCS="-include limits -include string -include cstring -include array -include map -include cmath -include stdexcept -include algorithm"
FLAGS="-O2 -fPIC -ffp-contract=off -DNO_CUDA -w"
pids=()
for f in wh convert data interp util swift; do
    g++ -std=c++11 $FLAGS $INCS -c "$SRC/$f.cpp" -o "$OUT/$f.o" &
    pids+=($!)
done
nvcc -std=c++17 -O2 -w -Xcompiler "-fPIC -ffp-contract=off -w" -I"$SRC" $INCS \
    -c "$HERE/ref_driver.cu" -o "$OUT/ref_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
nvcc -shared -o "$OUT/libglisser_ref.so" "$OUT"/*.o
echo "built $OUT/libglisser_ref.so"
