#!/usr/bin/env bash
# Test infrastructure: compiles the UNMODIFIED reference sources where they lie
# (default /root/reference, override with GLISSER_REF_DIR) together with
# oracle/ref_driver.cu into oracle/_ref/libglisser_ref.so.  Only this
# container has the reference tree; the library pins the oracle restatement and
# generates tests/golden/.  It is never shipped or linked by the product.
#
# The forced includes stand in for standard headers that the reference relies
# on transitively and that GCC 13 no longer pulls in.  C++11 for the .cpp files
# avoids the make_unique clash in src/util.h; nvcc needs C++17 for CCCL.
# -ffp-contract=off keeps the host arithmetic free of fused multiply-adds so
# that x86 and aarch64 builds of the oracle agree bit for bit.
set -euo pipefail
REF="${GLISSER_REF_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/wh.cu" ]; then
    echo "reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
INCS="-include limits -include string -include cstring -include array -include map -include cmath -include stdexcept -include algorithm"
FLAGS="-O2 -fPIC -ffp-contract=off -DNO_CUDA -w"
pids=()
for f in wh convert data interp util swift; do
    g++ -std=c++11 $FLAGS $INCS -c "$REF/src/$f.cpp" -o "$OUT/$f.o" &
    pids+=($!)
done
nvcc -std=c++17 -O2 -Xcompiler "-fPIC -ffp-contract=off -w" -I"$REF/src" $INCS \
    -c "$HERE/ref_driver.cu" -o "$OUT/ref_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
nvcc -shared -o "$OUT/libglisser_ref.so" "$OUT"/*.o
echo "built $OUT/libglisser_ref.so"
