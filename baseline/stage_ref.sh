#!/usr/bin/env bash
# Stages the reference's own sources (its src/ directory, unmodified) from the
# reference checkout named by GLISSER_REF_DIR into baseline/_ref/src, which is
# git-ignored: the copy never enters this repository's history, but it travels
# with the working tree to a GPU machine, where baseline/build_ref_gpu.sh
# compiles the reference's CUDA time-block path for timing and
# oracle/build_ref.sh its CPU path for the oracle's pin and the CPU baseline.
set -euo pipefail
REF="${GLISSER_REF_DIR:?set GLISSER_REF_DIR to the reference checkout}"
HERE="$(cd "$(dirname "$0")" && pwd)"
DST="$HERE/_ref/src"
if [ ! -f "$REF/src/wh.cu" ]; then
    echo "reference sources not found at $REF/src" >&2
    exit 2
fi
mkdir -p "$DST"
cp "$REF"/src/*.h "$REF"/src/*.cuh "$REF"/src/*.cu "$REF"/src/*.cpp "$DST"/
echo "staged $(ls "$DST" | wc -l) reference source files in $DST"
