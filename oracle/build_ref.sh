#!/bin/bash
# TEST INFRASTRUCTURE ONLY.
# Compiles the reference's own Serial and OpenMP runner code for the STFT hot
# path straight from the reference checkout into oracle/_ref/ (git-ignored):
#   oracle/_ref/libref_serial.so   Serial runner kernels + Default_Pipeline
#   oracle/_ref/libref_openmp.so   OpenMP runner kernels + Default_Pipeline
#   oracle/_ref/libref_openmp_fast.so  same, -O3 (timing only)
# The reference's full runner cannot be built (it needs IXWebSocket and
# capnproto); only the hot path is.  A stand-in for RunnerInterface.hpp is
# generated in a temporary directory from lines 13-104 of the real header
# (types, toQuot and the runnerFunction declarations, without the server
# includes), and Default_Pipeline is taken from lines 166-318 of
# GLOBAL/RunnerCommon.cpp.  No reference source is written into the repo.
#
# The reference checkout is taken from $OCS_REFERENCE, else from a directory
# named "reference" beside this repository's root.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${OCS_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
G="$REF/StandAlone/cross_gpgpu"
if [ ! -d "$G/GLOBAL" ]; then
    echo "reference checkout not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$OUT"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
{
    printf '#pragma once\n#include <vector>\n#include <string>\n#include <optional>\n#include <iostream>\n'
    sed -n '13,104p' "$G/GLOBAL/RunnerInterface.hpp"
} > "$TMP/RunnerInterface.hpp"
{
    printf '#include "RunnerInterface.hpp"\n'
    sed -n '166,318p' "$G/GLOBAL/RunnerCommon.cpp"
} > "$TMP/pipeline.cpp"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -ffp-contract=off -fPIC -shared -w"
$CXX $FLAGS -I"$TMP" -I"$G/Serial/kernel" "$G/Serial/src/functionImpl.cpp" "$TMP/pipeline.cpp" \
    "$HERE/ref_shim.cpp" -o "$OUT/libref_serial.so"
$CXX $FLAGS -fopenmp -I"$TMP" -I"$G/OpenMP/kernel" "$G/OpenMP/src/functionImpl.cpp" "$TMP/pipeline.cpp" \
    "$HERE/ref_shim.cpp" -o "$OUT/libref_openmp.so"
$CXX -std=c++17 -O3 -fPIC -shared -w -fopenmp -I"$TMP" -I"$G/OpenMP/kernel" "$G/OpenMP/src/functionImpl.cpp" \
    "$TMP/pipeline.cpp" "$HERE/ref_shim.cpp" -o "$OUT/libref_openmp_fast.so"
echo "built $OUT"
