#!/usr/bin/env bash
# Build oracle/_ref/ref_harness: the reference's own method-0 kernels
# (label_propagation/src/dpp/kernel.cuh, src/common/segmented_reduce.cuh) and
# host helpers (include/graph.h, src/common/outofcore.cuh), compiled from the
# reference tree where it lies and run on the CPU through oracle/refsim/simt_shim.h,
# plus the reference's loaders (include/graph.h) and accuracy measures (include/accuracy.h).
# Test infrastructure only.  Needs the reference tree: $GALP_REFERENCE, else a
# directory named "reference" beside the repository; exits 0 without building when it
# is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${GALP_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}"
LP="$REF/label_propagation"
if [ ! -f "$LP/src/common/segmented_reduce.cuh" ]; then
    echo "build_ref: reference tree not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
# The kernels of segmented_reduce.cuh end where `struct SegmentedReducer` (host
# launch code) begins; only that prefix is fed to the compiler, through a pipe.
g++ -std=c++17 -O2 -w -fopenmp \
    -include "$HERE/refsim/simt_shim.h" \
    -include <(sed '/^struct SegmentedReducer/,$d' "$LP/src/common/segmented_reduce.cuh") \
    -I "$HERE/refsim" -I "$LP/src" -I "$LP/include" \
    "$HERE/refsim/ref_harness.cpp" -o "$HERE/_ref/ref_harness"
echo "build_ref: built $HERE/_ref/ref_harness" >&2
# The reference's edge-list converter (utils/edgelist2bin.cpp), to check galp_convert.
if [ -f "$REF/utils/edgelist2bin.cpp" ]; then
    g++ -std=c++14 -O2 -w "$REF/utils/edgelist2bin.cpp" -o "$HERE/_ref/edgelist2bin"
fi
