#!/usr/bin/env bash
# Build the oracle pins.
#
#   oracle/liboracle.so   -- the C restatement (oracle/qg_oracle.c); always built.
#   oracle/_ref/ref_tool  -- the reference's own generator, validators and DP
#                            planner compiled from the reference checkout where
#                            the sources lie (only when that checkout exists).
#
# Test infrastructure only.  Outputs go to oracle/ and oracle/_ref/ (both
# git-ignored build products).  The reference sources are read in place and
# never copied.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${QG_REFERENCE_DIR:-/root/reference}"

CC=${CC:-gcc}
if ! $CC -O2 -fPIC -shared -fopenmp -o "$HERE/liboracle.so" "$HERE/qg_oracle.c" 2>/dev/null; then
    $CC -O2 -fPIC -shared -o "$HERE/liboracle.so" "$HERE/qg_oracle.c"
fi

if [ -d "$REF/host/host" ]; then
    OUT="$HERE/_ref"
    mkdir -p "$OUT/stub/CL"
    cp "$HERE/ref_stub/CL/opencl.h" "$OUT/stub/CL/opencl.h"
    # host/host/common.h:1 includes "CL\cl.h" with a backslash.
    printf '#include "CL/opencl.h"\n' > "$OUT/stub/CL\\cl.h"
    CXX=${CXX:-g++}
    $CXX -O1 -std=c++17 -w -fpermissive \
        -I"$OUT/stub" -I"$REF/host/host" -I"$REF/host/host/src" \
        "$HERE/ref_tool.cpp" \
        "$REF/host/host/generator.cpp" \
        "$REF/host/host/Validate.cpp" \
        "$REF/host/dynamic_programming.cpp" \
        -o "$OUT/ref_tool"
fi
