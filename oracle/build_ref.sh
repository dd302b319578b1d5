#!/usr/bin/env bash
# Build the oracle pins.
#
#   oracle/liboracle.so   -- the C restatement (oracle/qg_oracle.c); always built.
#   oracle/_ref/ref_tool  -- the reference's own generator, validators and DP
#                            planner compiled from the reference checkout where
#                            the sources lie (only when that checkout exists).
#   oracle/_ref/libref_kernels.so
#                         -- the reference's own OpenCL kernels (filter, sort,
#                            group-by, aggregation, hash build/probe) compiled as
#                            C++ through oracle/ref_kernels/clshim.h and driven
#                            by oracle/ref_kernels/*.cpp (same condition).  The
#                            kernel files are compiled from copies in
#                            oracle/_ref/kernels/ in which `__local int *`
#                            parameters lose their `__local` (a qualifier C++
#                            cannot express on a parameter); nothing else in
#                            them changes.
#
# Usage: oracle/build_ref.sh [REFERENCE_CHECKOUT]
# The reference checkout is the first argument, else $QG_REFERENCE_DIR; with
# neither (or a path that does not exist) only liboracle.so is built.
#
# Test infrastructure only.  Outputs go to oracle/ and oracle/_ref/ (both
# git-ignored build products).  The reference sources are read in place and
# never copied.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${QG_REFERENCE_DIR:-}}"

CC=${CC:-gcc}
if ! $CC -O2 -fPIC -shared -fopenmp -o "$HERE/liboracle.so" "$HERE/qg_oracle.c" 2>/dev/null; then
    $CC -O2 -fPIC -shared -o "$HERE/liboracle.so" "$HERE/qg_oracle.c"
fi

if [ -n "$REF" ] && [ -d "$REF/host/host" ]; then
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

if [ -n "$REF" ] && [ -d "$REF/kernel" ]; then
    OUT="$HERE/_ref"
    K="$OUT/kernels"
    mkdir -p "$K"
    for f in kernel/filter/filter_op.cl kernel/aggregation/1/group_by_cu_op_dp.cl \
             kernel/hj_filter_sort/1/hj_filter_sort_op.cl; do
        sed -E 's/__local[[:space:]]+(u?int)[[:space:]]*\*/\1 */g' "$REF/$f" > "$K/$(basename "$f")"
    done
    CXX=${CXX:-g++}
    RK="$HERE/ref_kernels"
    CXXF="-O2 -std=c++17 -fPIC -w -fpermissive -I$RK"
    $CXX $CXXF -DREF_FILTER_CL="\"$K/filter_op.cl\"" -c "$RK/ref_filter.cpp" -o "$K/ref_filter.o" & p1=$!
    $CXX $CXXF -DREF_GROUPBY_CL="\"$K/group_by_cu_op_dp.cl\"" -c "$RK/ref_groupby.cpp" -o "$K/ref_groupby.o" & p2=$!
    $CXX $CXXF -DREF_JOIN_CL="\"$K/hj_filter_sort_op.cl\"" -c "$RK/ref_join.cpp" -o "$K/ref_join.o" & p3=$!
    wait $p1
    wait $p2
    wait $p3
    $CXX -shared -o "$OUT/libref_kernels.so" "$K/ref_filter.o" "$K/ref_groupby.o" "$K/ref_join.o" -lpthread
fi
