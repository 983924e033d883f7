#!/usr/bin/env bash
# Compiles the reference solvers, unchanged, from their own sources into oracle/_ref/.
#
# These binaries are test infrastructure: the golden-fixture script and the CPU
# baseline run them as the checker.  Nothing in the product links or runs them.
#
#   k_cops_visibility     solvers/k_cops_visibility.cpp    (v1, 2p-column retrograde)
#   k_cops_visibility_v2  solvers/k_cops_visibility_v2.cpp (v2, macro-turn search)
#   k_cops_4              legacy/src/k_cops_4.cpp          (multithreaded, stay-allowed rules)
#   k_cops_visibility_stayCR  solvers/k_cops_visibility.cpp with its two self-edge switches
#                         (lines 63-64: SelfEdgeCop, SelfEdgeRobber) set to C, R (1 = TRUE):
#                         the stay-allowed rule sets 10, 01 and 11.  The switches are flipped in
#                         a temporary copy outside this repository; the reference tree is
#                         untouched and no reference source is kept.
#
# The reference's own build (build.py) is not used.  `-include cstddef` is needed
# because lib/include/Graph.h and AdjacencyList.h use size_t without its header
# on GCC 13.  The recipe needs the reference tree; it is skipped (exit 0) when the
# tree is absent, so a prebuilt oracle/_ref/ keeps working where it was copied.
set -euo pipefail
REF="${CR_REFERENCE_ROOT:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/solvers" ]; then
    echo "build_ref: reference tree not found at $REF; keeping existing $OUT" >&2
    exit 0
fi
mkdir -p "$OUT"
if [ -x "$OUT/k_cops_visibility" ] && [ -x "$OUT/k_cops_visibility_v2" ] && [ -x "$OUT/k_cops_4" ] \
   && [ -x "$OUT/k_cops_visibility_stay11" ] && [ -z "${CR_REBUILD_REF:-}" ]; then
    exit 0   # already built (set CR_REBUILD_REF=1 to force)
fi
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -include cstddef -Ofast -I "$REF/lib/include")
LIBSRC=("$REF/lib/src/Graph.cpp" "$REF/lib/src/AdjacencyList.cpp" "$REF/lib/src/fileio.cpp"
        "$REF/lib/src/Allocator.cpp" "$REF/lib/src/Profiler.cpp")
build_solver() {   # $1 = solver source relative to the reference root, $2 = output name
    "$CXX" "${FLAGS[@]}" "-DALGORITHM_INCLUDE=\"$REF/$1\"" "$REF/app/main.cpp" "${LIBSRC[@]}" \
        -o "$OUT/$2"
}
build_solver solvers/k_cops_visibility.cpp k_cops_visibility &
build_solver solvers/k_cops_visibility_v2.cpp k_cops_visibility_v2 &
"$CXX" "${FLAGS[@]}" -pthread "$REF/legacy/src/k_cops_4.cpp" "$REF/lib/src/Graph.cpp" \
    "$REF/lib/src/AdjacencyList.cpp" "$REF/lib/src/fileio.cpp" -o "$OUT/k_cops_4" &
STAY_TMP="$(mktemp -d)"
for rules in "TRUE FALSE 10" "FALSE TRUE 01" "TRUE TRUE 11"; do
    set -- $rules
    src="$STAY_TMP/k_cops_visibility_stay$3.cpp"
    sed -e "s/SelfEdgeCop c_edge = SelfEdgeCop::FALSE;/SelfEdgeCop c_edge = SelfEdgeCop::$1;/" \
        -e "s/SelfEdgeRobber r_edge = SelfEdgeRobber::FALSE;/SelfEdgeRobber r_edge = SelfEdgeRobber::$2;/" \
        "$REF/solvers/k_cops_visibility.cpp" > "$src"
    grep -q "SelfEdgeCop c_edge = SelfEdgeCop::$1;" "$src" && grep -q "SelfEdgeRobber r_edge = SelfEdgeRobber::$2;" "$src" \
        || { echo "build_ref: the self-edge switches were not found" >&2; exit 1; }
    "$CXX" "${FLAGS[@]}" "-DALGORITHM_INCLUDE=\"$src\"" "$REF/app/main.cpp" "${LIBSRC[@]}" \
        -o "$OUT/k_cops_visibility_stay$3" &
done
wait
rm -rf "$STAY_TMP"
echo "build_ref: built $(ls "$OUT" | tr '\n' ' ')"
