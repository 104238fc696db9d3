#!/usr/bin/env bash
# Compiles the reference's own SEM sources (SEMmesh.cpp, SEMsolver.cpp and the header-only
# finite-element code) from where they lie under the reference checkout, together with
# oracle/ref_harness.cpp, into oracle/_ref/libsemref_q<order>.so.  Test infrastructure only.
#
# The reference's CMake build needs its empty BLT submodule, so it is not used.  In its plain
# std::vector mode (USE_VECTOR) the SEM path needs no third-party library.  The polynomial
# order is a compile-time constant there (SEMdata.hpp) and the element scratch arrays are sized
# by ROW (SEMmacros.hpp, 64 = order 3), so for each order this writes patched copies of those
# two headers and a one-line commonConfig.hpp into oracle/_ref/shadow_q<order>/, which is put
# first on the include path.  Everything written goes under oracle/_ref/ (git-ignored).
#
# Usage: oracle/build_ref.sh [reference-root]
# The root of the reference checkout comes from the argument or else from SEMGB_REFERENCE_ROOT;
# with neither, nothing is built (the tests that need the compiled reference then skip).
set -euo pipefail
REF="${1:-${SEMGB_REFERENCE_ROOT:-}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ -z "$REF" ]; then
    echo "no reference checkout given (argument or SEMGB_REFERENCE_ROOT): compiled reference not built" >&2
    exit 0
fi
if [ ! -f "$REF/src/sem/solver/SEMsolver.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 1
fi
mkdir -p "$OUT"
build_one() {
    local Q=$1
    local SH="$OUT/shadow_q$Q"
    mkdir -p "$SH"
    printf '#ifndef COMMON_CONFIG_HPP\n#define COMMON_CONFIG_HPP\n#define USE_VECTOR\n#endif\n' > "$SH/commonConfig.hpp"
    sed -e "s/static constexpr int myOrderNumber=2;/static constexpr int myOrderNumber=$Q;/" \
        "$REF/src/sem/main/SEMdata.hpp" > "$SH/SEMdata.hpp"
    grep -q "myOrderNumber=$Q;" "$SH/SEMdata.hpp"
    sed -e "s/#define ROW 64/#define ROW 216/" "$REF/src/sem/main/SEMmacros.hpp" > "$SH/SEMmacros.hpp"
    grep -q "#define ROW 216" "$SH/SEMmacros.hpp"
    g++ -O2 -std=c++20 -fPIC -shared -ffp-contract=off -w \
        -I"$SH" -I"$REF/src/utils" -I"$REF/src/sem/finiteElements" -I"$REF/src/sem/mesh" \
        -I"$REF/src/sem/solver" -I"$REF/src/sem/main" \
        "$HERE/ref_harness.cpp" "$REF/src/sem/mesh/SEMmesh.cpp" \
        -o "$OUT/libsemref_q$Q.so"
}
for Q in 1 2 3 4 5; do
    build_one "$Q" &
done
wait
ls "$OUT"/libsemref_q*.so
