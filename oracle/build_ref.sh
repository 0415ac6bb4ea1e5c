#!/usr/bin/env bash
# build_ref.sh -- compile the reference's own host ADI path into oracle/_ref/ref_driver and its
# 1-D implicit heat path into oracle/_ref/ref_driver_1d.
#
# TEST INFRASTRUCTURE ONLY.  Reads the reference sources where they lie ($LSS_REFERENCE_DIR,
# else a `reference` folder beside the repository's folder), copies the headers it needs into
# oracle/_ref/src (git-ignored, never committed), applies four mechanical portability
# patches (MSVC-only std::exception(const char*) ctor; two shadowed template-template
# parameter names; one decltype on a non-class), and compiles oracle/ref_driver.cu and
# oracle/ref_driver_1d.cu against them.  Host code only runs; nvcc is used because the reference headers pull in
# thrust device headers.  -ffp-contract=off keeps the reference's two-rounding a*b+c.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${LSS_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
mkdir -p "$OUT"
fresh() { [ -x "$OUT/$1" ] && [ "$OUT/$1" -nt "$HERE/$1.cu" ] && [ "$OUT/$1" -nt "$0" ]; }
if fresh ref_driver && fresh ref_driver_1d; then
    echo "build_ref.sh: $OUT/ref_driver and $OUT/ref_driver_1d are up to date"
    exit 0
fi
if [ -d "$REF/pde_solvers" ]; then
    rm -rf "$OUT/src"
    mkdir -p "$OUT/src"
    ( cd "$REF" && find . \( -name '*.hpp' -o -name '*.cu' \) ! -path './.git/*' -print0 | \
        while IFS= read -r -d '' f; do mkdir -p "$OUT/src/$(dirname "$f")"; cp "$f" "$OUT/src/$f"; done )
elif [ -d "$OUT/src/pde_solvers" ] && [ -f "$OUT/src/.patched" ]; then
    # a machine without the reference checkout (the copy made where it was present travelled
    # with the repository): rebuild the driver for this host from that patched copy
    echo "build_ref.sh: reference not at $REF, rebuilding from the patched copy in $OUT/src" >&2
else
    echo "build_ref.sh: reference not found at $REF (skipping)" >&2
    exit 0
fi
cd "$OUT/src"
if [ ! -f .patched ]; then
find . -name '*.hpp' -print0 | xargs -0 sed -i 's/std::exception(/std::runtime_error(/g'
for f in sparse_solvers/general/core_sor_solver/lss_core_sor_solver.hpp \
         sparse_solvers/general/core_sor_solver_cuda/lss_core_sor_solver_cuda.hpp; do
    sed -i 's/template <typename fp_type, typename allocator> typename container/template <typename, typename> typename container/' "$f"
    sed -i 's/template <template <typename fp_type> typename traits>/template <template <typename> typename traits>/' "$f"
done
sed -i 's/decltype(errors)::value_type(0.0)/fp_type(0.0)/' sparse_solvers/general/core_sor_solver_cuda/lss_core_sor_solver_cuda.hpp
touch .patched
fi
CUS=$(find . -name '*.cu' ! -name main.cu | sort)
ARCH="${LSS_REF_ARCH:-sm_100}"
for d in ref_driver ref_driver_1d; do
    fresh "$d" && continue
    nvcc -std=c++17 -O2 -arch="$ARCH" -Xcompiler -ffp-contract=off \
        -include cmath -include stdexcept -I"$OUT/src" \
        "$HERE/$d.cu" $CUS -o "$OUT/$d" -lcusolver -lcusparse -lcublas &
done
wait
for d in ref_driver ref_driver_1d; do
    [ -x "$OUT/$d" ] || { echo "build_ref.sh: building $d failed" >&2; exit 1; }
done
echo "build_ref.sh: built $OUT/ref_driver and $OUT/ref_driver_1d"
