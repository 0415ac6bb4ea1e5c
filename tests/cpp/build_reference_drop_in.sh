#!/usr/bin/env bash
# build_reference_drop_in.sh -- compiles the GB300 device policy INTO the reference's own
# general_heston_equation (TEST INFRASTRUCTURE ONLY).
#
# Takes the patched build-time copy of the reference that oracle/build_ref.sh makes
# (oracle/_ref/src), copies it to oracle/_ref/dropin/src (git-ignored) and applies the two
# additions a maintainer makes: the enumerator tridiagonal_method_enum::GB300ThomasLUSolver
# (common/lss_enumerations.hpp) and the Device dispatch branch in
# implicit_solvers::general_heston_equation::solve
# (pde_solvers/two_dimensional/heat_type/lss_2d_general_heston_equation.hpp); the kernel
# specialisation itself is linear_system_solvers_gb300/cpp/lss_gb300_reference_kernel.hpp.
# Then builds tests/cpp/reference_drop_in_t.cu against that copy and liblss_adi.so into
# oracle/_ref/dropin/reference_drop_in_t.  Exit 3: no reference copy or library to build from.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
SRC="$ROOT/oracle/_ref/src"
OUT="$ROOT/oracle/_ref/dropin"
LIBDIR="$ROOT/linear_system_solvers_gb300/_build"
BIN="$OUT/reference_drop_in_t"
[ -f "$SRC/.patched" ] || { echo "build_reference_drop_in.sh: no patched reference copy at $SRC" >&2; exit 3; }
[ -f "$LIBDIR/liblss_adi.so" ] || { echo "build_reference_drop_in.sh: liblss_adi.so not built" >&2; exit 3; }
if [ -x "$BIN" ] && [ "$BIN" -nt "$HERE/reference_drop_in_t.cu" ] && [ "$BIN" -nt "$0" ] && \
   [ "$BIN" -nt "$ROOT/linear_system_solvers_gb300/cpp/lss_gb300_reference_kernel.hpp" ] && \
   [ "$BIN" -nt "$ROOT/include/lss_adi.h" ]; then
    echo "build_reference_drop_in.sh: $BIN is up to date"
    exit 0
fi
rm -rf "$OUT/src"
mkdir -p "$OUT"
cp -r "$SRC" "$OUT/src"
python3 - "$OUT/src" <<'PY'
import sys, os
root = sys.argv[1]
p = os.path.join(root, "common", "lss_enumerations.hpp")
s = open(p).read()
old = "    ThomasLUSolver,\n};"
assert s.count(old) == 1, "enumerator anchor"
s = s.replace(old, "    ThomasLUSolver,\n    GB300ThomasLUSolver,\n};")
open(p, "w").write(s)
p = os.path.join(root, "pde_solvers", "two_dimensional", "heat_type", "lss_2d_general_heston_equation.hpp")
s = open(p).read()
old = """        else
        {
            throw std::runtime_error("Not supported on Device");
        }"""
assert s.count(old) == 1, "dispatch anchor"
new = """        else if (solver_cfg_->tridiagonal_method() == tridiagonal_method_enum::GB300ThomasLUSolver)
        {
            typedef general_heston_equation_implicit_kernel<memory_space_enum::Device,
                                                            tridiagonal_method_enum::GB300ThomasLUSolver, fp_type,
                                                            container, allocator>
                dev_gb300_solver;
            dev_gb300_solver solver(ver_boundary_ptr, hor_boundary_pair_ptr, heat_data_trans_cfg_, discretization_cfg_,
                                    splitting_method_cfg_, solver_cfg_, grid_cfg);
            solver(prev_sol, next_sol, is_heat_source_set, heat_source);
            solution = next_sol;
        }
""" + old
s = s.replace(old, new)
open(p, "w").write(s)
PY
CUS=$(cd "$OUT/src" && find . -name '*.cu' ! -name main.cu | sort | sed "s|^\.|$OUT/src|")
nvcc -std=c++17 -O2 -arch="${LSS_REF_ARCH:-sm_100}" -Xcompiler -ffp-contract=off \
    -include cmath -include stdexcept -I"$OUT/src" -I"$ROOT/include" -I"$ROOT/linear_system_solvers_gb300/cpp" \
    "$HERE/reference_drop_in_t.cu" $CUS -o "$BIN" -L"$LIBDIR" -llss_adi -Xlinker -rpath -Xlinker "$LIBDIR" \
    -lcusolver -lcusparse -lcublas
echo "build_reference_drop_in.sh: built $BIN"
