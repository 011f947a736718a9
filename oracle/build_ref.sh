#!/bin/sh
# Compiles OpFlow's own CPU path (header-only C++ under the reference tree named by $OPFLOW_REFERENCE)
# into oracle/_ref/:
#   ref_driver  (oracle/ref/ref_driver.cpp): explicit evaluation, padding and StencilPad assembly dumps;
#   ref_solve   (oracle/ref/ref_solve.cpp):  HYPREEqnSolveHandler + PrecondStructSolver<PCG, PFMG>
#               over the vendored HYPRE struct solvers (built by oracle/build_hypre.sh).
# Used only to generate and re-check the golden fixtures under tests/golden/; nothing in the package
# links either binary.
#
# The reference needs C++26 and several external pieces that this toolchain (g++ 13) and image lack.
# The recipe bridges them without running the reference's build system:
#   * oracle/ref/shim/ : small stand-ins written for this project -- <print>, boost::core::demangle,
#     spdlog (its calls are compiled out by `if consteval`), the generated Version.hpp, and a serial
#     stand-in for the slice of oneTBB used by rangeFor (scheduling only; OpFlow's results do not depend
#     on the thread count).
#   * oracle/_ref/gen/OpFlowCoreNoSolvers.hpp : the reference's include/Core umbrella minus its HYPRE /
#     AMGCL solver headers (ref_driver emulates HYPREEqnSolveHandler::generateAb without HYPRE).
#   * oracle/_ref/gen/OpFlowCoreHYPRE.hpp : the same umbrella plus the HYPRE handler and the Struct
#     solver wrappers, still without AMGCL (which needs Boost) and UnifiedSolve.hpp (which includes it).
#   * oracle/_ref/gen/Core/Meta.hpp : the reference's Meta.hpp with its two C++26 pack-indexing
#     aliases (`T...[0]`, `T...[sizeof...(T) - 1]`) rewritten as std::tuple_element_t, generated by sed
#     at build time and never committed.
set -e
if [ -z "$OPFLOW_REFERENCE" ]; then echo "set OPFLOW_REFERENCE to the OpFlow source tree" >&2; exit 1; fi
REF="$OPFLOW_REFERENCE"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src/Core" ]; then echo "reference tree not found at $REF" >&2; exit 1; fi
mkdir -p "$OUT/gen/Core"
sed -e 's/T\.\.\.\[0\]/std::tuple_element_t<0, std::tuple<T...>>/' \
    -e 's/T\.\.\.\[sizeof\.\.\.(T) - 1\]/std::tuple_element_t<sizeof...(T) - 1, std::tuple<T...>>/' \
    "$REF/src/Core/Meta.hpp" > "$OUT/gen/Core/Meta.hpp"
grep -v -E 'HYPRE|AMGCL|Solvers/|UnifiedSolve|CSRMatrixGenerator|EquationHolder|StencilHolder' \
    "$REF/include/Core" > "$OUT/gen/OpFlowCoreNoSolvers.hpp"
grep -v -E 'AMGCL|UnifiedSolve|CSRMatrixGenerator|EquationHolder|StencilHolder|Solvers/SemiStruct/SemiStructSolverFAC|Solvers/IJ' \
    "$REF/include/Core" > "$OUT/gen/OpFlowCoreHYPRE.hpp"
CXXFLAGS="-std=c++23 -O2 -ffp-contract=off -w -include numeric -I$OUT/gen -I$HERE/ref/shim -I$HERE/ref -I$REF/src -I$REF/include"
${CXX:-g++} $CXXFLAGS -fopenmp -o "$OUT/ref_driver" "$HERE/ref/ref_driver.cpp" &
"$HERE/build_hypre.sh" > /dev/null
${CXX:-g++} $CXXFLAGS $(cat "$OUT/hypre/include_flags.txt") -o "$OUT/ref_solve" "$HERE/ref/ref_solve.cpp" \
    "$OUT/hypre/libHYPRE_struct.a" -lm
wait
echo "built $OUT/ref_driver $OUT/ref_solve"
