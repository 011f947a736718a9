#!/bin/sh
# Compiles OpFlow's own CPU path (header-only C++ under the reference tree) together with
# oracle/ref/ref_driver.cpp into oracle/_ref/ref_driver.  Used only to generate and re-check the
# golden fixtures under tests/golden/; nothing in the package links it.
#
# The reference needs C++26 and several external pieces that this toolchain (g++ 13) and image lack.
# The recipe bridges them without running the reference's build system:
#   * oracle/ref/shim/ : small stand-ins written for this project -- <print>, boost::core::demangle,
#     spdlog (its calls are compiled out by `if consteval`), the generated Version.hpp, and a serial
#     stand-in for the slice of oneTBB used by rangeFor (scheduling only; OpFlow's results do not depend
#     on the thread count).
#   * oracle/_ref/gen/OpFlowCoreNoSolvers.hpp : the reference's include/Core umbrella minus its HYPRE /
#     AMGCL solver headers (the driver emulates HYPREEqnSolveHandler::generateAb without HYPRE).
#   * oracle/_ref/gen/Core/Meta.hpp : the reference's Meta.hpp with its two C++26 pack-indexing
#     aliases (`T...[0]`, `T...[sizeof...(T) - 1]`) rewritten as std::tuple_element_t, generated by sed
#     at build time and never committed.
set -e
REF=${OPFLOW_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src/Core" ]; then echo "reference tree not found at $REF" >&2; exit 1; fi
mkdir -p "$OUT/gen/Core"
sed -e 's/T\.\.\.\[0\]/std::tuple_element_t<0, std::tuple<T...>>/' \
    -e 's/T\.\.\.\[sizeof\.\.\.(T) - 1\]/std::tuple_element_t<sizeof...(T) - 1, std::tuple<T...>>/' \
    "$REF/src/Core/Meta.hpp" > "$OUT/gen/Core/Meta.hpp"
# Umbrella of the reference's Core headers without the HYPRE / AMGCL solver layer (those need the
# vendored HYPRE and Boost builds, which this recipe does not perform).
grep -v -E 'HYPRE|AMGCL|Solvers/|UnifiedSolve|CSRMatrixGenerator|EquationHolder|StencilHolder' \
    "$REF/include/Core" > "$OUT/gen/OpFlowCoreNoSolvers.hpp"
${CXX:-g++} -std=c++23 -O2 -ffp-contract=off -fopenmp -w -include numeric \
    -I"$OUT/gen" -I"$HERE/ref/shim" -I"$REF/src" -I"$REF/include" \
    -o "$OUT/ref_driver" "$HERE/ref/ref_driver.cpp"
echo "built $OUT/ref_driver"
