#!/bin/sh
# Compiles the slice of the reference's vendored HYPRE 2.33.0 that OpFlow's HYPREEqnSolveHandler with
# PrecondStructSolver<PCG, PFMG> calls -- utilities, krylov (pcg.c), struct_mv (matvec, grids,
# vectors) and struct_ls (PFMG, the struct PCG interface) -- directly with the C compiler into
# oracle/_ref/hypre/libHYPRE_struct.a, without HYPRE's CMake/configure.  The generated configuration
# header is replaced by oracle/ref/shim_hypre/HYPRE_config.h (serial, double, host memory).
# Test infrastructure only: ref_solve (oracle/ref/ref_solve.cpp) links it to pin the GPU solves.
set -e
if [ -z "$OPFLOW_REFERENCE" ]; then echo "set OPFLOW_REFERENCE to the OpFlow source tree" >&2; exit 1; fi
H="$OPFLOW_REFERENCE/external/hypre/src"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref/hypre"
if [ ! -f "$H/HYPRE.h" ]; then echo "HYPRE sources not found under $H" >&2; exit 1; fi
INC="-I$HERE/ref/shim_hypre -I$H -I$H/utilities -I$H/krylov -I$H/struct_mv -I$H/struct_ls -I$H/sstruct_mv -I$H/sstruct_ls -I$H/parcsr_mv -I$H/parcsr_ls -I$H/IJ_mv -I$H/seq_mv -I$H/blas -I$H/lapack -I$H/multivector"
mkdir -p "$OUT/obj"
: > "$OUT/objs.txt"
for d in utilities krylov struct_mv struct_ls; do
  for f in "$H"/$d/*.c; do
    echo "$f $OUT/obj/${d}_$(basename "$f" .c).o" >> "$OUT/objs.txt"
  done
done
# compile in parallel; an object is rebuilt only when missing
JOBS=${JOBS:-$(nproc 2>/dev/null || echo 4)}
awk '{print $1" "$2}' "$OUT/objs.txt" | xargs -P "$JOBS" -n 2 sh -c \
  '[ -f "$1" ] || ${CC:-gcc} -O2 -fPIC -w '"$INC"' -c "$0" -o "$1"'
rm -f "$OUT/libHYPRE_struct.a"
ar rcs "$OUT/libHYPRE_struct.a" $(awk '{print $2}' "$OUT/objs.txt")
echo "$INC" > "$OUT/include_flags.txt"
echo "built $OUT/libHYPRE_struct.a"
