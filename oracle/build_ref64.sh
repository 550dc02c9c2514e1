#!/bin/sh
# oracle/build_ref64.sh — test infrastructure: the FP64 oracle.
#
#   sh oracle/build_ref64.sh N
#
# Builds oracle/_ref/libflipref64_nN.so: the reference's own sources with
# FLOAT set to double (src/common.h:10) and the driver's grid size N
# (src/flip3D.cpp:25) set to N, plus oracle/ref_harness.cpp. The reference
# tree is read-only, so the sources are copied into oracle/_ref/src64_nN/ and
# the two #define lines are edited there; nothing else changes. Compiled with
# the same flags and -include workarounds as the float build in
# oracle/Makefile. Needs the reference tree (build container only).
set -eu
N="$1"
REF="${REF:-/root/reference/src}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src64_n$N"
OBJ="$OUT/obj64_n$N"
CXX="${CXX:-g++}"

rm -rf "$SRC" "$OBJ"
mkdir -p "$SRC" "$OBJ"
cp -r "$REF"/. "$SRC"/
sed -i 's/^#define[[:space:]]\{1,\}FLOAT[[:space:]]\{1,\}float[[:space:]]*$/#define FLOAT double/' "$SRC/common.h"
sed -i "s/^#define[[:space:]]\{1,\}N[[:space:]]\{1,\}32[[:space:]]*\$/#define N $N/" "$SRC/flip3D.cpp"
grep -q '^#define FLOAT double$' "$SRC/common.h" || { echo "FLOAT define not found" >&2; exit 1; }
grep -q "^#define N $N\$" "$SRC/flip3D.cpp" || { echo "N define not found" >&2; exit 1; }

FLAGS="-O3 -fPIC -fopenmp -ffp-contract=off -w -I$SRC -I$SRC/rchandra"
INC="-include cmath -include limits -include vector -include map"
pids=""
cc() { $CXX $FLAGS $INC "$@" & pids="$pids $!"; }
for f in sorter mapper kernel implicit mesher exporter write_bmp; do
  cc -include algorithm -c "$SRC/$f.cpp" -o "$OBJ/$f.o"
done
cc -include algorithm -include "$HERE/ref_patch_rand.h" -c "$SRC/corrector.cpp" -o "$OBJ/corrector.o"
cc -include algorithm -Dmy_rand_shuffle=flipref_unused_shuffle -c "$SRC/utility.cpp" -o "$OBJ/utility.o"
cc -include algorithm -Dsolve=flipref_solver_solve_impl -c "$SRC/solver.cpp" -o "$OBJ/solver.o"
cc -include algorithm -c "$SRC/rchandra/CIsoSurface.cpp" -o "$OBJ/CIsoSurface.o"
cc -include algorithm -c "$SRC/rchandra/Vectors.cpp" -o "$OBJ/Vectors.o"
cc -c "$HERE/ref_harness.cpp" -o "$OBJ/ref_harness.o"
for p in $pids; do wait "$p"; done
$CXX -shared -fopenmp -o "$OUT/libflipref64_n$N.so" "$OBJ"/*.o
echo "$OUT/libflipref64_n$N.so"
