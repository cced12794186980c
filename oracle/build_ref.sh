#!/bin/sh
# Builds oracle/_ref/ref_gpblocks: the reference's own CPU stepper
# (GrossPitaevskii/GPBlocks.cpp + VortexState + Mesh + Output + Types), compiled
# unmodified from the reference tree, plus oracle/ref_gpblocks_harness.cpp.
# TEST INFRASTRUCTURE ONLY; needs the reference tree (default /root/reference).
set -e
REF=${SPACETIME_REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
# without the reference tree there is nothing to build: say so and succeed
[ -f "$REF/GrossPitaevskii/GPBlocks.cpp" ] || { echo "reference tree not found at $REF: oracle/_ref not built" >&2; exit 0; }
mkdir -p "$OUT"
# where the reference tree was found, for the tests that compare with its headers
echo "$REF" > "$OUT/ref_root.txt"
CXX=${CXX:-g++}
FLAGS="-O2 -ffp-contract=off -w -include $HERE/ref_compat.h -I$REF"
cd "$OUT"
$CXX $FLAGS -Dmain=gpblocks_reference_main -c "$REF/GrossPitaevskii/GPBlocks.cpp" -o GPBlocks.o &
$CXX $FLAGS -c "$REF/GrossPitaevskii/VortexState.cpp" -o VortexState.o &
$CXX $FLAGS -c "$REF/Mesh/DelaunayMesh.cpp" -o DelaunayMesh.o &
$CXX $FLAGS -c "$REF/Mesh/BuilderMesh.cpp" -o BuilderMesh.o &
$CXX $FLAGS -c "$REF/Mesh/Mesh.cpp" -o Mesh.o &
$CXX $FLAGS -c "$REF/Output/Text.cpp" -o Text.o &
$CXX $FLAGS -c "$REF/Output/Picture.cpp" -o Picture.o &
$CXX $FLAGS -c "$REF/Types/Random.cpp" -o Random.o &
$CXX $FLAGS -I"$REF" -c "$HERE/ref_gpblocks_harness.cpp" -o harness.o &
wait
$CXX -o ref_gpblocks harness.o GPBlocks.o VortexState.o DelaunayMesh.o BuilderMesh.o Mesh.o Text.o Picture.o Random.o -lm
echo "$OUT/ref_gpblocks"
