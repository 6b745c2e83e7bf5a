#!/bin/sh
# Compiles miniIsosurface's own CPU extraction programs from the reference
# sources where they lie, into oracle/_ref/ (git-ignored).  Test
# infrastructure: these binaries pin the oracle restatement and serve as the
# reference CPU baseline.  No reference source is copied.
#
#   flyingEdgesSerial  flyingEdges/serial/{main,FlyingEdgesAlgorithm}.cpp
#   flyingEdgesOpenMP  flyingEdges/openmp/{main,FlyingEdgesAlgorithm}.cpp
#   mcSerial           marchingCubes/serial/main.cpp
#   mcOpenMP           marchingCubes/openmp/main.cpp
#   mcOpenMPDupFree    marchingCubes/openmpDupFree/main.cpp
#   SameContentsCheck  utilities/tests/SameContentsCheck.cpp
#
# The reference's CMake files are not used (they need CMake >= 2.8 policies
# that current CMake rejects); the source lists below are the ones those
# CMakeLists.txt name.  Usage: sh oracle/build_ref.sh [reference root]
# (default: $MINIISO_REFERENCE, else the checkout's usual place).
set -e
REF=${1:-${MINIISO_REFERENCE:-/root/reference}}
OUT=$(cd "$(dirname "$0")" && pwd)/_ref
[ -d "$REF/flyingEdges" ] || { echo "no reference checkout at $REF" >&2; exit 1; }
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O3 -std=c++11 -w"
FE_UTIL="$REF/flyingEdges/util/Image3D.cpp $REF/flyingEdges/util/Timer.cpp $REF/flyingEdges/mantevoCommon/YAML_Doc.cpp $REF/flyingEdges/mantevoCommon/YAML_Element.cpp"
MC_UTIL="$REF/marchingCubes/util/Image3D.cpp $REF/marchingCubes/util/Timer.cpp $REF/marchingCubes/mantevoCommon/YAML_Doc.cpp $REF/marchingCubes/mantevoCommon/YAML_Element.cpp"
$CXX $FLAGS -o "$OUT/flyingEdgesSerial" "$REF/flyingEdges/serial/main.cpp" "$REF/flyingEdges/serial/FlyingEdgesAlgorithm.cpp" $FE_UTIL &
$CXX $FLAGS -fopenmp -o "$OUT/flyingEdgesOpenMP" "$REF/flyingEdges/openmp/main.cpp" "$REF/flyingEdges/openmp/FlyingEdgesAlgorithm.cpp" $FE_UTIL &
$CXX $FLAGS -o "$OUT/mcSerial" "$REF/marchingCubes/serial/main.cpp" $MC_UTIL &
$CXX $FLAGS -fopenmp -o "$OUT/mcOpenMP" "$REF/marchingCubes/openmp/main.cpp" $MC_UTIL &
$CXX $FLAGS -fopenmp -o "$OUT/mcOpenMPDupFree" "$REF/marchingCubes/openmpDupFree/main.cpp" $MC_UTIL &
$CXX $FLAGS -o "$OUT/SameContentsCheck" "$REF/utilities/tests/SameContentsCheck.cpp" -I"$REF/marchingCubes/util" &
wait
ls "$OUT"
