#!/bin/sh
# Builds the reference's own CPU code for the hemicube shoot path into oracle/_ref/.
#
# TEST INFRASTRUCTURE ONLY: the library this makes is the checker that pins the
# oracle restatement (oracle/oracle.c) and the product's host-side scene / camera
# code; nothing in the product links it.
#
# The reference is MSVC C++ (source/*.cpp).  The translation units used here are
# compiled from patched copies written into oracle/_ref/src/ (git-ignored, never
# committed).  The patches are mechanical portability fixes only:
#   * MSVC functional casts `unsigned int(x)`   -> `(unsigned int)(x)`
#     (source/Config.cpp:37-39, source/Patch.cpp:88-89, source/FormFactors.cpp:307,
#      source/Colors.cpp:116-118)
#   * `#include "model.h"` -> "Model.h" (case-sensitive file system)
#   * `static enum` / `const enum` -> `enum` (source/Camera.h:18, source/PrimitiveModel.h:16)
#   * <windows.h>, <crtdbg.h>, "OpenGL30Drv.h" and `__int32` replaced by tiny shims.
# No arithmetic is touched.  Usage:  sh oracle/build_ref.sh [reference_root]
set -e
REF=${1:-${RADIOSITY_REFERENCE:-/root/reference}}
SRCDIR="$REF/source"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$SRCDIR" ]; then
    echo "build_ref.sh: reference sources not found at $SRCDIR; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/src"

FILES="Config.cpp Config.h Patch.cpp Patch.h Model.cpp Model.h PrimitiveModel.cpp PrimitiveModel.h
ModelContainer.cpp ModelContainer.h WaveFrontModel.cpp WaveFrontModel.h LoadingModel.cpp LoadingModel.h
FormFactors.cpp FormFactors.h Vector.cpp Vector.h Transform.cpp Transform.h Camera.cpp Camera.h
Timer.cpp Timer.h Colors.cpp Colors.h Kernel_ProcessHemicube.h"
for f in $FILES; do
    sed -e 's/unsigned int(/(unsigned int)(/g' \
        -e 's/#include "model.h"/#include "Model.h"/' \
        -e 's/static enum/enum/' -e 's/const enum/enum/' \
        -e 's/#include <windows.h>//' -e 's/#include "OpenGL30Drv.h"//' \
        -e 's/#include <crtdbg.h>/#include "crtdbg_shim.h"/' \
        -e 's/\r$//' \
        "$SRCDIR/$f" > "$OUT/src/$f"
done
cat > "$OUT/src/crtdbg_shim.h" <<'EOF'
#pragma once
#define _ASSERT(x) ((void)0)
#define _ASSERTE(x) ((void)0)
EOF

CXX=${CXX:-g++}
FLAGS="-O2 -fPIC -fpermissive -w -ffp-contract=off -fno-fast-math -std=gnu++11 -D__int32=int -include crtdbg_shim.h -include algorithm -include cstring -I$OUT/src"
OBJS=""
for f in Config Patch Model PrimitiveModel ModelContainer WaveFrontModel LoadingModel FormFactors Vector Transform Camera Colors; do
    $CXX $FLAGS -c "$OUT/src/$f.cpp" -o "$OUT/src/$f.o" &
    OBJS="$OBJS $OUT/src/$f.o"
done
$CXX $FLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/src/ref_driver.o" &
wait
$CXX -shared -o "$OUT/libradref.so" $OBJS "$OUT/src/ref_driver.o"

# The reference's own delta-form-factor sum self-check (source/FormFactors.cpp:87-108,
# normally disabled by a commented-out #define) built as a stand-alone program.
$CXX $FLAGS -D__SUM_TEST -c "$OUT/src/FormFactors.cpp" -o "$OUT/src/FormFactors_sum.o"
$CXX $FLAGS -o "$OUT/ffsum" "$HERE/ref_ffsum_main.cpp" "$OUT/src/FormFactors_sum.o" "$OUT/src/Config.o"
echo "built $OUT/libradref.so and $OUT/ffsum"
