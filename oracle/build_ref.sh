#!/usr/bin/env bash
# Test infrastructure only: compiles the reference's own CPU code (GammaUNC/GST)
# from its sources where they lie, into oracle/_ref/.  Nothing here is shipped
# or timed as the product.
#
# Outputs (all under oracle/_ref/, git-ignored):
#   gentenc        the reference encoder CLI (codec/command_line.cpp)
#   libgstref.so   the reference encoder + CPU rANS + CPU wavelet, behind the
#                  small C harness in oracle/ref_harness.cpp
#
# The reference's OpenCL decode path (gpu/, ans/ans_ocl.cpp, codec/decoder.cpp)
# cannot be built here: there are no OpenCL headers.  codec/entropy.cpp includes
# ans_ocl.h (which pulls in gpu.h -> CL/cl.h) but only uses declarations from
# ans.h and histogram.h, so a two-line stand-in header written below replaces it.
#
# Usage: oracle/build_ref.sh            (reference at $GST_REFERENCE_DIR or /root/reference)
set -euo pipefail

REF="${GST_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"

if [ ! -d "$REF/ans" ] || [ ! -d "$REF/codec" ]; then
  echo "build_ref.sh: reference sources not found at $REF; skipping" >&2
  exit 0
fi

mkdir -p "$OUT/shim" "$OUT/obj"
cat > "$OUT/shim/ans_ocl.h" <<'EOF'
/* Stand-in for ans/ans_ocl.h without the OpenCL runtime: entropy.cpp needs only these. */
#include "ans.h"
#include "histogram.h"
EOF

CXX="${CXX:-g++}"
CC="${CC:-gcc}"
INC=(-I"$OUT/shim" -I"$REF/ans" -I"$REF/codec" -I"$REF/lib/include"
     -I"$REF/lib/vptree/include" -I"$REF/lib/vptree/src" -I"$REF/lib")
CXXFLAGS=(-std=c++14 -O2 -fPIC -w)
CFLAGS=(-O2 -fPIC -w)

CXX_SRCS=(
  ans/decode.cpp ans/encode.cpp ans/histogram.cpp ans/ans_ocl_encode.cpp
  codec/codec_base.cpp codec/dxt_image.cpp codec/image.cpp codec/encoder.cpp
  codec/data_stream.cpp codec/entropy.cpp codec/image_processing.cpp
  codec/image_utils.cpp codec/wavelet.cpp lib/vptree/src/vptree_cpp.cc
)
C_SRCS=(lib/vptree/src/pqueue.c lib/vptree/src/vptree.c lib/vptree/src/geom.c)

pids=()
objs=()
for s in "${CXX_SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  objs+=("$o")
  "$CXX" "${CXXFLAGS[@]}" "${INC[@]}" -c "$REF/$s" -o "$o" & pids+=($!)
done
for s in "${C_SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  objs+=("$o")
  "$CC" "${CFLAGS[@]}" "${INC[@]}" -c "$REF/$s" -o "$o" & pids+=($!)
done
"$CXX" "${CXXFLAGS[@]}" "${INC[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/obj/harness.o" & pids+=($!)
"$CXX" "${CXXFLAGS[@]}" "${INC[@]}" -c "$REF/codec/command_line.cpp" -o "$OUT/obj/command_line.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

"$CXX" -shared -o "$OUT/libgstref.so" "${objs[@]}" "$OUT/obj/harness.o" -lpthread
"$CXX" -o "$OUT/gentenc" "${objs[@]}" "$OUT/obj/command_line.o" -lpthread
echo "build_ref.sh: built $OUT/libgstref.so and $OUT/gentenc"
