#!/bin/sh
# Compiles the reference's own path-tracing code (its shaders/*.cu device
# code, BVH builders and exposure program, unmodified, from the reference
# source tree) for the host CPU together with our driver
# oracle/ref_harness/ref_harness.cpp, into oracle/_ref/libkpt_ref_host.so.
# The output is used only to generate and check the golden fixtures under
# tests/golden/; it is never committed.  Needs the reference tree (default
# /root/reference, or $KPT_REFERENCE) and the CUDA headers.
set -e
here=$(cd "$(dirname "$0")" && pwd)
R=${KPT_REFERENCE:-/root/reference}/KittlesPT
CUDA=${CUDA_HOME:-/usr/local/cuda}
[ -d "$R/src" ] || { echo "reference source tree not found at $R" >&2; exit 2; }
mkdir -p "$here/_ref/shim/GL"
: > "$here/_ref/shim/GL/gl.h"    # cuda_gl_interop.h includes <GL/gl.h>; no GL calls are made
${CXX:-g++} -std=c++17 -O2 -fPIC -fno-semantic-interposition -shared -ffp-contract=off -fpermissive -w -x c++ \
    -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
    -include "$here/ref_harness/ref_prelude.h" \
    -I"$CUDA/include" -I"$CUDA/include/cccl" -I"$here/_ref/shim" \
    -I"$R/src" -I"$R/thirdparty" -I"$R/thirdparty/glad/include" \
    "$here/ref_harness/ref_harness.cpp" -o "$here/_ref/libkpt_ref_host.so" -lpthread
echo "built $here/_ref/libkpt_ref_host.so"
