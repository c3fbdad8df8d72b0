#!/bin/sh
# Builds the reference's own path-tracing code, unmodified, for the checks and
# baselines of this repository.  TEST INFRASTRUCTURE ONLY: nothing here is
# part of the product or committed (oracle/_ref/ is git-ignored).
#
#   build_ref.sh stage  copies the reference files the builds need -- its
#                       KittlesPT/src tree and the glm and glad headers it
#                       includes -- from the reference source tree named by
#                       $KPT_REFERENCE into oracle/_ref/src, so that a machine
#                       without the reference tree can build from the copy;
#   build_ref.sh host   compiles its shaders/*.cu device code, BVH builders and
#                       exposure program for the host CPU with our driver
#                       oracle/ref_harness/ref_harness.cpp into
#                       oracle/_ref/libkpt_ref_host.so (the golden fixtures and
#                       the timed CPU baseline);
#   build_ref.sh gpu    compiles its shaders/*.cu as one CUDA translation unit
#                       for sm_103a with its GPU build's fast maths, with our
#                       driver oracle/ref_harness/ref_gpu_harness.cu, into
#                       oracle/_ref/libkpt_ref_gpu.so (its megakernel as the GPU
#                       baseline and GPU oracle);
#   build_ref.sh        stage (only when $KPT_REFERENCE is set), host and gpu.
#
# host and gpu read the staged copy.  Needs the CUDA toolkit.
set -e
here=$(cd "$(dirname "$0")" && pwd)
out="$here/_ref"
src="$out/src/KittlesPT"
CUDA=${CUDA_HOME:-/usr/local/cuda}
NVCC=${NVCC:-$CUDA/bin/nvcc}
what=${1:-all}

stage() {
    if [ -z "$KPT_REFERENCE" ]; then
        echo "build_ref.sh stage: set KPT_REFERENCE to the reference source tree (the directory holding KittlesPT/)" >&2
        exit 2
    fi
    R="$KPT_REFERENCE/KittlesPT"
    [ -d "$R/src/shaders" ] || { echo "build_ref.sh stage: no KittlesPT/src/shaders under $KPT_REFERENCE" >&2; exit 2; }
    rm -rf "$out/src"
    mkdir -p "$src/thirdparty/glad"
    cp -R "$R/src" "$src/src"
    cp -R "$R/thirdparty/glm" "$src/thirdparty/glm"
    cp -R "$R/thirdparty/glad/include" "$src/thirdparty/glad/include"
    echo "staged the reference sources in $out/src"
}

need_staged() {
    [ -d "$src/src/shaders" ] || {
        echo "build_ref.sh: no staged reference sources in $out/src; run 'KPT_REFERENCE=<tree> $0 stage' first" >&2
        exit 2
    }
    mkdir -p "$out/shim/GL"
    : > "$out/shim/GL/gl.h"    # cuda_gl_interop.h includes <GL/gl.h>; no GL calls are made
}

host() {
    need_staged
    ${CXX:-g++} -std=c++17 -O3 -fPIC -fno-semantic-interposition -shared -ffp-contract=off -fpermissive -w -x c++ \
        -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
        -include "$here/ref_harness/ref_prelude.h" \
        -I"$CUDA/include" -I"$CUDA/include/cccl" -I"$out/shim" \
        -I"$src/src" -I"$src/thirdparty" -I"$src/thirdparty/glad/include" \
        "$here/ref_harness/ref_harness.cpp" -o "$out/libkpt_ref_host.so.tmp" -lpthread -Wl,-z,defs
    mv "$out/libkpt_ref_host.so.tmp" "$out/libkpt_ref_host.so"
    echo "built $out/libkpt_ref_host.so"
}

gpu() {
    need_staged
    # -use_fast_math as the reference's own GPU build (KittlesPT.vcxproj); one
    # translation unit instead of its relocatable device code; host code
    # without contraction so the host BVH build matches the other builds
    "$NVCC" -std=c++17 -O3 -use_fast_math -gencode arch=compute_103a,code=sm_103a -lineinfo -shared \
        -Xcompiler -fPIC,-fpermissive,-ffp-contract=off -w -Xlinker -z,defs \
        -include "$here/ref_harness/ref_gpu_prelude.h" \
        -I"$out/shim" -I"$src/src" -I"$src/thirdparty" -I"$src/thirdparty/glad/include" \
        "$here/ref_harness/ref_gpu_harness.cu" -o "$out/libkpt_ref_gpu.so.tmp"
    mv "$out/libkpt_ref_gpu.so.tmp" "$out/libkpt_ref_gpu.so"
    echo "built $out/libkpt_ref_gpu.so"
}

case "$what" in
    stage) stage ;;
    host) host ;;
    gpu) gpu ;;
    all)
        if [ -n "$KPT_REFERENCE" ]; then stage; fi
        host
        gpu ;;
    *) echo "usage: $0 [stage|host|gpu]" >&2; exit 2 ;;
esac
