// ref_gpu_prelude.h -- force-included when the reference's own CUDA code is
// compiled for the GPU (oracle/build_ref.sh gpu).  It supplies what the
// reference's MSVC toolchain accepted and nvcc with g++ does not:
//
// * <cfloat> and <cstdint>, which the reference's headers use without
//   including them;
// * __forceinline__ written after `inline` (maths/vector_maths.cuh:46) --
//   CUDA's own definition of the macro repeats `inline`, so it is redefined
//   to the attribute alone;
// * a unary minus on const float3& (the helper_math overload in
//   maths/vector_types_extension.cuh takes a non-const reference).
//
// TEST INFRASTRUCTURE ONLY: used to build the reference's megakernel as the
// GPU baseline and GPU oracle, never by the product.
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>    // CUDA's own headers first, under CUDA's definition of
#include <cuda_bf16.h>    // __forceinline__ (they define functions with it)

#undef __forceinline__
#define __forceinline__ __attribute__((always_inline))

inline __host__ __device__ float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
