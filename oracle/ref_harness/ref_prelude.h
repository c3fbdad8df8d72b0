// ref_prelude.h -- force-included when the reference's own device code is
// compiled for the host CPU (oracle/build_ref.sh).  It gives g++ the view of
// the reference headers that nvcc has when it compiles the reference:
//
// * helper_math (maths/vector_types_extension.cuh) is included with
//   __CUDACC__ defined, so its host-only fallbacks (a NaN-asymmetric fminf,
//   int-only min/max, rsqrtf) are compiled out exactly as under nvcc, and the
//   float/int min/max overloads that CUDA's math headers provide are declared
//   here instead;
// * surf2Dread/surf2Dwrite act on float4 images held by the harness
//   (cudaBoundaryModeClamp reads, out-of-range writes dropped);
// * the few CUDA built-ins the reference kernels touch (thread indices,
//   __syncthreads, atomicAdd, bit casts) get host equivalents so that
//   shaders/histogram.cu and shaders/bloom.cu compile; their kernel bodies
//   then run one thread at a time.
//
// It also supplies two things the reference's MSVC toolchain accepted:
// a unary minus on const float3& and __forceinline__ after inline.
#pragma once
#include <cfloat>
#include <cmath>
#include <math.h>   // the C++ wrapper: float overloads of pow, log2, ... in the global namespace,
                    // as CUDA's and MSVC's headers provide them
#include <cstdint>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include <device_launch_parameters.h>

using std::isnan;
using std::isinf;

#undef __forceinline__
#define __forceinline__ __attribute__((always_inline))

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline double max(float a, double b) { return fmax((double)a, b); }
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }

#define __CUDACC__
#include "maths/vector_types_extension.cuh"
#undef __CUDACC__

inline float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned int u) { float f; std::memcpy(&f, &u, 4); return f; }

struct HostSurface { float4* data; int w, h; };
inline std::vector<HostSurface>& host_surfaces() { static std::vector<HostSurface> v(1); return v; }
template <class T>
inline T surf2Dread(cudaSurfaceObject_t s, int xb, int y, cudaSurfaceBoundaryMode = cudaBoundaryModeTrap) {
    HostSurface& hs = host_surfaces()[s];
    int x = xb / (int)sizeof(float4);
    if (x < 0) x = 0;
    if (x > hs.w - 1) x = hs.w - 1;
    if (y < 0) y = 0;
    if (y > hs.h - 1) y = hs.h - 1;
    return hs.data[(size_t)y * hs.w + x];
}
template <class T>
inline void surf2Dwrite(T v, cudaSurfaceObject_t s, int xb, int y, cudaSurfaceBoundaryMode = cudaBoundaryModeTrap) {
    HostSurface& hs = host_surfaces()[s];
    int x = xb / (int)sizeof(float4);
    if (x < 0 || y < 0 || x >= hs.w || y >= hs.h) return;
    hs.data[(size_t)y * hs.w + x] = v;
}

// one-thread-at-a-time stand-ins for the launch built-ins (the CUDA header
// declares them const; the names are redirected to writable variables)
inline uint3 kpt_host_threadIdx;
inline uint3 kpt_host_blockIdx;
inline dim3 kpt_host_blockDim;
#define threadIdx kpt_host_threadIdx
#define blockIdx kpt_host_blockIdx
#define blockDim kpt_host_blockDim
inline void __syncthreads() {}
template <class T> inline T atomicAdd(T* p, T v) { T o = *p; *p = o + v; return o; }
