// kpt_device.cuh -- device data layout and maths for the GB300 path tracer.
//
// Layout in HBM (all arrays are owned by the context, see kpt_api.cu):
//   nodes      : BvhNode[ ]   64 B per interior node; each node carries the
//                              boxes of both children, so one pop reads one
//                              64-byte record (four 16-byte loads) instead of
//                              two 32-byte child records;
//   tris       : float4[3*T]  per triangle in BVH leaf order:
//                              (v0.xyz, local id), (v1-v0, 0), (v2-v0, 0);
//   shade      : TriShade[T]  per triangle in mesh order: uvs, local
//                              geometric normal, material, emissive rank;
//   meshes     : MeshRec[ ]   BLAS root, offsets;
//   instances  : InstRec[ ]   traversal inverse, shading model matrix,
//                              material override, light range;
//   tlas       : BvhNode[ ]   same node format over instances.
//
// Arithmetic: ray/box and ray/triangle tests use IEEE round-to-nearest
// operations with no contraction (__fmul_rn, __fadd_rn, __frcp_rn), so that
// closest-hit ids and distances are bit-identical to the reference
// algorithm evaluated in IEEE single precision.  Shading follows the
// reference's GPU build (fast maths: approximate exp, sin, cos, pow,
// reciprocal and square root, FMA contraction).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kpt {

// ---------------------------------------------------------------------------
// records shared with the host code

struct __align__(16) BvhNode {
    float4 a;      // c0.min.x c0.min.y c0.min.z c0.max.x
    float4 b;      // c0.max.y c0.max.z c1.min.x c1.min.y
    float4 c;      // c1.min.z c1.max.x c1.max.y c1.max.z
    int4 d;        // c0.ref c0.count c1.ref c1.count  (count 0: interior node index)
};

struct __align__(16) TriShade {
    float2 uv0, uv1, uv2;
    float gnx, gny, gnz;      // local geometric normal (Triangle constructor)
    int material;
    int emissive_rank;        // index among the mesh's emissive triangles, -1 if none
    int pad;
};

struct __align__(16) MeshRec {
    int node_root;            // interior root node, -1 when the root is a leaf
    int leaf_first;           // root leaf: first triangle (global, leaf order)
    int leaf_count;
    int ntris;
    int tri_base;             // first triangle of this mesh in leaf-order arrays
    int shade_base;           // first triangle of this mesh in shade[]
    int n_emissive;           // emissive triangles under the mesh's own materials
    int pad;
};

struct __align__(16) InstRec {
    float4 inv[3];            // rows of the traversal inverse (object <- world)
    float4 model[3];          // rows of the shading model matrix (inverse of the inverse)
    int mesh;
    int material;             // override, -1: per-triangle materials
    int light_first;          // first light of this instance, -1: none
    int light_all;            // 1: every triangle is a light (emissive override)
    int prim_base;            // first triangle of this instance in the expanded numbering
    int pad0, pad1, pad2;
};

struct __align__(16) LightRec {  // one emissive triangle of one instance
    float3 p0, p1, p2;        // object-space vertices (Triangle::sample, triangle.cuh:104-118)
    float3 gn;                // local geometric normal
    float2 uv0, uv1, uv2;
    float area;               // object-space area, as the host computes it (pod_types.hpp:143-146)
    float tri_area;           // Triangle::getArea (triangle.cuh:120-122)
    int inst;
    int tri;                  // local triangle index (mesh order)
    int material;
    int pad;
};

constexpr int BLAS_STACK = 48;   // traversal stack entries per ray for a BLAS (the reference has 16)
constexpr int TLAS_STACK = 32;   // traversal stack entries per ray for the TLAS (the reference has 16)
constexpr int STACK_WORDS = BLAS_STACK + TLAS_STACK;

struct MatRec {  // same layout as the C-ABI kpt_material (72 bytes)
    float albedo[3];
    float metallic, roughness, transmission, ior;
    float emission[3];
    float emission_scale, normal_scale;
    int albedo_tex, orm_tex, transmission_tex, emission_tex, normal_tex, pad;
};

struct __align__(16) TexRec { int w, h, ch; long long offset; int pad; };

struct SceneView {
    const BvhNode* nodes;
    const float4* tris;
    const TriShade* shade;
    const MeshRec* meshes;
    const InstRec* inst;
    const BvhNode* tlas;
    const LightRec* lights;
    const MatRec* materials;
    const TexRec* textures;
    const uint8_t* pixels;
    long long npixels;
    int ntlas, nlights, ninst, ntextures;
    float4 tlas_lo, tlas_hi;  // root bounds of the TLAS
    int tlas_root_leaf;       // single instance: the TLAS root is that instance
    int fetch_batch;          // queue traversal: finished lanes of a warp wait for this many to fetch together
};

// Nishita and sun parameters of one frame.
struct SkyParams {
    float3 sun_dir;
    float sun_emission;
    float3 sigma_r;
    float sigma_m, sigma_am, h_r, h_m;
    float inv_h_r, inv_h_m;   // 1 / scale heights
    float earth_r, atm_r;
    float cos_half_sun;       // LeSun threshold
    float sun_radius_m;       // physical radius of the sun disc at 1 AU
    float3 sun_radiance;      // Nishita radiance towards the sun (constant per frame)
    int gpu_arith;            // 1: sky and sun in the reference GPU build's arithmetic, 0: IEEE
};

// ---------------------------------------------------------------------------
// IEEE-exact helpers (never contracted)

__device__ __forceinline__ float xm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xdot(float3 a, float3 b) {
    return xa(xa(xm(a.x, b.x), xm(a.y, b.y)), xm(a.z, b.z));
}
__device__ __forceinline__ float3 xcross(float3 a, float3 b) {
    return make_float3(xs(xm(a.y, b.z), xm(a.z, b.y)), xs(xm(a.z, b.x), xm(a.x, b.z)),
                       xs(xm(a.x, b.y), xm(a.y, b.x)));
}
__device__ __forceinline__ float3 xsub3(float3 a, float3 b) { return make_float3(xs(a.x, b.x), xs(a.y, b.y), xs(a.z, b.z)); }
__device__ __forceinline__ float3 xmul3(float3 a, float s) { return make_float3(xm(a.x, s), xm(a.y, s), xm(a.z, s)); }
__device__ __forceinline__ float3 xnormalize(float3 v) {
    float inv = __frcp_rn(__fsqrt_rn(xdot(v, v)));
    return xmul3(v, inv);
}
// row . (v, w) for a matrix row (c0, c1, c2, c3) of a column-major Mat4,
// in the order of Matrix4x4::operator* (matrix_maths.cuh:258-267)
__device__ __forceinline__ float xrow(float4 r, float3 v, float w) {
    return xa(xa(xa(xm(r.x, v.x), xm(r.y, v.y)), xm(r.z, v.z)), xm(r.w, w));
}

// ---------------------------------------------------------------------------
// fast (reference GPU build) helpers

__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) {
    a = a + b;
    return a;
}
__device__ __forceinline__ float3 operator+(float3 a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
__device__ __forceinline__ float3 operator-(float3 a, float s) { return make_float3(a.x - s, a.y - s, a.z - s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 v) { return sqrtf(dot(v, v)); }
__device__ __forceinline__ float3 normalize(float3 v) { return v * rsqrtf(dot(v, v)); }
__device__ __forceinline__ float Sqr(float v) { return v * v; }
__device__ __forceinline__ float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
__device__ __forceinline__ float saturatef_(float v) { return clampf(v, 0.0f, 1.0f); }
__device__ __forceinline__ bool nonzero(float3 v) { return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f; }
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - 2.0f * n * dot(n, i); }
__device__ __forceinline__ float AbsDot(float3 a, float3 b) { return fabsf(dot(a, b)); }
__device__ __forceinline__ float3 row3(const float4* m, float3 v, float w) {
    return make_float3(m[0].x * v.x + m[0].y * v.y + m[0].z * v.z + m[0].w * w,
                       m[1].x * v.x + m[1].y * v.y + m[1].z * v.z + m[1].w * w,
                       m[2].x * v.x + m[2].y * v.y + m[2].z * v.z + m[2].w * w);
}

constexpr float PI_F = 3.14159265358979323846f;
constexpr float INV_PI_F = 0.31830988618379067154f;
constexpr float TRI_EPS = 1.0e-5f;   // maths/constants.cuh:20
constexpr float HIT_EPS = 0.001f;    // maths/constants.cuh:21

// PCG hash sampler (shaders/samplers.cuh:9-48)
__device__ __forceinline__ uint32_t pcg_hash(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
// Argument evaluation order of the reference's three calls that draw two
// random values in one expression, which C++ leaves unspecified; a set bit
// means right to left.  The reference's GPU build (nvcc) evaluates all three
// left to right (RNG_ORDER_GPU, measured against its own megakernel on the
// GPU: every other order disagrees with it on 15-65% of the samples); its
// host build (g++) evaluates all three right to left.
constexpr int RNG_PAIR = 1;       // make_float2(get1D(), get1D())          samplers.cuh:37-40
constexpr int RNG_SUN = 2;        // make_float3(get2D()*2-1, get1D()*2-1)  integrator.cuh:155
constexpr int RNG_BSDF = 4;       // sampleF(wo, get2D(), get2D())          integrator.cuh:382
constexpr int RNG_ORDER_GPU = 0;
constexpr int RNG_ORDER_HOST = RNG_PAIR | RNG_SUN | RNG_BSDF;

struct Sampler {
    uint32_t seed;
    __device__ __forceinline__ void init(int px, int py, int width, int index) {
        seed = (uint32_t)(px + py * width);
        float f = (index == 0) ? 1.0f : (float)index;
        seed = (uint32_t)__fmul_rn((float)seed, f);
    }
    __device__ __forceinline__ float get1D() {
        seed = pcg_hash(seed);
        return __fmul_rn((float)seed, 1.0f / 4294967295.0f);
    }
    // make_float2(get1D(), get1D()) (samplers.cuh:37-40) in the argument
    // evaluation order of bit RNG_PAIR of `order` (0: left to right)
    __device__ __forceinline__ float2 get2D(int order) {
        float a = get1D(), b = get1D();
        return (order & RNG_PAIR) == 0 ? make_float2(a, b) : make_float2(b, a);
    }
};

}  // namespace kpt
