// kpt_pathfn.cuh -- device functions shared by the path kernels
// (kpt_path.cu) and the adjoint replay (kpt_adjoint.cu): camera rays, the
// surface interaction, materials, emission, the sun disc and warp-level
// helpers.  Fast maths except where stated.
#pragma once
#include "kpt_internal.h"
#include "kpt_shade.cuh"
#include "kpt_trace.cuh"

namespace kpt {

// Camera::generateRay (camera.cuh:16-25) in IEEE arithmetic.
__device__ __forceinline__ XRay camera_ray(const FrameParams& F, int x, int y) {
    float ux = __fdiv_rn(xa((float)x, 0.5f), (float)F.W);
    float uy = __fdiv_rn(xa((float)y, 0.5f), (float)F.H);
    float nx = xs(xm(2.0f, ux), 1.0f), ny = xs(xm(2.0f, uy), 1.0f);
    float3 ndc = make_float3(nx, ny, 1.0f);
    float tcx = xrow(F.inv_proj[0], ndc, 1.0f), tcy = xrow(F.inv_proj[1], ndc, 1.0f);
    float tcz = xrow(F.inv_proj[2], ndc, 1.0f), tcw = xrow(F.inv_proj[3], ndc, 1.0f);
    float3 v = xnormalize(make_float3(__fdiv_rn(tcx, tcw), __fdiv_rn(tcy, tcw), __fdiv_rn(tcz, tcw)));
    float3 w = make_float3(xrow(F.inv_view[0], v, 0.0f), xrow(F.inv_view[1], v, 0.0f), xrow(F.inv_view[2], v, 0.0f));
    return make_xray(F.cam_pos, xnormalize(w));
}

struct Surf {
    float3 pos, ng, wo;
    float2 uv;
    int material, light;
    bool backface;
};

__device__ __forceinline__ int light_of(const InstRec& ir, const TriShade& sh, int tri) {
    if (ir.light_first < 0) return -1;
    if (ir.light_all) return ir.light_first + tri;
    return sh.emissive_rank >= 0 ? ir.light_first + sh.emissive_rank : -1;
}

// Intersection::getSurfaceInteraction (interaction.cu:11-38).
__device__ __forceinline__ Surf surface_at(const SceneView& s, int inst, int tri, float t, float u, float v,
                                           float3 ro, float3 rd) {
    Surf si;
    const InstRec& ir = s.inst[inst];
    const MeshRec& m = s.meshes[ir.mesh];
    const TriShade sh = s.shade[m.shade_base + tri];
    float4 model[3] = {ir.model[0], ir.model[1], ir.model[2]};
    si.wo = -rd;
    si.pos = ro + (t * rd);
    si.ng = normalize(row3(model, make_float3(sh.gnx, sh.gny, sh.gnz), 0.0f));
    float b0 = 1.0f - u - v;
    si.uv = make_float2(b0 * sh.uv0.x + u * sh.uv1.x + v * sh.uv2.x, b0 * sh.uv0.y + u * sh.uv1.y + v * sh.uv2.y);
    si.backface = false;
    if (!(dot(si.ng, si.wo) > 0.0f)) {
        si.ng = si.ng * -1.0f;
        si.backface = true;
    }
    si.material = ir.material >= 0 ? ir.material : sh.material;
    si.light = light_of(ir, sh, tri);
    return si;
}

__device__ __forceinline__ float3 emission_of(const SceneView& s, int mat, float2 uv) {  // light.cu:21-33
    const MatRec& m = s.materials[mat];
    float3 em = make_float3(m.emission[0], m.emission[1], m.emission[2]) * m.emission_scale;
    if (m.emission_tex >= 0) {
        float3 t = texture_eval(s, m.emission_tex, uv);
        em = em * make_float3(powf(t.x, 2.2f), powf(t.y, 2.2f), powf(t.z, 2.2f));
    }
    return em;
}

// Material::getBSDF (material.cu:17-70).
__device__ __forceinline__ Bsdf bsdf_at(const SceneView& s, const Surf& si) {
    const MatRec& m = s.materials[si.material];
    float3 alb = make_float3(m.albedo[0], m.albedo[1], m.albedo[2]);
    float rough = m.roughness, metal = m.metallic, trans = m.transmission;
    float3 n = si.ng;
    if (m.albedo_tex >= 0) {
        float3 t = texture_eval(s, m.albedo_tex, si.uv);
        alb = alb * make_float3(srgb_decode(t.x), srgb_decode(t.y), srgb_decode(t.z));
    }
    if (m.orm_tex >= 0) {
        float3 t = texture_eval(s, m.orm_tex, si.uv);
        rough *= t.y;
        metal *= t.z;
    }
    if (m.transmission_tex >= 0) trans *= texture_eval(s, m.transmission_tex, si.uv).x;
    if (m.normal_tex >= 0) {
        float3 t = texture_eval(s, m.normal_tex, si.uv);
        float3 mn = (t * 2.0f) - 1.0f;
        mn.x *= m.normal_scale;
        mn.y *= m.normal_scale;
        float3 sn = mul(onb_frisvad(n), normalize(mn));
        n = (dot(si.wo, sn) > 0.0f) ? sn : n;
    }
    Bsdf b;
    b.basis = onb_frisvad(n);
    b.albedo = alb;
    b.alpha = Sqr(rough);
    b.metallic = metal;
    b.transmission = trans;
    b.ior = m.ior;
    b.backface = si.backface;
    return b;
}

__device__ __forceinline__ bool unoccluded(const FrameParams& F, const Surf& si, float3 target,
                                           TraceStats& st, int* stack) {  // integrator.cuh:124-131
    float3 o = si.backface ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
    float3 d = normalize(target - o);
    float tmax = length(target - o) - 0.11f;
    return !trace_any(F.scene, make_xray(o, d), 0.0f, tmax, st, stack);
}

// LeSun (integrator.cuh:135-143): the sun disc at the first miss.
__device__ __forceinline__ float le_sun(const SkyParams& P, float3 d) {
    float sim = dot(d, P.sun_dir);
    float sr = P.sun_emission * 6.0e5f;
    return sr * powf(1.0f / sr, (float)(!(sim > P.cos_half_sun)));
}

__device__ __forceinline__ void flush_stats(const TraceStats& st, unsigned long long* counters) {
    if (!counters) return;
    unsigned v[4] = {st.box_tests, st.tri_tests, st.inst_xforms, st.overflow};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned long long x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(counters + k, x);
    }
}

// Appends the lanes of a (possibly divergent) warp that reach this call to a
// list with one atomic; returns each lane's slot.
__device__ __forceinline__ int group_append(int* counter) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
    return g.shfl(base, 0) + (int)g.thread_rank();
}

// Appends `want` lanes of the warp to a list: returns each lane's slot.
__device__ __forceinline__ int warp_append(bool want, int* counter) {
    unsigned mask = __ballot_sync(0xffffffffu, want);
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(mask) - 1 && mask) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, mask ? __ffs(mask) - 1 : 0);
    return base + __popc(mask & ((1u << lane) - 1u));
}

}  // namespace kpt
