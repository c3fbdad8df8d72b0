// kpt_path.cu -- path tracing and ray tracing kernels (compiled with
// -use_fast_math, the reference GPU build's arithmetic, except for the
// IEEE-exact traversal and camera rays in kpt_trace.cuh / kpt_device.cuh).
//
// k_path follows the megakernel computePathTraceSamplesMegaKernel
// (shaders/kernels.cu:385-451) and Integrator::Li (shaders/integrator.cuh:
// 241-402).  Differences in structure, none of which changes a sample:
//   * one launch computes many samples per pixel (sample index = the
//     reference's frame index) and accumulates them in sample order, so the
//     accumulation sum equals the reference's frame-by-frame sum;
//   * the Nishita radiance towards the sun, which sampleLdSun recomputes on
//     every call (integrator.cuh:169), is a per-frame constant computed once
//     by k_sky_constants with the same function;
//   * each instance carries its shading model matrix, which the reference
//     recomputes per hit and per light sample as the inverse of the mesh
//     inverse (interaction.cu:20, light.cu:36);
//   * work is handed out per pixel from a global counter (persistent
//     threads), so warps refill as their paths finish.
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
    int material, light, inst, tri;
    bool backface;
};

__device__ __forceinline__ int light_of(const SceneView& s, const InstRec& ir, const TriShade& sh, int tri) {
    if (ir.light_first < 0) return -1;
    if (ir.light_all) return ir.light_first + tri;
    return sh.emissive_rank >= 0 ? ir.light_first + sh.emissive_rank : -1;
}

// Intersection::getSurfaceInteraction (interaction.cu:11-38).
__device__ __forceinline__ Surf surface_at(const SceneView& s, const Hit& h, const XRay& r) {
    Surf si;
    const InstRec& ir = s.inst[h.inst];
    const MeshRec& m = s.meshes[ir.mesh];
    const TriShade sh = s.shade[m.shade_base + h.tri];
    float4 model[3] = {ir.model[0], ir.model[1], ir.model[2]};
    si.wo = -r.d;
    si.pos = r.o + (h.t * r.d);
    si.ng = normalize(row3(model, make_float3(sh.gnx, sh.gny, sh.gnz), 0.0f));
    float b0 = 1.0f - h.u - h.v;
    si.uv = make_float2(b0 * sh.uv0.x + h.u * sh.uv1.x + h.v * sh.uv2.x,
                        b0 * sh.uv0.y + h.u * sh.uv1.y + h.v * sh.uv2.y);
    si.backface = false;
    if (!(dot(si.ng, si.wo) > 0.0f)) {
        si.ng = si.ng * -1.0f;
        si.backface = true;
    }
    si.material = ir.material >= 0 ? ir.material : sh.material;
    si.light = light_of(s, ir, sh, h.tri);
    si.inst = h.inst;
    si.tri = h.tri;
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

struct SampleOut {
    float3 L, albedo;
    int first_inst, first_tri;
    float first_t;
};

// Integrator::Li (integrator.cuh:241-402) with LeSun (:135-143),
// sampleLdSun (:147-186), sampleLd (:188-220) and russianRoulette
// (maths/sampling.cuh:19-31).
__device__ SampleOut path_sample(const FrameParams& F, XRay ray, Sampler& S, TraceStats& st, int* stack) {
    const SceneView& s = F.scene;
    const SkyParams& P = F.sky;
    const int order = F.rng_order;
    const float3 observer = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const float3 sun_rad = *F.sun_radiance;
    float3 L = make_float3(0.0f, 0.0f, 0.0f), beta = make_float3(1.0f, 1.0f, 1.0f);
    int depth = 0;
    float p_b = 1.0f;
    float3 prev_pos = make_float3(0.0f, 0.0f, 0.0f);
    bool any_non_specular = false;
    SampleOut out;
    out.albedo = make_float3(0.0f, 0.0f, 0.0f);
    out.first_inst = -1;
    out.first_tri = -1;
    out.first_t = __int_as_float(0x7f800000);
    const int nl = s.nlights;
    while (nonzero(beta)) {
        S.seed = S.seed + (uint32_t)depth;
        const bool first = depth == 0;
        Hit h = trace_closest(s, ray, 0.0f, __int_as_float(0x7f800000), st, stack);
        if (h.inst < 0) {
            float3 sk = nishita(P, observer, ray.d);
            if (first) {
                float sim = dot(ray.d, P.sun_dir);
                float sr = P.sun_emission * 6.0e5f;
                float ls = sr * powf(1.0f / sr, (float)(!(sim > P.cos_half_sun)));
                sk = sk * ls;
                out.albedo = sk;
            }
            L = L + sk * beta;
            break;
        }
        if (first) {
            out.first_inst = h.inst;
            out.first_tri = h.tri;
            out.first_t = h.t;
        }
        Surf si = surface_at(s, h, ray);
        float3 Le = make_float3(0.0f, 0.0f, 0.0f);
        if (si.light >= 0) Le = emission_of(s, si.material, si.uv);
        if (nonzero(Le)) {
            float w_l = 1.0f;
            if (si.light >= 0 && !first) {
                const LightRec& lt = s.lights[si.light];
                float pmf = 1.0f / (float)nl;
                float dist = length(si.pos - prev_pos);
                float cosl = AbsDot(normalize(si.pos - prev_pos), si.ng);
                float lpdf = pmf * ((1.0f / lt.area) / (cosl / Sqr(dist)));
                w_l = Sqr(p_b) / (Sqr(p_b) + Sqr(lpdf));
            }
            L = L + Le * w_l * beta;
        }
        Bsdf bsdf = bsdf_at(s, si);
        if (first) {
            out.albedo = nonzero(Le) ? Le : bsdf.albedo;
            bsdf.albedo = make_float3(1.0f, 1.0f, 1.0f);
        }
        if (any_non_specular && bsdf.alpha < 0.3f) bsdf.alpha = clampf(2.0f * bsdf.alpha, 0.1f, 0.3f);
        const float3 wo = -ray.d;
        if (!(bsdf.alpha < 0.001f)) {
            if (S.get1D() < 0.5f) {
                // sampleLdSun: jittered point on the sun disc at 1 AU
                float3 Ld = make_float3(0.0f, 0.0f, 0.0f);
                const float dsun = 149.597e9f;
                float3 sun_pos = P.sun_dir * dsun;
                float3 off;
                if (order == 0) {
                    float2 a = S.get2D(0);
                    float b = S.get1D();
                    off = make_float3(a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f);
                } else {
                    float b = S.get1D();
                    float2 a = S.get2D(1);
                    off = make_float3(a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f);
                }
                float3 target = sun_pos + (off * P.sun_radius_m);
                float3 fcos = bsdf.f(wo, P.sun_dir) * fmaxf(0.0f, dot(P.sun_dir, (si.backface ? -1.0f : 1.0f) * si.ng));
                if (nonzero(fcos) && nonzero(sun_rad) && unoccluded(F, si, target, st, stack)) {
                    float area = PI_F * Sqr(P.sun_radius_m);
                    float3 sn = normalize(target - sun_pos), wi = normalize(target - si.pos);
                    float th = AbsDot(sn, -wi);
                    float pdf = (1.0f / area) / (th / Sqr(dsun));
                    Ld = (fcos * sun_rad * 6.0e5f) / pdf;
                }
                L = L + Ld * beta / 0.5f;
            } else {
                // sampleLd: uniform light pick, uniform point on the triangle
                float3 Ld = make_float3(0.0f, 0.0f, 0.0f);
                float X = S.get1D();
                if (nl >= 1) {
                    int li = min((int)(X * (float)nl), nl - 1);
                    const LightRec& lt = s.lights[li];
                    float prob = 1.0f / (float)nl;
                    float2 u = S.get2D(order);
                    const InstRec& lir = s.inst[lt.inst];
                    float4 model[3] = {lir.model[0], lir.model[1], lir.model[2]};
                    float bx, by;
                    if (u.x < u.y) { bx = u.x / 2.0f; by = u.y - bx; }
                    else { by = u.y / 2.0f; bx = u.x - by; }
                    float bz = 1.0f - bx - by;
                    float2 luv = make_float2(bx * lt.uv0.x + by * lt.uv1.x + bz * lt.uv2.x,
                                             bx * lt.uv0.y + by * lt.uv1.y + bz * lt.uv2.y);
                    float3 p = (lt.p0 * bx) + (lt.p1 * by) + (lt.p2 * bz);
                    p = row3(model, p, 1.0f);
                    float3 gn = row3(model, lt.gn, 0.0f);
                    float pdf = 1.0f / lt.tri_area;
                    pdf *= Sqr(length(p - si.pos));
                    pdf /= AbsDot(normalize(p - si.pos), gn);
                    float3 wi = normalize(p - si.pos);
                    float3 Lem = emission_of(s, lt.material, luv);
                    if (!(pdf <= 0.0f || !nonzero(Lem))) {
                        float3 fcos = bsdf.f(wo, wi) * fmaxf(0.0f, dot(wi, (si.backface ? -1.0f : 1.0f) * si.ng));
                        if (nonzero(fcos) && unoccluded(F, si, p, st, stack)) {
                            float p_l = prob * pdf;
                            float pb = bsdf.pdf(wo, wi);
                            float w_l = Sqr(p_l) / (Sqr(p_l) + Sqr(pb));
                            Ld = (Lem * fcos * w_l) / p_l;
                        }
                    }
                }
                L = L + Ld * beta / (1.0f - 0.5f);
            }
        }
        if (depth++ == F.max_depth) break;
        float2 u, X;
        if (order == 0) { u = S.get2D(0); X = S.get2D(0); }
        else { X = S.get2D(1); u = S.get2D(1); }
        BsdfSample bs = bsdf.sample(wo, u, X);
        if (bs.scatter == SC_ABSORBED || !nonzero(bs.f)) break;
        beta = beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
        p_b = bsdf.pdf(wo, bs.wi);
        any_non_specular = true;
        prev_pos = si.pos;
        float3 o = (bs.scatter & SC_TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
        ray = make_xray(o, bs.wi);
        float mx = fmaxf(beta.x, fmaxf(beta.y, beta.z));
        if (mx < 1.0f && depth > 1) {
            float q = fmaxf(0.0f, 1.0f - mx);
            if (S.get1D() < q) break;
            beta = beta / (1.0f - q);
        }
    }
    // RGBSpectrum::clampOutput (color.cuh:295-302)
    if (isnan(L.x) || isnan(L.y) || isnan(L.z) || isinf(L.x) || isinf(L.y) || isinf(L.z))
        L = make_float3(0.0f, 0.0f, 0.0f);
    else
        L = make_float3(clampf(L.x, 0.0f, 1.0e8f), clampf(L.y, 0.0f, 1.0e8f), clampf(L.z, 0.0f, 1.0e8f));
    out.L = L;
    return out;
}

__device__ __forceinline__ void flush_stats(const TraceStats& st, unsigned long long* counters) {
    if (!counters) return;
    unsigned v[4] = {st.box_tests, st.tri_tests, st.inst_xforms, st.overflow};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned long long x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(counters + k, x);
    }
}

// One pixel per work item; all of its samples in sample order.
__global__ void __launch_bounds__(PATH_BLOCK) k_path(FrameParams F) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    const int npix = F.W * F.H;
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(F.work_counter, PATH_BLOCK);
        __syncthreads();
        int base = s_item;
        __syncthreads();
        if (base >= npix) break;
        int p = base + threadIdx.x;
        if (p < npix) {
            int x = p % F.W, y = p / F.W;
            float4 acc = F.acc ? F.acc[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            SampleOut so;
            for (int k = 0; k < F.nsamples; ++k) {
                Sampler S;
                S.init(x, y, F.W, F.sample0 + k);
                S.get1D();   // BoxFilter::sample, result discarded (kernels.cu:397-402)
                S.get1D();
                so = path_sample(F, camera_ray(F, x, y), S, st, stack);
                acc.x += so.L.x;
                acc.y += so.L.y;
                acc.z += so.L.z;
                if (F.sample_out) F.sample_out[(size_t)k * npix + p] = make_float4(so.L.x, so.L.y, so.L.z, 0.0f);
            }
            if (F.acc) F.acc[p] = make_float4(acc.x, acc.y, acc.z, 1.0f);
            if (F.albedo) F.albedo[p] = make_float4(so.albedo.x, so.albedo.y, so.albedo.z, 0.0f);
            if (F.first_hit) F.first_hit[p] = make_int4(so.first_inst, so.first_tri, __float_as_int(so.first_t), 0);
        }
    }
    flush_stats(st, F.counters);
}

// Nishita radiance towards the sun: a per-frame constant.
__global__ void k_sky_constants(FrameParams F, float3* sun_radiance) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const SkyParams& P = F.sky;
        *sun_radiance = nishita(P, make_float3(0.0f, P.earth_r + 1.0f, 0.0f), P.sun_dir);
    }
}

// Sky radiance for a list of directions (tests and tools).
__global__ void k_sky(SkyParams P, int n, const float3* dirs, float3* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = nishita(P, make_float3(0.0f, P.earth_r + 1.0f, 0.0f), dirs[i]);
}

// Closest hit for a batch of rays: persistent, one ray per thread per step.
__global__ void __launch_bounds__(TRACE_BLOCK) k_trace(SceneView s, int n, const float3* o, const float3* d,
                                                       float tmin, float tmax, int* inst, int* tri, float* t,
                                                       float2* uv, unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        XRay r = make_xray(o[i], d[i]);
        Hit h = trace_closest(s, r, tmin, tmax, st, stack);
        inst[i] = h.inst;
        tri[i] = h.tri;
        t[i] = h.t;
        if (uv) uv[i] = make_float2(h.u, h.v);
    }
    flush_stats(st, counters);
}

__global__ void __launch_bounds__(TRACE_BLOCK) k_occluded(SceneView s, int n, const float3* o, const float3* d,
                                                          float tmin, const float* tmax, uint8_t* out,
                                                          unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = trace_any(s, make_xray(o[i], d[i]), tmin, tmax[i], st, stack) ? 1 : 0;
    flush_stats(st, counters);
}

// Closest hit plus `nbounces` diffuse bounces per ray: cosine-weighted about
// the geometric normal facing the incoming ray, origin offset 1e-3 along it,
// two PCG draws seeded with 4 * ray index + bounce.  IEEE arithmetic so that
// every bounce is bit-identical to the oracle's.  Writes (nbounces+1) x n.
__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_bounces(SceneView s, int n, const float3* o, const float3* d,
                                                               int nbounces, int* inst, int* tri, float* t,
                                                               unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        XRay r = make_xray(o[i], d[i]);
        for (int b = 0; b <= nbounces; ++b) {
            size_t k = (size_t)b * n + i;
            Hit h = trace_closest(s, r, 0.0f, __int_as_float(0x7f800000), st, stack);
            inst[k] = h.inst;
            tri[k] = h.tri;
            t[k] = h.t;
            if (h.inst < 0) {
                for (int bb = b + 1; bb <= nbounces; ++bb) {
                    size_t kk = (size_t)bb * n + i;
                    inst[kk] = -1;
                    tri[kk] = -1;
                    t[kk] = __int_as_float(0x7f800000);
                }
                break;
            }
            if (b == nbounces) break;
            const InstRec& ir = s.inst[h.inst];
            const TriShade sh = s.shade[s.meshes[ir.mesh].shade_base + h.tri];
            float3 gn = make_float3(sh.gnx, sh.gny, sh.gnz);
            float3 nn = xnormalize(make_float3(xrow(ir.model[0], gn, 0.0f), xrow(ir.model[1], gn, 0.0f),
                                               xrow(ir.model[2], gn, 0.0f)));
            if (xdot(nn, r.d) > 0.0f) nn = make_float3(-nn.x, -nn.y, -nn.z);
            float3 p = make_float3(xa(r.o.x, xm(h.t, r.d.x)), xa(r.o.y, xm(h.t, r.d.y)), xa(r.o.z, xm(h.t, r.d.z)));
            // Malley's method: rejection-sampled unit-disk point lifted to the hemisphere
            Sampler S;
            S.seed = (uint32_t)i * 4u + (uint32_t)b;
            float lx = 0.0f, ly = 0.0f, r2 = 0.0f;
            for (int q = 0; q < 64; ++q) {
                float u0 = S.get1D(), u1 = S.get1D();
                float a = xs(xm(2.0f, u0), 1.0f), c = xs(xm(2.0f, u1), 1.0f);
                float m = xa(xm(a, a), xm(c, c));
                if (m < 1.0f) { lx = a; ly = c; r2 = m; break; }
            }
            float3 l = make_float3(lx, ly, __fsqrt_rn(xs(1.0f, r2)));
            float3 w = onb_apply_exact(nn, l);
            r = make_xray(make_float3(xa(p.x, xm(nn.x, HIT_EPS)), xa(p.y, xm(nn.y, HIT_EPS)), xa(p.z, xm(nn.z, HIT_EPS))), w);
        }
    }
    flush_stats(st, counters);
}

}  // namespace kpt
