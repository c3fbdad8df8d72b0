// kpt_path.cu -- path tracing and ray tracing kernels (compiled with
// -use_fast_math, the reference GPU build's arithmetic, except for the
// IEEE-exact traversal, camera rays and sky geometry).
//
// One frame of the plain method follows the megakernel
// computePathTraceSamplesMegaKernel (shaders/kernels.cu:385-451) and
// Integrator::Li (shaders/integrator.cuh:241-402), reorganised for the GPU
// without changing any sample:
//   * k_primary traces each pixel's camera ray once per frame.  The camera
//     ray is the same for every sample (the reference computes a filter
//     jitter and then discards it, kernels.cu:397-402), so its closest hit,
//     the visible-surface albedo and -- for a miss -- the sky radiance are
//     per-pixel quantities;
//   * k_primary_sky evaluates the sky once per missing pixel, over a
//     compacted list (every lane runs the same 16x8-step march);
//   * k_paths is persistent: each thread walks work items (sample, hit
//     pixel) round-robin and advances one bounce per loop iteration, taking a
//     new item as soon as its path ends, so lanes stay busy while paths of
//     different lengths finish;
//   * a path whose ray leaves the scene does not march the sky inline: it
//     queues (item, direction, throughput) and k_sky_queue evaluates the queue
//     coherently, adding sky * throughput to the sample -- a miss is always the
//     last event of a path (integrator.cuh:315-325), so the sum is unchanged;
//   * the Nishita radiance towards the sun, which sampleLdSun recomputes on
//     every call (integrator.cuh:169), is a per-frame constant (k_sky_constants);
//   * each instance carries its shading model matrix, which the reference
//     recomputes per hit and per light sample (interaction.cu:20, light.cu:36).
// k_accumulate (kpt_post.cu) then clamps each sample and adds them per pixel
// in sample order, as the reference's frame-by-frame accumulation does.
#include <cooperative_groups.h>

#include "kpt_internal.h"
#include "kpt_shade.cuh"
#include "kpt_trace.cuh"

namespace cg = cooperative_groups;

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

// Appends `want` lanes of the warp to a list: returns each lane's slot.
__device__ __forceinline__ int warp_append(bool want, int* counter) {
    unsigned mask = __ballot_sync(0xffffffffu, want);
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(mask) - 1 && mask) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, mask ? __ffs(mask) - 1 : 0);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// camera rays: one per pixel per frame

__global__ void __launch_bounds__(PATH_BLOCK) k_primary(FrameParams F) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    const int npix = F.W * F.H;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    Hit h;
    h.inst = -1;
    XRay r;
    if (p < npix) {
        r = camera_ray(F, p % F.W, p / F.W);
        h = trace_closest(F.scene, r, 0.0f, __int_as_float(0x7f800000), st, stack);
    }
    const bool hit = p < npix && h.inst >= 0;
    const bool miss = p < npix && h.inst < 0;
    int j = warp_append(hit, F.counts);
    int m = warp_append(miss, F.counts + 1);
    if (hit) {
        PrimaryRec pr;
        pr.t = h.t;
        pr.u = h.u;
        pr.v = h.v;
        pr.inst = h.inst;
        pr.tri = h.tri;
        pr.pad0 = pr.pad1 = pr.pad2 = 0;
        F.primary[p] = pr;
        F.hit_list[j] = p;
        F.hit_index[p] = j;
        // visible-surface albedo (integrator.cuh:352-357): emission, else the BSDF albedo
        Surf si = surface_at(F.scene, h.inst, h.tri, h.t, h.u, h.v, r.o, r.d);
        float3 Le = si.light >= 0 ? emission_of(F.scene, si.material, si.uv) : make_float3(0.0f, 0.0f, 0.0f);
        float3 alb = nonzero(Le) ? Le : bsdf_at(F.scene, si).albedo;
        if (F.albedo) F.albedo[p] = make_float4(alb.x, alb.y, alb.z, 0.0f);
        if (F.first_hit) F.first_hit[p] = make_int4(h.inst, h.tri, __float_as_int(h.t), 0);
    } else if (miss) {
        F.miss_list[m] = p;
        F.hit_index[p] = -1;
        if (F.first_hit) F.first_hit[p] = make_int4(-1, -1, 0x7f800000, 0);
    }
    flush_stats(st, F.counters ? F.counters + 4 : nullptr);
}

// sky (times LeSun) of every pixel whose camera ray misses
__global__ void __launch_bounds__(PATH_BLOCK) k_primary_sky(FrameParams F) {
    const int n = F.counts[1];
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int p = F.miss_list[i];
        XRay r = camera_ray(F, p % F.W, p / F.W);
        float3 sk = nishita(P, obs, r.d) * le_sun(P, r.d);
        float4 v = make_float4(sk.x, sk.y, sk.z, 0.0f);
        F.pixel_sky[p] = v;
        if (F.albedo) F.albedo[p] = v;
    }
}

// ---------------------------------------------------------------------------
// paths

struct PathState {
    float3 o, d, beta, L, prev_pos;
    float p_b;
    uint32_t seed;
    int depth, item, pixel;
    bool any_ns;
};

// One bounce of Integrator::Li (integrator.cuh:266-399) with LeSun, sampleLdSun
// (:147-186), sampleLd (:188-220) and russianRoulette (maths/sampling.cuh:19-31).
// Returns false when the path has ended.
__device__ __forceinline__ bool bounce(const FrameParams& F, PathState& ps, TraceStats& st, int* stack) {
    const SceneView& s = F.scene;
    const SkyParams& P = F.sky;
    const int order = F.rng_order;
    const int nl = s.nlights;
    Sampler S;
    S.seed = ps.seed + (uint32_t)ps.depth;
    const bool first = ps.depth == 0;
    int inst, tri;
    float t, u, v;
    if (first) {
        const PrimaryRec pr = F.primary[ps.pixel];
        inst = pr.inst; tri = pr.tri; t = pr.t; u = pr.u; v = pr.v;
    } else {
        Hit h = trace_closest(s, make_xray(ps.o, ps.d), 0.0f, __int_as_float(0x7f800000), st, stack);
        inst = h.inst; tri = h.tri; t = h.t; u = h.u; v = h.v;
    }
    if (inst < 0) {
        // the sky is evaluated by k_sky_queue; the path ends here.  The lanes
        // that missed together take consecutive queue slots with one atomic.
        cg::coalesced_group g = cg::coalesced_threads();
        int q0 = 0;
        if (g.thread_rank() == 0) q0 = atomicAdd(F.counts + 2, (int)g.size());
        int q = g.shfl(q0, 0) + (int)g.thread_rank();
        F.sky_queue[2 * (size_t)q] = make_float4(__int_as_float(ps.item), ps.d.x, ps.d.y, ps.d.z);
        F.sky_queue[2 * (size_t)q + 1] = make_float4(ps.beta.x, ps.beta.y, ps.beta.z, 0.0f);
        return false;
    }
    Surf si = surface_at(s, inst, tri, t, u, v, ps.o, ps.d);
    float3 Le = make_float3(0.0f, 0.0f, 0.0f);
    if (si.light >= 0) Le = emission_of(s, si.material, si.uv);
    if (nonzero(Le)) {
        float w_l = 1.0f;
        if (si.light >= 0 && !first) {
            const LightRec& lt = s.lights[si.light];
            float pmf = 1.0f / (float)nl;
            float dist = length(si.pos - ps.prev_pos);
            float cosl = AbsDot(normalize(si.pos - ps.prev_pos), si.ng);
            float lpdf = pmf * ((1.0f / lt.area) / (cosl / Sqr(dist)));
            w_l = Sqr(ps.p_b) / (Sqr(ps.p_b) + Sqr(lpdf));
        }
        ps.L = ps.L + Le * w_l * ps.beta;
    }
    Bsdf bsdf = bsdf_at(s, si);
    if (first) bsdf.albedo = make_float3(1.0f, 1.0f, 1.0f);   // demodulate (bsdf.cuh:286-288)
    if (ps.any_ns && bsdf.alpha < 0.3f) bsdf.alpha = clampf(2.0f * bsdf.alpha, 0.1f, 0.3f);
    const float3 wo = -ps.d;
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
            const float3 sun_rad = *F.sun_radiance;
            if (nonzero(fcos) && nonzero(sun_rad) && unoccluded(F, si, target, st, stack)) {
                float area = PI_F * Sqr(P.sun_radius_m);
                float3 sn = normalize(target - sun_pos), wi = normalize(target - si.pos);
                float th = AbsDot(sn, -wi);
                float pdf = (1.0f / area) / (th / Sqr(dsun));
                Ld = (fcos * sun_rad * 6.0e5f) / pdf;
            }
            ps.L = ps.L + Ld * ps.beta / 0.5f;
        } else {
            // sampleLd: uniform light pick, uniform point on the triangle
            float3 Ld = make_float3(0.0f, 0.0f, 0.0f);
            float X = S.get1D();
            if (nl >= 1) {
                int li = min((int)(X * (float)nl), nl - 1);
                const LightRec& lt = s.lights[li];
                float prob = 1.0f / (float)nl;
                float2 uu = S.get2D(order);
                const InstRec& lir = s.inst[lt.inst];
                float4 model[3] = {lir.model[0], lir.model[1], lir.model[2]};
                float bx, by;
                if (uu.x < uu.y) { bx = uu.x / 2.0f; by = uu.y - bx; }
                else { by = uu.y / 2.0f; bx = uu.x - by; }
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
            ps.L = ps.L + Ld * ps.beta / (1.0f - 0.5f);
        }
    }
    if (ps.depth++ == F.max_depth) return false;
    float2 uu, X;
    if (order == 0) { uu = S.get2D(0); X = S.get2D(0); }
    else { X = S.get2D(1); uu = S.get2D(1); }
    BsdfSample bs = bsdf.sample(wo, uu, X);
    if (bs.scatter == SC_ABSORBED || !nonzero(bs.f)) return false;
    ps.beta = ps.beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
    ps.p_b = bsdf.pdf(wo, bs.wi);
    ps.any_ns = true;
    ps.prev_pos = si.pos;
    ps.o = (bs.scatter & SC_TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
    ps.d = bs.wi;
    float mx = fmaxf(ps.beta.x, fmaxf(ps.beta.y, ps.beta.z));
    if (mx < 1.0f && ps.depth > 1) {
        float q = fmaxf(0.0f, 1.0f - mx);
        if (S.get1D() < q) {
            ps.seed = S.seed;
            return false;
        }
        ps.beta = ps.beta / (1.0f - q);
    }
    ps.seed = S.seed;
    return nonzero(ps.beta);   // while (throughput) (integrator.cuh:266)
}

__global__ void __launch_bounds__(PATH_BLOCK) k_paths(FrameParams F) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    const int nhit = F.counts[0];
    const long long total = (long long)nhit * F.nsamples;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long next = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    PathState ps;
    ps.item = -1;
    for (;;) {
        if (ps.item < 0) {
            if (next >= total) break;
            const int item = (int)next;
            next += stride;
            const int k = item / nhit;
            const int p = F.hit_list[item - k * nhit];
            const int x = p % F.W, y = p / F.W;
            Sampler S;
            S.init(x, y, F.W, F.sample0 + k);
            S.get1D();   // BoxFilter::sample, result discarded (kernels.cu:397-402)
            S.get1D();
            XRay r = camera_ray(F, x, y);
            ps.o = r.o;
            ps.d = r.d;
            ps.beta = make_float3(1.0f, 1.0f, 1.0f);
            ps.L = make_float3(0.0f, 0.0f, 0.0f);
            ps.prev_pos = make_float3(0.0f, 0.0f, 0.0f);
            ps.p_b = 1.0f;
            ps.seed = S.seed;
            ps.depth = 0;
            ps.item = item;
            ps.pixel = p;
            ps.any_ns = false;
        }
        if (!bounce(F, ps, st, stack)) {
            F.radiance[ps.item] = make_float4(ps.L.x, ps.L.y, ps.L.z, 0.0f);
            ps.item = -1;
        }
    }
    flush_stats(st, F.counters);
}

// sky * throughput of every path that left the scene, added to its sample
__global__ void __launch_bounds__(PATH_BLOCK) k_sky_queue(FrameParams F) {
    const int n = F.counts[2];
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = F.sky_queue[2 * (size_t)i], b = F.sky_queue[2 * (size_t)i + 1];
        int item = __float_as_int(a.x);
        float3 sk = nishita(P, obs, make_float3(a.y, a.z, a.w));
        float4 L = F.radiance[item];
        F.radiance[item] = make_float4(L.x + sk.x * b.x, L.y + sk.y * b.y, L.z + sk.z * b.z, 0.0f);
    }
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

// ---------------------------------------------------------------------------
// ray queries

// Closest hit for a batch of rays, one ray per thread per step.
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
// the geometric normal facing the incoming ray (Malley's method: a uniform
// unit-disk point, rejection-sampled from pairs of PCG draws seeded with
// 4 * ray index + bounce, lifted to the hemisphere and rotated by the Frisvad
// basis), origin offset 1e-3 along the normal.  IEEE arithmetic throughout,
// so every bounce is bit-identical to the oracle's.  Writes (nbounces+1) x n.
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
