// kpt_path.cu -- path tracing and ray tracing kernels (compiled with
// -use_fast_math, the reference GPU build's arithmetic, except for the
// IEEE-exact traversal, camera rays and sky geometry).
//
// One frame of the plain method follows the megakernel
// computePathTraceSamplesMegaKernel (shaders/kernels.cu:385-451) and
// Integrator::Li (shaders/integrator.cuh:241-402), reorganised for the GPU
// as a wavefront without changing any sample:
//   * k_primary traces each pixel's camera ray once per frame.  The camera
//     ray is the same for every sample (the reference computes a filter
//     jitter and then discards it, kernels.cu:397-402), so its closest hit,
//     the visible-surface albedo and -- for a miss -- the sky radiance are
//     per-pixel quantities;
//   * k_primary_sky evaluates the sky once per missing pixel, over a
//     compacted list (every lane runs the same 16x8-step march);
//   * the work items (sample, hit pixel) then advance as a wave, one path
//     vertex per level: k_shade shades every path entering the level and
//     writes its light sample's shadow ray and its continuation to compacted
//     queues, k_shadow traces the shadow rays, k_extend the continuations.
//     The ray kernels hold no shading state, so they run at full occupancy,
//     and every lane of a warp runs the same kind of query;
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
#include "kpt_internal.h"
#include "kpt_pathfn.cuh"

namespace kpt {

// ---------------------------------------------------------------------------
// camera rays: one per pixel per frame

// A block covers a 2 TILE_W x 2 TILE_H tile of pixels, each warp a TILE_W x
// TILE_H part of it, so that a warp's camera rays are neighbours in both
// directions (the launch has primary_blocks(W, H) blocks of PATH_BLOCK
// threads).
__global__ void __launch_bounds__(PATH_BLOCK) k_primary(FrameParams F) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    const int tiles_x = (F.W + 2 * TILE_W - 1) / (2 * TILE_W);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = (blockIdx.x % tiles_x) * (2 * TILE_W) + (w & 1) * TILE_W + (lane % TILE_W);
    const int y = (blockIdx.x / tiles_x) * (2 * TILE_H) + (w >> 1) * TILE_H + (lane / TILE_W);
    const bool in = x < F.W && y < F.H;
    const int p = y * F.W + x;
    Hit h;
    h.inst = -1;
    XRay r;
    if (in) {
        r = camera_ray(F, x, y);
        h = trace_closest(F.scene, r, 0.0f, __int_as_float(0x7f800000), st, stack);
    }
    const bool hit = in && h.inst >= 0;
    const bool miss = in && h.inst < 0;
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
        // Ray::getPointAt, IEEE: the visible surface's position (interaction.cu:23)
        if (F.vis)
            F.vis[p] = make_float4(__fadd_rn(r.o.x, __fmul_rn(h.t, r.d.x)), __fadd_rn(r.o.y, __fmul_rn(h.t, r.d.y)),
                                   __fadd_rn(r.o.z, __fmul_rn(h.t, r.d.z)), h.t);
    } else if (miss) {
        F.miss_list[m] = p;
        F.hit_index[p] = -1;
        if (F.first_hit) F.first_hit[p] = make_int4(-1, -1, 0x7f800000, 0);
        if (F.vis) F.vis[p] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0x7f800000));
    }
    flush_stats(st, F.counters ? F.counters + 4 : nullptr);
    if (F.counters && threadIdx.x == 0) {   // camera rays of this block: its tile inside the image
        const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
        const int nb = min(2 * TILE_W, F.W - tx * 2 * TILE_W) * min(2 * TILE_H, F.H - ty * 2 * TILE_H);
        if (nb > 0) atomicAdd(F.counters + 14, (unsigned long long)nb);
    }
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
// paths: one wave of work items advanced level by level

// Shadow ray of Integrator::unoccluded (integrator.cuh:124-131): from the
// offset surface point towards `target`, stopping 0.11 short of it.
__device__ __forceinline__ void shadow_ray(const Surf& si, float3 target, float3& o, float3& d, float& tmax) {
    o = si.backface ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
    d = normalize(target - o);
    tmax = length(target - o) - 0.11f;
}

__device__ __forceinline__ void emit_shadow(const FrameParams& F, const Surf& si, float3 target, float3 contrib,
                                            int item, int* counter, bool from_back) {
    float3 o, d;
    float tmax;
    shadow_ray(si, target, o, d, tmax);
    int j = group_append(counter);
    if (from_back) j = F.cap - 1 - j;
    ShadowRec r;
    r.o_tmax = make_float4(o.x, o.y, o.z, tmax);
    r.d_item = make_float4(d.x, d.y, d.z, __int_as_float(item));
    r.contrib = make_float4(contrib.x, contrib.y, contrib.z, 0.0f);
    F.shadow[j] = r;
}

// One vertex of Integrator::Li (integrator.cuh:266-399) for every path of the
// wave entering `level`: emission with its MIS weight, one light sample --
// LeSun / sampleLdSun (:135-186) or sampleLd (:188-220) -- whose shadow ray
// goes to k_shadow with the radiance it would add, the BSDF sample and
// russianRoulette (maths/sampling.cuh:19-31).  A path whose ray left the
// scene goes to the sky queue.  The radiance of each item is kept in
// `radiance` and receives its terms in the reference's order: this vertex's
// emission here, its light sample in k_shadow, the next vertex's terms at the
// next level, the sky last.  Level 0 starts the paths of items
// wave0 .. wave0+cap-1 from the camera-ray hits of k_primary.
// One vertex of Integrator::Li for one path (the loop body of shade_level,
// below): `h` is the path's hit at this level; o, d the ray that found it;
// beta, p_b, prev and seed the path's throughput, BSDF pdf, previous vertex
// and random-number state; L its radiance so far.  The vertex's outcomes go
// to `sink`: the sky direction of a path that left the scene (its last
// term), the radiance after this vertex's emission, the shadow ray of its
// light sample with the radiance it adds if unoccluded (sun: true for a sun
// sample), and the continuation (a PathRec, the next level's input).
template <class Sink>
__device__ __forceinline__ void shade_vertex(const FrameParams& F, int level, const PrimaryRec& h, float3 o, float3 d,
                                             float3 beta, float3 prev, float3 L, float p_b, uint32_t seed, int item,
                                             Sink& sink) {
    const SceneView& s = F.scene;
    const SkyParams& P = F.sky;
    const int order = F.rng_order;
    const int nl = s.nlights;
    const bool first = level == 0;
    if (h.inst < 0) {
        sink.sky(item, d, beta, L);   // the path ends here: the sky is its last term
        return;
    }
    Sampler S;
    S.seed = seed + (uint32_t)level;
    Surf si = surface_at(s, h.inst, h.tri, h.t, h.u, h.v, o, d);
    float3 Le = make_float3(0.0f, 0.0f, 0.0f);
    if (si.light >= 0) Le = emission_of(s, si.material, si.uv);
    if (nonzero(Le)) {
        float w_l = 1.0f;
        if (si.light >= 0 && !first) {
            const LightRec& lt = s.lights[si.light];
            float pmf = 1.0f / (float)nl;
            float dist = length(si.pos - prev);
            float cosl = AbsDot(normalize(si.pos - prev), si.ng);
            float lpdf = pmf * ((1.0f / lt.area) / (cosl / Sqr(dist)));
            w_l = Sqr(p_b) / (Sqr(p_b) + Sqr(lpdf));
        }
        L = L + Le * w_l * beta;
    }
    Bsdf bsdf = bsdf_at(s, si);
    if (first) bsdf.albedo = make_float3(1.0f, 1.0f, 1.0f);   // demodulate (bsdf.cuh:286-288)
    if (!first && bsdf.alpha < 0.3f) bsdf.alpha = clampf(2.0f * bsdf.alpha, 0.1f, 0.3f);
    const float3 wo = -d;
    if (!(bsdf.alpha < 0.001f)) {
        // The light sample: each branch draws its numbers and sets up its
        // direction; the BSDF is then evaluated once for all lanes (the
        // sun / area-light choice is random per lane, so both branches
        // run in every warp), and each branch finishes its own sample.
        const bool sun = S.get1D() < 0.5f;
        const float dsun = 149.597e9f;
        // the sun's centre at 1 AU, each product rounded on its own:
        // target - sun_pos below cancels two values near 1.5e11, which a
        // fused multiply-add would shift by up to half their ulp (~1e-5
        // of the difference) -- as the reference's GPU build does, with
        // gpu_arith
        const float3 sun_pos = P.gpu_arith ? P.sun_dir * dsun
                                           : make_float3(__fmul_rn(P.sun_dir.x, dsun), __fmul_rn(P.sun_dir.y, dsun),
                                                         __fmul_rn(P.sun_dir.z, dsun));
        float3 wi = P.sun_dir, target, Lem;
        float pdf = 0.0f, prob = 0.0f;
        bool eval;
        if (sun) {
            // sampleLdSun: jittered point on the sun disc at 1 AU
            float3 off;
            if ((order & RNG_SUN) == 0) {
                float2 a = S.get2D(order);
                float b = S.get1D();
                off = make_float3(a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f);
            } else {
                float b = S.get1D();
                float2 a = S.get2D(order);
                off = make_float3(a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f);
            }
            target = P.gpu_arith ? sun_pos + (off * P.sun_radius_m)
                                 : make_float3(__fadd_rn(sun_pos.x, __fmul_rn(off.x, P.sun_radius_m)),
                                               __fadd_rn(sun_pos.y, __fmul_rn(off.y, P.sun_radius_m)),
                                               __fadd_rn(sun_pos.z, __fmul_rn(off.z, P.sun_radius_m)));
            eval = true;
        } else {
            // sampleLd: uniform light pick, uniform point on the triangle
            float X = S.get1D();
            eval = false;
            if (nl >= 1) {
                int li = min((int)(X * (float)nl), nl - 1);
                const LightRec& lt = s.lights[li];
                prob = 1.0f / (float)nl;
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
                pdf = 1.0f / lt.tri_area;
                pdf *= Sqr(length(p - si.pos));
                pdf /= AbsDot(normalize(p - si.pos), gn);
                wi = normalize(p - si.pos);
                Lem = emission_of(s, lt.material, luv);
                target = p;
                eval = !(pdf <= 0.0f || !nonzero(Lem));
            }
        }
        float3 fcos = make_float3(0.0f, 0.0f, 0.0f);
        if (eval) fcos = bsdf.f(wo, wi) * fmaxf(0.0f, dot(wi, (si.backface ? -1.0f : 1.0f) * si.ng));
        if (sun) {
            const float3 sun_rad = *F.sun_radiance;
            if (nonzero(fcos) && nonzero(sun_rad)) {
                float area = PI_F * Sqr(P.sun_radius_m);
                float3 sn = normalize(target - sun_pos), wt = normalize(target - si.pos);
                float th = AbsDot(sn, -wt);
                float spdf = (1.0f / area) / (th / Sqr(dsun));
                float3 Ld = (fcos * sun_rad * 6.0e5f) / spdf;
                float3 c = Ld * beta / 0.5f;
                if (!(c.x == 0.0f && c.y == 0.0f && c.z == 0.0f))
                    sink.shadow(si, target, c, item, true);
            }
        } else if (eval && nonzero(fcos)) {
            float p_l = prob * pdf;
            float pb = bsdf.pdf(wo, wi);
            float w_l = Sqr(p_l) / (Sqr(p_l) + Sqr(pb));
            float3 Ld = (Lem * fcos * w_l) / p_l;
            float3 c = Ld * beta / (1.0f - 0.5f);
            if (!(c.x == 0.0f && c.y == 0.0f && c.z == 0.0f))
                sink.shadow(si, target, c, item, false);
        }
    }
    sink.radiance(item, L);
    if (level == F.max_depth) return;
    float2 uu, X;
    if ((order & RNG_BSDF) == 0) { uu = S.get2D(order); X = S.get2D(order); }
    else { X = S.get2D(order); uu = S.get2D(order); }
    BsdfSample bs = bsdf.sample(wo, uu, X);
    if (bs.scatter == SC_ABSORBED || !nonzero(bs.f)) return;
    beta = beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
    p_b = bsdf.pdf(wo, bs.wi);
    o = (bs.scatter & SC_TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
    float mx = fmaxf(beta.x, fmaxf(beta.y, beta.z));
    if (mx < 1.0f && level >= 1) {
        float q = fmaxf(0.0f, 1.0f - mx);
        if (S.get1D() < q) return;
        beta = beta / (1.0f - q);
    }
    if (!nonzero(beta)) return;   // while (throughput) (integrator.cuh:266)
    PathRec pr;
    pr.o_pb = make_float4(o.x, o.y, o.z, p_b);
    pr.d_seed = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, __uint_as_float(S.seed));
    pr.beta_item = make_float4(beta.x, beta.y, beta.z, __int_as_float(item));
    pr.prev = make_float4(si.pos.x, si.pos.y, si.pos.z, 0.0f);
    sink.next(pr);
}

// The wave's sink: sky lookups, shadow rays and continuations appended to the
// level's compacted queues, the radiance written back to the item.
struct WaveSink {
    const FrameParams& F;
    int* here;        // level_counts of this level
    int* ahead;       // level_counts of the next level
    PathRec* out;     // the next level's paths
    __device__ __forceinline__ void sky(int item, float3 d, float3 beta, float3) {
        const int q = group_append(F.counts + 2);
        F.sky_queue[2 * (size_t)q] = make_float4(__int_as_float(item), d.x, d.y, d.z);
        F.sky_queue[2 * (size_t)q + 1] = make_float4(beta.x, beta.y, beta.z, 0.0f);
    }
    __device__ __forceinline__ void radiance(int item, float3 L) {
        F.radiance[item] = make_float4(L.x, L.y, L.z, 0.0f);
    }
    __device__ __forceinline__ void shadow(const Surf& si, float3 target, float3 c, int item, bool sun) {
        if (sun) emit_shadow(F, si, target, c, item, here + 1, false);
        else emit_shadow(F, si, target, c, item, here + 2, true);
    }
    __device__ __forceinline__ void next(const PathRec& pr) {
        const int j = group_append(ahead);
        out[j] = pr;
    }
};

// The lobe family of a path's hit, for grouping the shading of a level:
// 0 opaque dielectric, 1 conductor, 2 transparent dielectric, 3 mixed
// (fractional metallic or transmission, or a texture that makes them so),
// 4 no hit (the path leaves the scene).
__device__ __forceinline__ int lobe_family(const SceneView& s, const PrimaryRec& h) {
    if (h.inst < 0) return 4;
    const InstRec& ir = s.inst[h.inst];
    const int m = ir.material >= 0 ? ir.material : s.shade[s.meshes[ir.mesh].shade_base + h.tri].material;
    const MatRec& mr = s.materials[m];
    if (mr.orm_tex >= 0 || mr.transmission_tex >= 0) return 3;
    if (mr.metallic == 0.0f) return mr.transmission == 0.0f ? 0 : (mr.transmission == 1.0f ? 2 : 3);
    return mr.metallic == 1.0f ? 1 : 3;
}

__device__ __forceinline__ void shade_path(const FrameParams& F, bool first, int level, long long wave0, int i,
                                           int* here, int* next, PathRec* out) {
    float3 o, d, beta, prev, L;
    float p_b;
    uint32_t seed;
    int item;
    PrimaryRec h;
    if (first) {
        // items are pixel-major: the samples of one camera hit are
        // neighbours (one surface point, one material)
        item = (int)(wave0 + i);
        const int hj = item / F.nsamples;
        const int k = item - hj * F.nsamples;
        const int p = F.hit_list[hj];
        const int x = p % F.W, y = p / F.W;
        Sampler S0;
        S0.init(x, y, F.W, F.sample0 + k);
        S0.get1D();   // BoxFilter::sample, result discarded (kernels.cu:397-402)
        S0.get1D();
        XRay r = camera_ray(F, x, y);
        o = r.o;
        d = r.d;
        beta = make_float3(1.0f, 1.0f, 1.0f);
        prev = make_float3(0.0f, 0.0f, 0.0f);
        L = make_float3(0.0f, 0.0f, 0.0f);
        p_b = 1.0f;
        seed = S0.seed;
        h = F.primary[p];
    } else {
        const PathRec pr = F.paths[level & 1][i];
        o = make_float3(pr.o_pb.x, pr.o_pb.y, pr.o_pb.z);
        p_b = pr.o_pb.w;
        d = make_float3(pr.d_seed.x, pr.d_seed.y, pr.d_seed.z);
        seed = __float_as_uint(pr.d_seed.w);
        beta = make_float3(pr.beta_item.x, pr.beta_item.y, pr.beta_item.z);
        item = __float_as_int(pr.beta_item.w);
        prev = make_float3(pr.prev.x, pr.prev.y, pr.prev.z);
        h = F.hits[i];
        const float4 l4 = F.radiance[item];
        L = make_float3(l4.x, l4.y, l4.z);
    }
    WaveSink sink{F, here, next, out};
    shade_vertex(F, level, h, o, d, beta, prev, L, p_b, seed, item, sink);
}

// BOUNCE: levels >= 1 only (the host launches level 0 with BOUNCE false and
// every later level with BOUNCE true, whatever F.group_lobes, so that each
// level's shading is the same compiled code in every configuration)
template <bool BOUNCE>
__device__ __forceinline__ void shade_level(const FrameParams& F, int level, long long wave0) {
    const bool first = !BOUNCE && level == 0;
    int n;
    if (first) {
        const long long left = (long long)F.counts[0] * F.nsamples - wave0;
        n = (int)(left < 0 ? 0 : (left < F.cap ? left : F.cap));
    } else {
        n = F.level_counts[LEVEL_WORDS * level];
    }
    PathRec* out = F.unsorted ? F.unsorted : F.paths[(level + 1) & 1];
    int* here = F.level_counts + LEVEL_WORDS * level;
    int* next = F.level_counts + LEVEL_WORDS * (level + 1);
    // the wave's paths entering level 0 (levels >= 1 count theirs as they
    // are appended); read back by kpt_get_level_counts
    if (first && blockIdx.x == 0 && threadIdx.x == 0) here[0] = n;
    if (!BOUNCE) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            shade_path(F, first, level, wave0, i, here, next, out);
        return;
    }
    // Levels >= 1: the blocks stride over the level's paths in windows.
    // With F.group_lobes > 0 a window holds up to F.group_lobes paths, sized
    // so that every block gets the same number of windows, and is regrouped
    // by the lobe family of its hits (a counting sort in shared memory) so
    // that a warp mostly runs one family's code -- a level's paths hit every
    // kind of material in queue order; the block synchronises once per
    // window, not once per path of a thread.  Otherwise a window is one
    // block of paths in queue order.  Every path is shaded exactly once and
    // its result does not depend on its slot.
    const bool group = F.group_lobes > 0;
    __shared__ int fam_count[8];
    __shared__ int order[SHADE_WINDOW];
    __shared__ unsigned char fam_of[SHADE_WINDOW];
    const int lane = threadIdx.x & 31;
    int win = blockDim.x;
    if (group && n > 0) {
        const int wmax = max((int)blockDim.x, (min(F.group_lobes, SHADE_WINDOW) / (int)blockDim.x) * (int)blockDim.x);
        const int per_sweep = gridDim.x * wmax;   // n <= 2^25 and per_sweep <= 2^21: no overflow
        const int sweeps = (n + per_sweep - 1) / per_sweep;
        win = (n + gridDim.x * sweeps - 1) / (gridDim.x * sweeps);
    }
    // the counting loops run over whole blocks (full warps for the warp votes)
    const int span = (win + blockDim.x - 1) / blockDim.x * blockDim.x;
    for (int w0 = blockIdx.x * win; w0 < n; w0 += gridDim.x * win) {
        const int m = min(win, n - w0);
        if (group) {
            if (threadIdx.x < 8) fam_count[threadIdx.x] = 0;
            __syncthreads();
            // count each family (one shared atomic per family present in a warp)
            for (int j = threadIdx.x; j < span; j += blockDim.x) {
                const int f = j < m ? lobe_family(F.scene, F.hits[w0 + j]) : 5;
                fam_of[j] = (unsigned char)f;
                const unsigned peers = __match_any_sync(0xffffffffu, f);
                if (lane == __ffs(peers) - 1) atomicAdd(&fam_count[f], __popc(peers));
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int off = 0;
                for (int k = 0; k < 6; ++k) {
                    const int c = fam_count[k];
                    fam_count[k] = off;
                    off += c;
                }
            }
            __syncthreads();
            // place: the family's offset + the paths of the family placed before
            for (int j = threadIdx.x; j < span; j += blockDim.x) {
                const int f = fam_of[j];
                const unsigned peers = __match_any_sync(0xffffffffu, f);
                const int leader = __ffs(peers) - 1;
                int b = 0;
                if (lane == leader) b = atomicAdd(&fam_count[f], __popc(peers));
                b = __shfl_sync(0xffffffffu, b, leader);
                order[b + __popc(peers & ((1u << lane) - 1u))] = w0 + j;
            }
            __syncthreads();
        }
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            shade_path(F, false, level, wave0, group ? order[j] : w0 + j, here, next, out);
        if (group) __syncthreads();
    }
}

// one kernel per block-size bound, so that the register allocation of the
// default launch does not depend on the largest one; k_shade* shade level 0
// (camera hits), k_shade_bounce* levels >= 1 (held to 64 registers: their
// window loop would otherwise take the allocation past it and cost a quarter
// of the resident warps)
__global__ void __launch_bounds__(PATH_BLOCK) k_shade(FrameParams F, int level, long long wave0) {
    shade_level<false>(F, level, wave0);
}
__global__ void __launch_bounds__(SHADE_MAX_BLOCK) k_shade_wide(FrameParams F, int level, long long wave0) {
    shade_level<false>(F, level, wave0);
}
__global__ void __launch_bounds__(PATH_BLOCK, 8) k_shade_bounce(FrameParams F, int level, long long wave0) {
    shade_level<true>(F, level, wave0);
}
__global__ void __launch_bounds__(SHADE_MAX_BLOCK, 4) k_shade_bounce_wide(FrameParams F, int level, long long wave0) {
    shade_level<true>(F, level, wave0);
}

// Rays the wave traced: extension rays (paths entering levels >= 1) and
// shadow rays (every level), from the level counters before the next wave
// clears them; the camera rays are counted by k_primary.
__global__ void k_count_rays(FrameParams F) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long ext = 0, shd = 0;
    for (int l = 0; l <= F.max_depth; ++l) {
        const int* lc = F.level_counts + LEVEL_WORDS * l;
        if (l > 0) ext += (unsigned)lc[0];
        shd += (unsigned)lc[1] + (unsigned)lc[2];
    }
    F.counters[12] += ext;
    F.counters[13] += shd;
}

// ---------------------------------------------------------------------------
// octant sort of the continuations: rays of one warp then share a direction
// octant (the queue order otherwise follows the pixels, so origins are
// already coherent).  A path's result does not depend on its queue slot.

__device__ __forceinline__ int octant(float4 d) {
    return (d.x < 0.0f ? 1 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 4 : 0);
}

__global__ void __launch_bounds__(256) k_sort_count(FrameParams F, int level) {
    __shared__ int h[8];
    if (threadIdx.x < 8) h[threadIdx.x] = 0;
    __syncthreads();
    const int n = F.level_counts[LEVEL_WORDS * level];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[octant(F.unsorted[i].d_seed)], 1);
    __syncthreads();
    if (threadIdx.x < 8 && h[threadIdx.x]) atomicAdd(&F.octants[16 * level + threadIdx.x], h[threadIdx.x]);
}

__global__ void __launch_bounds__(256) k_sort_scatter(FrameParams F, int level) {
    const int n = F.level_counts[LEVEL_WORDS * level];
    const int* cnt = F.octants + 16 * level;
    int* cursor = F.octants + 16 * level + 8;
    int off[8];
    int acc = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        off[o] = acc;
        acc += cnt[o];
    }
    PathRec* out = F.paths[level & 1];
    const int lane = threadIdx.x & 31;
    // warp-uniform loop: every lane takes part in the warp-level appends
    for (int w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < n; w0 += gridDim.x * blockDim.x) {
        const int i = w0 + lane;
        const bool ok = i < n;
        PathRec r;
        int o = 8;
        if (ok) {
            r = F.unsorted[i];
            o = octant(r.d_seed);
        }
        const unsigned same = __match_any_sync(0xffffffffu, o);
        const int leader = __ffs(same) - 1;
        int b = 0;
        if (ok && lane == leader) b = atomicAdd(cursor + o, __popc(same));
        b = __shfl_sync(0xffffffffu, b, leader);
        if (ok) {
            int dst = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) dst = (q == o) ? off[q] : dst;
            out[dst + b + __popc(same & ((1u << lane) - 1u))] = r;
        }
    }
}

// Closest hits of the paths entering `level` (1 .. max_depth).
struct ExtendQueue {
    const PathRec* in;
    PrimaryRec* out;
    __device__ __forceinline__ void ray(int i, float3& o, float3& d, float& tmin, float& tmax) const {
        const float4 a = in[i].o_pb, b = in[i].d_seed;
        o = make_float3(a.x, a.y, a.z);
        d = make_float3(b.x, b.y, b.z);
        tmin = 0.0f;
        tmax = __int_as_float(0x7f800000);
    }
    __device__ __forceinline__ bool closest(int i, const Hit& h, float3&, float3&) const {
        PrimaryRec r;
        r.t = h.t;
        r.u = h.u;
        r.v = h.v;
        r.inst = h.inst;
        r.tri = h.tri;
        r.pad0 = r.pad1 = r.pad2 = 0;
        out[i] = r;
        return false;
    }
    __device__ __forceinline__ void any(int, bool) const {}
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_extend(FrameParams F, int level) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    int* lc = F.level_counts + LEVEL_WORDS * level;
    ExtendQueue q{F.paths[level & 1], F.hits};
    trace_queue<false>(F.scene, lc[0], lc + 3, q, st, stack);
    flush_stats(st, F.counters);
}

// Shadow rays of `level` (sun rays from the front of the buffer, light rays
// from the back): an unoccluded ray adds its radiance to its item.
struct ShadowQueue {
    const ShadowRec* rec;
    float4* radiance;
    int nsun, cap;
    __device__ __forceinline__ int slot(int i) const { return i < nsun ? i : cap - 1 - (i - nsun); }
    __device__ __forceinline__ void ray(int i, float3& o, float3& d, float& tmin, float& tmax) const {
        const int j = slot(i);
        const float4 a = rec[j].o_tmax, b = rec[j].d_item;
        o = make_float3(a.x, a.y, a.z);
        d = make_float3(b.x, b.y, b.z);
        tmin = 0.0f;
        tmax = a.w;
    }
    __device__ __forceinline__ bool closest(int, const Hit&, float3&, float3&) const { return false; }
    __device__ __forceinline__ void any(int i, bool occluded) const {
        if (occluded) return;
        const int j = slot(i);
        const int item = __float_as_int(rec[j].d_item.w);
        const float4 c = rec[j].contrib;
        const float4 L = radiance[item];
        radiance[item] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
    }
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_shadow(FrameParams F, int level) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    int* lc = F.level_counts + LEVEL_WORDS * level;
    // the sky queue cannot grow while this kernel runs (k_shade(level) has
    // ended, k_shade(level + 1) waits for it): its length ends level's range
    if (blockIdx.x == 0 && threadIdx.x == 0) lc[5] = F.counts[2];
    ShadowQueue q{F.shadow, F.radiance, lc[1], F.cap};
    trace_queue<true>(F.scene, lc[1] + lc[2], lc + 4, q, st, stack);
    flush_stats(st, F.counters + 8);
}

// ---------------------------------------------------------------------------
// Temporal accumulation in the reference GPU build's arithmetic
// (kpt_settings.temporal_arith = 1): computeVelocity, testReprojection and
// reprojectAccumulate (kernels.cu:164-223, 299-327) with the matrix
// inverses, products and divisions computed per pixel as that build computes
// them -- this translation unit's fast maths: contracted products,
// approximate reciprocal and square root.  The reference inverts four
// camera matrices and the previous model matrix for every pixel, and the
// velocity of a still camera is then a few ulps, not zero: the previous
// pixel coordinate, truncated, and the bilinear weights follow those ulps.
// The order of operations is the reference's (Mat4 products row by row left
// to right, Mat4::inverse's closed form, lerp as a + t (b - a)).

struct M4 {
    float4 c[4];   // columns
};

__device__ __forceinline__ M4 m4_load(const float4* cols) {
    M4 m;
    for (int k = 0; k < 4; ++k) m.c[k] = cols[k];
    return m;
}

// Mat4 * float4 (matrix_maths.cuh:258-267)
__device__ __forceinline__ float4 m4_apply(const M4& m, float4 v) {
    return make_float4(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w,
                       m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w,
                       m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w,
                       m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w);
}

// Mat4 * Mat4 (matrix_maths.cuh:269-283): column j is a * b.c[j]
__device__ __forceinline__ M4 m4_mul(const M4& a, const M4& b) {
    M4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = m4_apply(a, b.c[j]);
    return r;
}

// Mat4::inverse (matrix_maths.cuh:304-354): cofactors of the column-major
// entries, the identity when |det| < 1e-6
__device__ __forceinline__ M4 m4_inverse(const M4& m) {
    const float4 c0 = m.c[0], c1 = m.c[1], c2 = m.c[2], c3 = m.c[3];
    const float s00 = c2.z * c3.w - c3.z * c2.w;
    const float s01 = c2.y * c3.w - c3.y * c2.w;
    const float s02 = c2.y * c3.z - c3.y * c2.z;
    const float s03 = c2.x * c3.w - c3.x * c2.w;
    const float s04 = c2.x * c3.z - c3.x * c2.z;
    const float s05 = c2.x * c3.y - c3.x * c2.y;
    const float det = c0.x * (c1.y * s00 - c1.z * s01 + c1.w * s02) - c0.y * (c1.x * s00 - c1.z * s03 + c1.w * s04) +
                      c0.z * (c1.x * s01 - c1.y * s03 + c1.w * s05) - c0.w * (c1.x * s02 - c1.y * s04 + c1.z * s05);
    M4 r;
    if (fabsf(det) < 1e-6f) {
        r.c[0] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        r.c[1] = make_float4(0.0f, 1.0f, 0.0f, 0.0f);
        r.c[2] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        r.c[3] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        return r;
    }
    const float id = 1.0f / det;
    r.c[0].x = (c1.y * s00 - c1.z * s01 + c1.w * s02) * id;
    r.c[0].y = -(c0.y * s00 - c0.z * s01 + c0.w * s02) * id;
    r.c[0].z = (c0.y * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.y * c3.w - c1.w * c3.y) + c0.w * (c1.y * c3.z - c1.z * c3.y)) * id;
    r.c[0].w = -(c0.y * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.y * c2.w - c1.w * c2.y) + c0.w * (c1.y * c2.z - c1.z * c2.y)) * id;
    r.c[1].x = -(c1.x * s00 - c1.z * s03 + c1.w * s04) * id;
    r.c[1].y = (c0.x * s00 - c0.z * s03 + c0.w * s04) * id;
    r.c[1].z = -(c0.x * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.z - c1.z * c3.x)) * id;
    r.c[1].w = (c0.x * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.z - c1.z * c2.x)) * id;
    r.c[2].x = (c1.x * s01 - c1.y * s03 + c1.w * s05) * id;
    r.c[2].y = -(c0.x * s01 - c0.y * s03 + c0.w * s05) * id;
    r.c[2].z = (c0.x * (c1.y * c3.w - c1.w * c3.y) - c0.y * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.y - c1.y * c3.x)) * id;
    r.c[2].w = -(c0.x * (c1.y * c2.w - c1.w * c2.y) - c0.y * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.y - c1.y * c2.x)) * id;
    r.c[3].x = -(c1.x * s02 - c1.y * s04 + c1.z * s05) * id;
    r.c[3].y = (c0.x * s02 - c0.y * s04 + c0.z * s05) * id;
    r.c[3].z = -(c0.x * (c1.y * c3.z - c1.z * c3.y) - c0.y * (c1.x * c3.z - c1.z * c3.x) + c0.z * (c1.x * c3.y - c1.y * c3.x)) * id;
    r.c[3].w = (c0.x * (c1.y * c2.z - c1.z * c2.y) - c0.y * (c1.x * c2.z - c1.z * c2.x) + c0.z * (c1.x * c2.y - c1.y * c2.x)) * id;
    return r;
}

__device__ __forceinline__ float4 tex_clamp(const float4* t, int W, int H, int x, int y) {   // cudaBoundaryModeClamp
    x = min(max(x, 0), W - 1);
    y = min(max(y, 0), H - 1);
    return t[(size_t)y * W + x];
}

__device__ __forceinline__ float4 lerp_fm(float4 a, float4 b, float t) {
    return make_float4(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w));
}

__global__ void k_temporal_gpu(TemporalParams T) {
    const int npix = T.W * T.H;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int x = p % T.W, y = p / T.W;
    const int j = T.hit_index[p];
    float4 L = j < 0 ? T.pixel_sky[p] : T.radiance[(size_t)j * T.nsamples + T.sample];
    // RGBSpectrum::clampOutput (color.cuh:295-302)
    if (isnan(L.x) || isnan(L.y) || isnan(L.z) || isinf(L.x) || isinf(L.y) || isinf(L.z))
        L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float3 curr = make_float3(fmaxf(0.0f, fminf(L.x, 1.0e8f)), fmaxf(0.0f, fminf(L.y, 1.0e8f)),
                                    fmaxf(0.0f, fminf(L.z, 1.0e8f)));
    float4 out = make_float4(curr.x, curr.y, curr.z, 0.0f);
    if (j < 0) {
        if (T.depth_out) T.depth_out[p] = T.vis[p].w;
    } else {
        const PrimaryRec pr = T.primary[p];
        const TemporalGpuInst& I = T.ginst[pr.inst];
        // the visible surface as the reference's GPU build finds it
        // (VisibleSurface, packing.cuh:156-176): the camera ray of
        // Camera::generateRay (camera.cuh:16-25) with the pixel's
        // uv = (pixel + 1/2) / resolution (shading_kernel.cuh:23), the hit
        // triangle's distance by Triangle::intersect (triangle.cuh:66-102) on
        // the ray in object space (Ray::transform), the point o + t d
        // (Ray::getPointAt), the distance as its depth
        const float ux = ((float)x + 0.5f) / (float)T.W, uy = ((float)y + 0.5f) / (float)T.H;
        const float4 tc = m4_apply(m4_load(T.inv_proj), make_float4(2.0f * ux - 1.0f, 2.0f * uy - 1.0f, 1.0f, 1.0f));
        float3 v = make_float3(tc.x / tc.w, tc.y / tc.w, tc.z / tc.w);
        v = v * rsqrtf(dot(v, v));
        const float4 tw = m4_apply(m4_load(T.inv_view), make_float4(v.x, v.y, v.z, 0.0f));
        float3 rd = make_float3(tw.x, tw.y, tw.z);
        rd = rd * rsqrtf(dot(rd, rd));
        const float3 ro = make_float3(T.inv_view[3].x, T.inv_view[3].y, T.inv_view[3].z);
        const M4 im = m4_load(I.inv_model);
        const float4 oo = m4_apply(im, make_float4(ro.x, ro.y, ro.z, 1.0f));
        const float4 od = m4_apply(im, make_float4(rd.x, rd.y, rd.z, 0.0f));
        const int li = T.tri_leaf[I.tri_base + pr.tri];
        const float4 ta = T.tris[3 * (size_t)li], tb = T.tris[3 * (size_t)li + 1], tc2 = T.tris[3 * (size_t)li + 2];
        const float3 v0 = make_float3(ta.x, ta.y, ta.z), e1 = make_float3(tb.x, tb.y, tb.z),
                     e2 = make_float3(tc2.x, tc2.y, tc2.z);
        const float3 pvec = cross(make_float3(od.x, od.y, od.z), e2);
        const float inv_det = 1.0f / dot(e1, pvec);
        const float3 tvec = make_float3(oo.x, oo.y, oo.z) - v0;
        const float3 qvec = cross(tvec, e1);
        const float th = inv_det * dot(e2, qvec);
        const float3 wp = ro + th * rd;
        if (T.depth_out) T.depth_out[p] = th;
        // computeVelocity (kernels.cu:164-192)
        const M4 cvp = m4_mul(m4_inverse(m4_load(T.inv_proj)), m4_inverse(m4_load(T.inv_view)));
        const M4 pvp = m4_mul(m4_inverse(m4_load(T.prev_inv_proj)), m4_inverse(m4_load(T.prev_inv_view)));
        const M4 pmodel = m4_inverse(m4_load(I.prev_inv_model));
        const float4 pos = make_float4(wp.x, wp.y, wp.z, 1.0f);
        const float4 l4 = m4_apply(m4_load(I.inv_model), pos);
        const float4 local = make_float4(l4.x, l4.y, l4.z, 1.0f);
        const float4 cc = m4_apply(cvp, pos);
        const float4 pc = m4_apply(m4_mul(pvp, pmodel), local);
        const float cx = cc.x / cc.w, cy = cc.y / cc.w;
        const float px = pc.x / pc.w, py = pc.y / pc.w;
        const float vx = (cx + 1.0f) / 2.0f - (px + 1.0f) / 2.0f;
        const float vy = (cy + 1.0f) / 2.0f - (py + 1.0f) / 2.0f;
        // reprojectAccumulate (kernels.cu:299-327)
        const float qx = (float)x - vx * (float)T.W;
        const float qy = (float)y - vy * (float)T.H;
        if (!(qx < 0.0f || qx >= (float)T.W || qy < 0.0f || qy >= (float)T.H)) {
            // testReprojection (kernels.cu:206-223)
            const int ix = (int)qx, iy = (int)qy;
            const float d2 = T.prev_depth[(size_t)min(max(iy, 0), T.H - 1) * T.W + min(max(ix, 0), T.W - 1)];
            const float4 w4 = m4_apply(pmodel, local);
            const float dx = T.prev_inv_view[3].x - w4.x, dy = T.prev_inv_view[3].y - w4.y,
                        dz = T.prev_inv_view[3].z - w4.z;
            const float d1 = sqrtf(dx * dx + dy * dy + dz * dz);
            if (fabsf(d1 - d2) < d2 * 0.045f) {
                // DeviceTextureBuffer::textureReadBilinear (device_texture_buffer.cuh:42-80), alpha point-sampled
                const float ws = qx - (float)ix, wt = qy - (float)iy;
                const float4 c0 = tex_clamp(T.hist_in, T.W, T.H, ix, iy), c1 = tex_clamp(T.hist_in, T.W, T.H, ix + 1, iy);
                const float4 c2 = tex_clamp(T.hist_in, T.W, T.H, ix, iy + 1),
                             c3 = tex_clamp(T.hist_in, T.W, T.H, ix + 1, iy + 1);
                float4 prev = lerp_fm(lerp_fm(c0, c1, ws), lerp_fm(c2, c3, ws), wt);
                prev.w = c0.w;
                const float alpha = 1.0f / fminf(prev.w + 1.0f, 16.0f);
                out = make_float4(prev.x + alpha * (curr.x - prev.x), prev.y + alpha * (curr.y - prev.y),
                                  prev.z + alpha * (curr.z - prev.z), prev.w + 1.0f);
            }
        }
    }
    T.hist_out[p] = out;
}

// ---------------------------------------------------------------------------
// A batch's ray stages: the extension rays of level + 1 and the shadow rays
// of level of every job, each traced by one persistent launch from one queue
// spanning the jobs, in the batch's merged scene (every job's BLAS and TLAS
// nodes, triangles, meshes and instances, indices moved by the job's
// offsets).  An entry's job is found by its place in the prefix sums; its
// TLAS root is the job's; its result goes to the job's own buffers, in the
// job's own numbering, so each job's frame is the one it renders alone.

__global__ void k_batch_level(BatchQueues Q, int level) {
    // one warp: lane j takes jobs j, j + 32, ...; the prefix sums by warp scans
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    if (lane == 0) {
        Q.ext_prefix[0] = Q.shd_prefix[0] = 0;
        Q.fetch[0] = Q.fetch[1] = 0;
    }
    int e_base = 0, s_base = 0;
    for (int j0 = 0; j0 < Q.njobs; j0 += 32) {
        const int j = j0 + lane;
        int e = 0, sh = 0;
        if (j < Q.njobs) {
            const BatchJob& J = Q.jobs[j];
            if (level <= J.max_depth) {
                int* lc = J.level_counts + LEVEL_WORDS * level;
                sh = lc[1] + lc[2];
                // the job's sky queue cannot grow before its k_shade(level + 1):
                // its length ends level's range (as k_shadow records it)
                lc[5] = J.counts[2];
                if (level + 1 <= J.max_depth) e = J.level_counts[LEVEL_WORDS * (level + 1)];
            }
        }
        for (int o = 1; o < 32; o <<= 1) {
            const int te = __shfl_up_sync(0xffffffffu, e, o), ts = __shfl_up_sync(0xffffffffu, sh, o);
            if (lane >= o) {
                e += te;
                sh += ts;
            }
        }
        if (j < Q.njobs) {
            Q.ext_prefix[j + 1] = e_base + e;
            Q.shd_prefix[j + 1] = s_base + sh;
        }
        e_base += __shfl_sync(0xffffffffu, e, 31);
        s_base += __shfl_sync(0xffffffffu, sh, 31);
    }
}

// the job whose range of a prefix array holds entry i: the last j with prefix[j] <= i
__device__ __forceinline__ int batch_job_of(const int* prefix, int njobs, int i) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct BatchExtendQueue {
    BatchQueues Q;
    int level;   // the level the paths enter
    int cur;     // job of the entry being set up (ray() then root())
    __device__ __forceinline__ void ray(int i, float3& o, float3& d, float& tmin, float& tmax) {
        cur = batch_job_of(Q.ext_prefix, Q.njobs, i);
        const PathRec& p = Q.jobs[cur].paths[level & 1][i - __ldg(Q.ext_prefix + cur)];
        const float4 a = p.o_pb, b = p.d_seed;
        o = make_float3(a.x, a.y, a.z);
        d = make_float3(b.x, b.y, b.z);
        tmin = 0.0f;
        tmax = __int_as_float(0x7f800000);
    }
    __device__ __forceinline__ void root(int, float4& lo, float4& hi, int& root, int& ninst) const {
        const BatchJob& J = Q.jobs[cur];
        lo = J.tlas_lo;
        hi = J.tlas_hi;
        root = J.tlas_root;
        ninst = J.ninst;
    }
    __device__ __forceinline__ bool closest(int i, const Hit& h, float3&, float3&) const {
        const int j = batch_job_of(Q.ext_prefix, Q.njobs, i);
        const BatchJob& J = Q.jobs[j];
        PrimaryRec r;
        r.t = h.t;
        r.u = h.u;
        r.v = h.v;
        r.inst = h.inst >= 0 ? h.inst - J.inst_base : -1;
        r.tri = h.tri;
        r.pad0 = r.pad1 = r.pad2 = 0;
        J.hits[i - __ldg(Q.ext_prefix + j)] = r;
        return false;
    }
    __device__ __forceinline__ void any(int, bool) const {}
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_extend_batch(SceneView s, BatchQueues Q, int level,
                                                                               unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    BatchExtendQueue q{Q, level, 0};
    trace_queue<false, BatchExtendQueue, 1, true>(s, __ldg(Q.ext_prefix + Q.njobs), Q.fetch, q, st, stack);
    flush_stats(st, counters);
}

struct BatchShadowQueue {
    BatchQueues Q;
    int level;
    int cur;
    // the entry's record: sun rays from the front of the job's buffer, light rays from the back
    __device__ __forceinline__ const ShadowRec& rec(int j, int i) const {
        const BatchJob& J = Q.jobs[j];
        const int k = i - __ldg(Q.shd_prefix + j);
        const int nsun = J.level_counts[LEVEL_WORDS * level + 1];
        return J.shadow[k < nsun ? k : J.cap - 1 - (k - nsun)];
    }
    __device__ __forceinline__ void ray(int i, float3& o, float3& d, float& tmin, float& tmax) {
        cur = batch_job_of(Q.shd_prefix, Q.njobs, i);
        const ShadowRec& r = rec(cur, i);
        const float4 a = r.o_tmax, b = r.d_item;
        o = make_float3(a.x, a.y, a.z);
        d = make_float3(b.x, b.y, b.z);
        tmin = 0.0f;
        tmax = a.w;
    }
    __device__ __forceinline__ void root(int, float4& lo, float4& hi, int& root, int& ninst) const {
        const BatchJob& J = Q.jobs[cur];
        lo = J.tlas_lo;
        hi = J.tlas_hi;
        root = J.tlas_root;
        ninst = J.ninst;
    }
    __device__ __forceinline__ bool closest(int, const Hit&, float3&, float3&) const { return false; }
    __device__ __forceinline__ void any(int i, bool occluded) const {
        if (occluded) return;
        const int j = batch_job_of(Q.shd_prefix, Q.njobs, i);
        const ShadowRec& r = rec(j, i);
        const int item = __float_as_int(r.d_item.w);
        const float4 c = r.contrib;
        float4* rad = Q.jobs[j].radiance;
        const float4 L = rad[item];
        rad[item] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
    }
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_shadow_batch(SceneView s, BatchQueues Q, int level,
                                                                               unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    BatchShadowQueue q{Q, level, 0};
    trace_queue<true, BatchShadowQueue, 1, true>(s, __ldg(Q.shd_prefix + Q.njobs), Q.fetch + 1, q, st, stack);
    flush_stats(st, counters ? counters + 8 : nullptr);
}

__global__ void k_merge_nodes(const BvhNode* src, int n, BvhNode* dst, int node_add, int leaf_add) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BvhNode b = src[i];
    b.d.x += b.d.y == 0 ? node_add : leaf_add;
    b.d.z += b.d.w == 0 ? node_add : leaf_add;
    dst[i] = b;
}

__global__ void k_merge_meshes(const MeshRec* src, int n, MeshRec* dst, int node_add, int tri_add) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MeshRec m = src[i];
    if (m.node_root >= 0) m.node_root += node_add;
    m.leaf_first += tri_add;
    m.tri_base += tri_add;
    dst[i] = m;
}

__global__ void k_merge_inst(const InstRec* src, int n, InstRec* dst, int mesh_add) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    InstRec r = src[i];
    r.mesh += mesh_add;
    dst[i] = r;
}

// sky * throughput of every path that left the scene, added to its sample:
// the whole queue (level < 0), or the entries k_shade(level) appended, from
// the end of level - 1's range (the wave's starting length for level 0) to
// the length k_shadow(level) recorded
__global__ void __launch_bounds__(PATH_BLOCK) k_sky_queue(FrameParams F, int level) {
    int i0 = 0, n = F.counts[2];
    if (level >= 0) {
        const int* mark = F.level_counts + 5;
        i0 = mark[LEVEL_WORDS * (level > 0 ? level - 1 : F.max_depth + 1)];
        n = mark[LEVEL_WORDS * level];
    }
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    for (int i = i0 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = F.sky_queue[2 * (size_t)i], b = F.sky_queue[2 * (size_t)i + 1];
        int item = __float_as_int(a.x);
        float3 sk = nishita(P, obs, make_float3(a.y, a.z, a.w));
        float4 L = F.radiance[item];
        F.radiance[item] = make_float4(L.x + sk.x * b.x, L.y + sk.y * b.y, L.z + sk.z * b.z, 0.0f);
    }
}

// The sun's constants in the reference GPU build's arithmetic (fast sine,
// cosine and tangent): its direction, getSunDirection (integrator.cuh:222-230),
// LeSun's threshold (:137) and the disc radius at 1 AU,
// angularDiameterToPhysicalDiameter / 2 (atmosphere.cuh:79-82).
__global__ void k_sun_constants_gpu(float phi, float theta, float diameter, float* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float3 d = normalize(make_float3(cosf(phi) * cosf(theta), sinf(theta), sinf(phi) * cosf(theta)));
    out[0] = d.x;
    out[1] = d.y;
    out[2] = d.z;
    out[3] = cosf(diameter / 2.0f);
    out[4] = (2.0f * 149.597e9f * tanf(diameter / 2.0f)) / 2.0f;
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

// Closest hit / occlusion for a batch of rays.
struct RayBatch {
    const float3 *o, *d;
    float tmin, tmax;
    const float* tmax_each;
    int *inst, *tri;
    float* t;
    float2* uv;
    uint8_t* occ;
    __device__ __forceinline__ void ray(int i, float3& ro, float3& rd, float& t0, float& t1) const {
        ro = o[i];
        rd = d[i];
        t0 = tmin;
        t1 = tmax_each ? tmax_each[i] : tmax;
    }
    __device__ __forceinline__ bool closest(int i, const Hit& h, float3&, float3&) const {
        inst[i] = h.inst;
        tri[i] = h.tri;
        t[i] = h.t;
        if (uv) uv[i] = make_float2(h.u, h.v);
        return false;
    }
    __device__ __forceinline__ void any(int i, bool occluded) const { occ[i] = occluded ? 1 : 0; }
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_trace(SceneView s, int n, const float3* o,
                                                                       const float3* d, float tmin, float tmax,
                                                                       int* inst, int* tri, float* t, float2* uv,
                                                                       int* next, unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    RayBatch q{o, d, tmin, tmax, nullptr, inst, tri, t, uv, nullptr};
    trace_queue<false>(s, n, next, q, st, stack);
    flush_stats(st, counters);
}

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_occluded(SceneView s, int n, const float3* o,
                                                                          const float3* d, float tmin,
                                                                          const float* tmax, uint8_t* out, int* next,
                                                                          unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    RayBatch q{o, d, tmin, 0.0f, tmax, nullptr, nullptr, nullptr, nullptr, out};
    trace_queue<true>(s, n, next, q, st, stack);
    flush_stats(st, counters);
}

// The diffuse bounce of ray i after hit h at bounce b: cosine-weighted about
// the geometric normal facing the incoming ray (Malley's method: a uniform
// unit-disk point rejection-sampled from pairs of PCG draws seeded with
// 4 * ray index + bounce, lifted to the hemisphere, rotated by the Frisvad
// basis), origin offset 1e-3 along the normal; IEEE arithmetic throughout.
__device__ __forceinline__ void diffuse_bounce(const SceneView& s, const Hit& h, float3 ro, float3 rd, int i, int b,
                                               float3* no, float3* nd) {
    const InstRec& ir = s.inst[h.inst];
    const TriShade sh = s.shade[s.meshes[ir.mesh].shade_base + h.tri];
    float3 gn = make_float3(sh.gnx, sh.gny, sh.gnz);
    float3 nn = xnormalize(make_float3(xrow(ir.model[0], gn, 0.0f), xrow(ir.model[1], gn, 0.0f),
                                       xrow(ir.model[2], gn, 0.0f)));
    if (xdot(nn, rd) > 0.0f) nn = make_float3(-nn.x, -nn.y, -nn.z);
    float3 p = make_float3(xa(ro.x, xm(h.t, rd.x)), xa(ro.y, xm(h.t, rd.y)), xa(ro.z, xm(h.t, rd.z)));
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
    *nd = onb_apply_exact(nn, l);
    *no = make_float3(xa(p.x, xm(nn.x, HIT_EPS)), xa(p.y, xm(nn.y, HIT_EPS)), xa(p.z, xm(nn.z, HIT_EPS)));
}

// Bounce chains on the queue traversal: entry i is ray i; after each closest
// hit the lane writes bounce b's hit and continues with the next bounce ray
// (diffuse_bounce), so chains of different lengths share warps.
struct BounceQueue {
    const float3 *o, *d;
    int n, nbounces;
    int *inst, *tri;
    float* t;
    const SceneView* s;
    int b;   // bounce of the chain this lane is tracing
    float3 ro, rd;
    __device__ __forceinline__ void ray(int i, float3& oo, float3& dd, float& tmin, float& tmax) {
        b = 0;
        ro = oo = o[i];
        rd = dd = d[i];
        tmin = 0.0f;
        tmax = __int_as_float(0x7f800000);
    }
    __device__ __forceinline__ bool closest(int i, const Hit& h, float3& no, float3& nd) {
        const size_t k = (size_t)b * n + i;
        inst[k] = h.inst;
        tri[k] = h.tri;
        t[k] = h.t;
        if (h.inst < 0) {
            for (int bb = b + 1; bb <= nbounces; ++bb) {
                const size_t kk = (size_t)bb * n + i;
                inst[kk] = -1;
                tri[kk] = -1;
                t[kk] = __int_as_float(0x7f800000);
            }
            return false;
        }
        if (b == nbounces) return false;
        diffuse_bounce(*s, h, ro, rd, i, b, &no, &nd);
        ++b;
        ro = no;
        rd = nd;
        return true;
    }
    __device__ __forceinline__ void any(int, bool) {}
};

// Closest hit plus `nbounces` diffuse bounces per ray: cosine-weighted about
// the geometric normal facing the incoming ray (Malley's method: a uniform
// unit-disk point, rejection-sampled from pairs of PCG draws seeded with
// 4 * ray index + bounce, lifted to the hemisphere and rotated by the Frisvad
// basis), origin offset 1e-3 along the normal.  IEEE arithmetic throughout,
// so every bounce is bit-identical to the oracle's.  Writes (nbounces+1) x n.
// The chains run on the queue traversal (BounceQueue above).
__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_trace_chains(SceneView s, int n, const float3* o,
                                                                              const float3* d, int nbounces, int* inst,
                                                                              int* tri, float* t, int* next,
                                                                              unsigned long long* counters) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    BounceQueue q{o, d, n, nbounces, inst, tri, t, &s, 0, make_float3(0.0f, 0.0f, 0.0f), make_float3(0.0f, 0.0f, 0.0f)};
    trace_queue<false, BounceQueue, 2>(s, n, next, q, st, stack);
    flush_stats(st, counters);
}

}  // namespace kpt
