// kpt_adjoint.cu -- path-replay adjoint of the plain method (no counterpart in
// the reference).
//
// The differentiated image is, per pixel, the mean over samples of the
// clamped path radiance (what the accumulation adds per frame, before the
// post chain).  For dLoss/dimage given per pixel, the adjoint replays every
// sample's path with the forward's random numbers -- the same camera ray,
// traversal, light sample and BSDF sample as k_shade -- and keeps, per
// vertex, the throughput beta_k, the radiance the vertex adds c_k, the weight
// to the next vertex w_k and their derivatives.  With
// R_k = c_k + w_k R_{k+1} (R after the last vertex: the sky if the path
// escaped), the gradient is sum_k beta_k (dc_k + dw_k R_{k+1}) plus the sky
// terms.  Sampled directions, lobe / light / sun choices, Russian roulette,
// pdfs and MIS weights are held fixed (detached sampling), so the result is
// the derivative of the estimator with respect to the BSDF values (per
// material albedo and roughness) and the sky radiance (Rayleigh r, g, b, Mie,
// both scale heights).  Nothing is stored between the forward and the
// adjoint: each sample is recomputed from its RNG stream.  The replay runs as
// a wavefront (k_adj_shade / k_adj_shadow per level with the forward's
// k_extend, then k_adj_sweep); adjoint_items replays one sample per thread
// and writes the frozen-path records (kpt_adjoint_records_device).
#include "kpt_adjoint.cuh"
#include "kpt_pathfn.cuh"

namespace kpt {

// Gradient slots: material m -> 4 m + (albedo r, g, b, roughness); then the
// sky parameters.  Accumulated per block in shared memory (double), then
// added to the output.
struct GradAcc {
    double* s;
    __device__ __forceinline__ void add(int i, float v) {
        if (v != 0.0f) atomicAdd(s + i, (double)v);
    }
};

__device__ __forceinline__ void grad_begin(double* sg, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) sg[i] = 0.0;
    __syncthreads();
}
__device__ __forceinline__ void grad_end(const double* sg, int n, double* out) {
    __syncthreads();
    if (!out) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (sg[i] != 0.0) atomicAdd(out + i, sg[i]);
}

// g * x per channel, 0 where the weight g is 0 (a clamped channel: its
// derivative terms may be infinite)
__device__ __forceinline__ float3 wmul(float3 g, float3 x) {
    return make_float3(g.x != 0.0f ? g.x * x.x : 0.0f, g.y != 0.0f ? g.y * x.y : 0.0f, g.z != 0.0f ? g.z * x.z : 0.0f);
}
__device__ __forceinline__ float wdot(float3 g, float3 x) {
    const float3 p = wmul(g, x);
    return p.x + p.y + p.z;
}

// clampOutput (color.cuh:295-302) per channel and its derivative mask
__device__ __forceinline__ float clamp_out(float v, float* mask) {
    bool ok = !(isnan(v) || isinf(v));
    *mask = (ok && v >= 0.0f && v <= 1.0e8f) ? 1.0f : 0.0f;
    return ok ? fminf(fmaxf(v, 0.0f), 1.0e8f) : 0.0f;
}

// Texture factors of the material at a hit: albedo (sRGB-decoded texel) and
// roughness (ORM green), 1 without a texture (material.cu:17-70).
struct MatFactors {
    float3 alb_tex;
    float rough_tex, rough_eff;
};
__device__ __forceinline__ MatFactors mat_factors(const SceneView& s, const Surf& si) {
    const MatRec& m = s.materials[si.material];
    MatFactors f;
    f.alb_tex = make_float3(1.0f, 1.0f, 1.0f);
    f.rough_tex = 1.0f;
    if (m.albedo_tex >= 0) {
        float3 t = texture_eval(s, m.albedo_tex, si.uv);
        f.alb_tex = make_float3(srgb_decode(t.x), srgb_decode(t.y), srgb_decode(t.z));
    }
    if (m.orm_tex >= 0) f.rough_tex = texture_eval(s, m.orm_tex, si.uv).y;
    f.rough_eff = m.roughness * f.rough_tex;
    return f;
}

// d(sun radiance)/d(sky parameters): the Nishita radiance towards the sun is
// a per-frame constant (k_sky_constants), so is its Jacobian (in double
// precision, see nishita_jacobian_d).
__global__ void k_adjoint_constants(FrameParams F, AdjParams A) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const SkyParams& P = F.sky;
        float3 J[SKY_PARAMS];
        nishita_jacobian_d(P, make_float3(0.0f, P.earth_r + 1.0f, 0.0f), P.sun_dir, J);
        for (int i = 0; i < SKY_PARAMS; ++i) A.sun_J[i] = J[i];
    }
}

// Sky radiance and its Jacobian for a list of directions (tests and tools):
// out[7 i] = L, out[7 i + 1 + k] = dL/d(sky parameter k).
__global__ void k_sky_grad(SkyParams P, int n, const float3* dirs, float3* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 J[SKY_PARAMS];
    out[7 * (size_t)i] = nishita_grad(P, make_float3(0.0f, P.earth_r + 1.0f, 0.0f), dirs[i], J);
    for (int k = 0; k < SKY_PARAMS; ++k) out[7 * (size_t)i + 1 + k] = J[k];
}

// The double-precision sky Jacobian where the single-precision march is
// ill-conditioned: near the horizon and the sun.
__device__ __forceinline__ bool sky_in_band(const SkyParams& P, float3 d) {
    return fabsf(d.y) < 0.05f || dot(d, P.sun_dir) > 0.995f;
}

// Queues an escape's sky Jacobian (direction d) with its gradient weight w
// in queue q (count, capacity cap); false when there is no queue or it is
// full (the caller evaluates the Jacobian at once).
__device__ __forceinline__ bool sky_push(float4* q, int* count, int cap, float3 d, float3 w) {
    if (!q) return false;
    const int i = atomicAdd(count, 1);
    if (i >= cap) return false;
    q[2 * (size_t)i] = make_float4(d.x, d.y, d.z, 0.0f);
    q[2 * (size_t)i + 1] = make_float4(w.x, w.y, w.z, 0.0f);
    return true;
}
__device__ __forceinline__ bool sky_defer(const AdjParams& A, float3 d, float3 w) {
    return sky_push(A.skyq, A.skyq_count, A.skyq_cap, d, w);
}

// Pixels whose camera ray misses: every sample is sky(d) * LeSun(d).
__global__ void __launch_bounds__(PATH_BLOCK) k_adjoint_miss(FrameParams F, AdjParams A) {
    extern __shared__ double sg[];
    const int ng = 4 * A.nmat + ADJ_SKY_PARAMS;
    grad_begin(sg, ng);
    GradAcc acc{sg};
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const int n = F.counts[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = F.miss_list[i];
        XRay r = camera_ray(F, p % F.W, p / F.W);
        float3 J[SKY_PARAMS];
        const float ls = le_sun(P, r.d);
        float3 L = nishita_grad(P, obs, r.d, J) * ls;
        float3 m;
        float3 Lc = make_float3(clamp_out(L.x, &m.x), clamp_out(L.y, &m.y), clamp_out(L.z, &m.z));
        if (A.image) A.image[p] = make_float4(Lc.x, Lc.y, Lc.z, 0.0f);
        if (!A.adjoint) continue;   // the forward half of a split adjoint: the image only
        const float4 a = A.adjoint[p];
        const float3 g = make_float3(a.x, a.y, a.z) * m * ls;   // mean over identical samples
        bool done = false;
        if (sky_in_band(P, r.d)) {
            done = sky_defer(A, r.d, g);
            if (!done) nishita_jacobian_d(P, obs, r.d, J);
        }
        if (!done)
            for (int k = 0; k < SKY_PARAMS; ++k) acc.add(4 * A.nmat + k, wdot(g, J[k]));
    }
    grad_end(sg, ng, A.grad);
}

// Replay of every (sample, hit pixel) item, one per thread; REC also writes
// each vertex's frozen quantities to A.rec (the records path).
template <bool REC>
__device__ __forceinline__ void adjoint_items(const FrameParams& F, const AdjParams& A, GradAcc& acc, int* stack,
                                              double* gsky) {
    constexpr int MV = ADJ_MAX_VERTICES;
    const SceneView& s = F.scene;
    const SkyParams& P = F.sky;
    const int order = F.rng_order;
    const int nl = s.nlights;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const int nhit = F.counts[0];
    const long long total = (long long)nhit * F.nsamples;
    const float3 sun_rad = *F.sun_radiance;
    TraceStats st = {0, 0, 0, 0};
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
         it += (long long)gridDim.x * blockDim.x) {
        const int item = (int)it;
        const int hj = item / F.nsamples;   // items are pixel-major, as in the forward
        const int ks = item - hj * F.nsamples;
        const int p = F.hit_list[hj];
        const int x = p % F.W, y = p / F.W;
        Sampler S0;
        S0.init(x, y, F.W, F.sample0 + ks);
        S0.get1D();   // BoxFilter::sample, result discarded (kernels.cu:397-402)
        S0.get1D();
        XRay cam = camera_ray(F, x, y);
        float3 o = cam.o, d = cam.d, beta = make_float3(1.0f, 1.0f, 1.0f), prev = make_float3(0.0f, 0.0f, 0.0f);
        float p_b = 1.0f;
        uint32_t seed = S0.seed;
        PrimaryRec h = F.primary[p];
        // per vertex: throughput, added radiance, weight to the next vertex and
        // derivatives (albedo per channel, roughness), radiance per unit sun radiance
        float3 vb[MV], vc[MV], vw[MV], vdca[MV], vdcr[MV], vdwa[MV], vdwr[MV], vcs[MV];
        int vm[MV];
        AdjRec lrec[REC ? MV : 1];
        int nv = 0;
        bool escaped = false;
        float3 s_end = make_float3(0.0f, 0.0f, 0.0f), b_end = s_end, d_end = s_end;
        for (int level = 0;; ++level) {
            if (level > 0) {
                Hit hh = trace_closest(s, make_xray(o, d), 0.0f, __int_as_float(0x7f800000), st, stack);
                h.t = hh.t; h.u = hh.u; h.v = hh.v; h.inst = hh.inst; h.tri = hh.tri;
            }
            if (h.inst < 0) {
                // the sky the path escapes to, by the forward's march; its
                // Jacobian is needed only in the reverse sweep
                escaped = true;
                s_end = nishita(P, obs, d);
                b_end = beta;
                d_end = d;
                break;
            }
            const bool first = level == 0;
            Sampler S;
            S.seed = seed + (uint32_t)level;
            Surf si = surface_at(s, h.inst, h.tri, h.t, h.u, h.v, o, d);
            float3 c = make_float3(0.0f, 0.0f, 0.0f);
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
                c = Le * w_l;
            }
            const float3 emit = c;
            Bsdf bsdf = bsdf_at(s, si);
            const MatFactors mf = mat_factors(s, si);
            // d albedo / d parameter (0 at the demodulated first vertex, bsdf.cuh:286-288)
            const float3 dalb = first ? make_float3(0.0f, 0.0f, 0.0f) : mf.alb_tex;
            if (first) bsdf.albedo = make_float3(1.0f, 1.0f, 1.0f);
            // d alpha / d roughness: alpha = (roughness * texel)^2, then regularised
            float dal = 2.0f * mf.rough_eff * mf.rough_tex;
            if (!first && bsdf.alpha < 0.3f) {
                float a2 = 2.0f * bsdf.alpha;
                dal *= (a2 > 0.1f && a2 < 0.3f) ? 2.0f : 0.0f;
                bsdf.alpha = clampf(2.0f * bsdf.alpha, 0.1f, 0.3f);
            }
            const float3 wo = -d;
            float3 dca = make_float3(0.0f, 0.0f, 0.0f), dcr = dca, cs = dca;
            int nee = 0;
            bool nee_vis = false;
            float3 nwi = dca, nfac = dca;
            float ncos = 0.0f;
            if (!(bsdf.alpha < 0.001f)) {
                if (S.get1D() < 0.5f) {
                    // sampleLdSun
                    const float dsun = 149.597e9f;
                    // rounded product by product, as the forward's shading does
                    const float3 sun_pos = make_float3(__fmul_rn(P.sun_dir.x, dsun), __fmul_rn(P.sun_dir.y, dsun),
                                                       __fmul_rn(P.sun_dir.z, dsun));
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
                    const float3 target = make_float3(__fadd_rn(sun_pos.x, __fmul_rn(off.x, P.sun_radius_m)),
                                                      __fadd_rn(sun_pos.y, __fmul_rn(off.y, P.sun_radius_m)),
                                                      __fadd_rn(sun_pos.z, __fmul_rn(off.z, P.sun_radius_m)));
                    const float cf = fmaxf(0.0f, dot(P.sun_dir, (si.backface ? -1.0f : 1.0f) * si.ng));
                    FGrad fg;
                    float3 fcos = bsdf_f_grad(bsdf, wo, P.sun_dir, fg) * cf;
                    nee = 1;
                    if (nonzero(fcos) && nonzero(sun_rad) && unoccluded(F, si, target, st, stack)) {
                        float area = PI_F * Sqr(P.sun_radius_m);
                        float3 sn = normalize(target - sun_pos), wi = normalize(target - si.pos);
                        float th = AbsDot(sn, -wi);
                        float pdf = (1.0f / area) / (th / Sqr(dsun));
                        const float k = 6.0e5f / pdf / 0.5f;
                        c = c + fcos * sun_rad * k;
                        cs = fcos * k;
                        dca = fg.da * dalb * cf * sun_rad * k;
                        dcr = fg.dal * dal * cf * sun_rad * k;
                        nee_vis = true;
                        nfac = make_float3(k, k, k);
                    }
                    nwi = mul_t(bsdf.basis, P.sun_dir);
                    ncos = cf;
                } else {
                    // sampleLd
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
                        float3 lp = (lt.p0 * bx) + (lt.p1 * by) + (lt.p2 * bz);
                        lp = row3(model, lp, 1.0f);
                        float3 gn = row3(model, lt.gn, 0.0f);
                        float pdf = 1.0f / lt.tri_area;
                        pdf *= Sqr(length(lp - si.pos));
                        pdf /= AbsDot(normalize(lp - si.pos), gn);
                        float3 wi = normalize(lp - si.pos);
                        float3 Lem = emission_of(s, lt.material, luv);
                        nee = 2;
                        if (!(pdf <= 0.0f || !nonzero(Lem))) {
                            const float cf = fmaxf(0.0f, dot(wi, (si.backface ? -1.0f : 1.0f) * si.ng));
                            FGrad fg;
                            float3 fcos = bsdf_f_grad(bsdf, wo, wi, fg) * cf;
                            nwi = mul_t(bsdf.basis, wi);
                            ncos = cf;
                            if (nonzero(fcos) && unoccluded(F, si, lp, st, stack)) {
                                float p_l = prob * pdf;
                                float pb = bsdf.pdf(wo, wi);
                                float w_l = Sqr(p_l) / (Sqr(p_l) + Sqr(pb));
                                const float3 k = Lem * (w_l / p_l / (1.0f - 0.5f));
                                c = c + fcos * k;
                                dca = fg.da * dalb * cf * k;
                                dcr = fg.dal * dal * cf * k;
                                nee_vis = true;
                                nfac = k;
                            }
                        }
                    }
                }
            }
            vb[nv] = beta;
            vc[nv] = c;
            vdca[nv] = dca;
            vdcr[nv] = dcr;
            vcs[nv] = cs;
            vm[nv] = si.material;
            vw[nv] = vdwa[nv] = vdwr[nv] = make_float3(0.0f, 0.0f, 0.0f);
            if (REC) {
                AdjRec& r = lrec[nv];
                r.item = item;
                r.vertex = nv;
                r.material = si.material;
                r.flags = (first ? ADJ_FIRST : 0) | (si.backface ? ADJ_BACKFACE : 0) | (nee_vis ? ADJ_NEE_UNOCCLUDED : 0);
                r.lobe = LOBE_NONE;
                r.nee = nee;
                r.pixel = p;
                r.alb_tex[0] = mf.alb_tex.x; r.alb_tex[1] = mf.alb_tex.y; r.alb_tex[2] = mf.alb_tex.z;
                r.rough_tex = mf.rough_tex;
                r.metallic = bsdf.metallic;
                r.transmission = bsdf.transmission;
                r.ior = bsdf.ior;
                r.eta = 1.0f;
                float3 lwo = mul_t(bsdf.basis, wo);
                r.wo[0] = lwo.x; r.wo[1] = lwo.y; r.wo[2] = lwo.z;
                r.cosw = 0.0f; r.pdf = 0.0f; r.rr = 1.0f;
                r.wi[0] = r.wi[1] = r.wi[2] = r.wm[0] = r.wm[1] = r.wm[2] = 0.0f;
                r.nwi[0] = nwi.x; r.nwi[1] = nwi.y; r.nwi[2] = nwi.z;
                r.ncos = ncos;
                r.nfac[0] = nfac.x; r.nfac[1] = nfac.y; r.nfac[2] = nfac.z;
                r.emit[0] = emit.x; r.emit[1] = emit.y; r.emit[2] = emit.z;
                r.miss[0] = r.miss[1] = r.miss[2] = 0.0f;
                r.pad0 = 0;
                r.pad1 = r.pad2 = r.pad3 = r.pad4 = 0.0f;
            }
            const int vi = nv++;
            if (level == F.max_depth || nv == MV) break;
            float2 uu, X;
            if ((order & RNG_BSDF) == 0) { uu = S.get2D(order); X = S.get2D(order); }
            else { X = S.get2D(order); uu = S.get2D(order); }
            FGrad sg;
            SampleInfo sinfo;
            BsdfSample bs = bsdf_sample_grad(bsdf, wo, uu, X, sg, sinfo);
            if (bs.scatter == SC_ABSORBED || !nonzero(bs.f)) break;
            const float cw = AbsDot(si.ng, bs.wi);
            float3 w = bs.f * cw / bs.pdf;
            float3 dwa = sg.da * dalb * cw / bs.pdf, dwr = sg.dal * dal * cw / bs.pdf;
            beta = beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
            p_b = bsdf.pdf(wo, bs.wi);
            o = (bs.scatter & SC_TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
            float rr = 1.0f;
            bool killed = false;
            float mx = fmaxf(beta.x, fmaxf(beta.y, beta.z));
            if (mx < 1.0f && level >= 1) {
                float q = fmaxf(0.0f, 1.0f - mx);
                if (S.get1D() < q) killed = true;
                else {
                    beta = beta / (1.0f - q);
                    rr = 1.0f / (1.0f - q);
                }
            }
            vw[vi] = w * rr;
            vdwa[vi] = dwa * rr;
            vdwr[vi] = dwr * rr;
            if (REC) {
                AdjRec& r = lrec[vi];
                r.lobe = sinfo.lobe;
                r.eta = sinfo.eta;
                r.wi[0] = sinfo.wi.x; r.wi[1] = sinfo.wi.y; r.wi[2] = sinfo.wi.z;
                r.wm[0] = sinfo.wm.x; r.wm[1] = sinfo.wm.y; r.wm[2] = sinfo.wm.z;
                r.cosw = cw;
                r.pdf = bs.pdf;
                r.rr = killed ? 0.0f : rr;
                r.pad0 = sinfo.tir | (sinfo.inside << 1);
            }
            if (killed || !nonzero(beta)) break;
            prev = si.pos;
            d = bs.wi;
            seed = S.seed;
        }
        // the sample's radiance (the forward's sum), its clamp and the weight
        // dLoss/d(sample) = dLoss/dimage / nsamples on unclamped channels
        float3 L = make_float3(0.0f, 0.0f, 0.0f);
        for (int k = 0; k < nv; ++k) L = L + vb[k] * vc[k];
        if (escaped) L = L + b_end * s_end;
        float3 msk;
        const float3 Lc = make_float3(clamp_out(L.x, &msk.x), clamp_out(L.y, &msk.y), clamp_out(L.z, &msk.z));
        const float inv_n = 1.0f / (float)F.nsamples;
        const float4 a = A.adjoint[p];
        const float3 g = make_float3(a.x, a.y, a.z) * msk * inv_n;
        if (A.image) {
            atomicAdd(&A.image[p].x, Lc.x * inv_n);
            atomicAdd(&A.image[p].y, Lc.y * inv_n);
            atomicAdd(&A.image[p].z, Lc.z * inv_n);
        }
        // reverse sweep: R = radiance from vertex k on, per unit throughput at k
        float3 R = escaped ? s_end : make_float3(0.0f, 0.0f, 0.0f);
        if (nonzero(g)) {
            if (escaped) {
                // The sky Jacobian at the escape: near the sun (Mie forward
                // peak) and the horizon the single-precision march's
                // derivatives are ill-conditioned, so there it is evaluated
                // in double.  Both kinds are queued for batched kernels
                // (k_adjoint_sky_d / _f), which march on full warps instead
                // of the few lanes of a warp that escape together here.
                const float3 gb = wmul(g, b_end);
                const bool band = sky_in_band(P, d_end);
                const bool done = band ? sky_defer(A, d_end, gb)
                                       : sky_push(A.skyqf, A.skyqf_count, A.skyqf_cap, d_end, gb);
                if (!done) {
                    float3 J_end[SKY_PARAMS];
                    if (band) nishita_jacobian_d(P, obs, d_end, J_end);
                    else nishita_grad(P, obs, d_end, J_end);
                    for (int i = 0; i < SKY_PARAMS; ++i) gsky[i] += wdot(gb, J_end[i]);
                }
            }
            for (int k = nv - 1; k >= 0; --k) {
                const float3 gb = wmul(g, vb[k]);
                const float3 ta = wmul(gb, vdca[k] + wmul(vdwa[k], R));
                const int m4 = 4 * vm[k];
                acc.add(m4 + 0, ta.x);
                acc.add(m4 + 1, ta.y);
                acc.add(m4 + 2, ta.z);
                acc.add(m4 + 3, wdot(gb, vdcr[k] + wmul(vdwr[k], R)));
                if (nonzero(vcs[k])) {
                    const float3 gs = wmul(gb, vcs[k]);
                    for (int i = 0; i < SKY_PARAMS; ++i) gsky[i] += wdot(gs, A.sun_J[i]);
                }
                R = vc[k] + vw[k] * R;
            }
        }
        if (REC && nv > 0) {
            lrec[nv - 1].flags |= ADJ_LAST | (escaped ? ADJ_ESCAPED : 0);
            lrec[nv - 1].miss[0] = d_end.x;
            lrec[nv - 1].miss[1] = d_end.y;
            lrec[nv - 1].miss[2] = d_end.z;
            const int base = atomicAdd(A.rec_count, nv);
            for (int k = 0; k < nv; ++k) {
                lrec[k].g[0] = g.x;
                lrec[k].g[1] = g.y;
                lrec[k].g[2] = g.z;
                if (base + k < A.max_rec) A.rec[base + k] = lrec[k];
            }
        }
    }
}

template <bool REC>
__device__ __forceinline__ void adjoint_block(const FrameParams& F, const AdjParams& A) {
    extern __shared__ double sg[];
    const int ng = 4 * A.nmat + ADJ_SKY_PARAMS;
    grad_begin(sg, ng);
    GradAcc acc{sg};
    int stack[STACK_WORDS];
    double gsky[SKY_PARAMS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    adjoint_items<REC>(F, A, acc, stack, gsky);
    for (int i = 0; i < SKY_PARAMS; ++i) {   // one shared add per warp per sky parameter
        double v = gsky[i];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(sg + 4 * A.nmat + i, v);
    }
    grad_end(sg, ng, A.grad);
}


// The deferred sky Jacobians: weight . J(d) per queued escape, summed into
// the sky parameters' gradients; in double (DBL, the band near the horizon
// and the sun) or single precision.
template <bool DBL>
__device__ __forceinline__ void sky_jacobians(const FrameParams& F, const float4* q, const int* count, int cap,
                                              double* grad) {
    __shared__ double sg[SKY_PARAMS];
    if (threadIdx.x < SKY_PARAMS) sg[threadIdx.x] = 0.0;
    __syncthreads();
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const int n = min(*count, cap);
    double gsky[SKY_PARAMS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = q[2 * (size_t)i], b = q[2 * (size_t)i + 1];
        float3 J[SKY_PARAMS];
        if (DBL) nishita_jacobian_s(P, obs, make_float3(a.x, a.y, a.z), J);
        else nishita_grad(P, obs, make_float3(a.x, a.y, a.z), J);
        const float3 w = make_float3(b.x, b.y, b.z);
        for (int k = 0; k < SKY_PARAMS; ++k) gsky[k] += wdot(w, J[k]);
    }
    for (int k = 0; k < SKY_PARAMS; ++k) {
        double v = gsky[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(sg + k, v);
    }
    __syncthreads();
    if (threadIdx.x < SKY_PARAMS && sg[threadIdx.x] != 0.0) atomicAdd(grad + threadIdx.x, sg[threadIdx.x]);
}

__global__ void __launch_bounds__(PATH_BLOCK) k_adjoint_sky_d(FrameParams F, AdjParams A) {
    sky_jacobians<true>(F, A.skyq, A.skyq_count, A.skyq_cap, A.grad + 4 * A.nmat);
}
__global__ void __launch_bounds__(PATH_BLOCK) k_adjoint_sky_f(FrameParams F, AdjParams A) {
    sky_jacobians<false>(F, A.skyqf, A.skyqf_count, A.skyqf_cap, A.grad + 4 * A.nmat);
}
__global__ void __launch_bounds__(PATH_BLOCK) k_adjoint_rec(FrameParams F, AdjParams A) { adjoint_block<true>(F, A); }

// ---------------------------------------------------------------------------
// The wavefront replay (kpt_adjoint_device): the estimator of adjoint_items
// with its rays traced by the forward's queue kernels.  Per level,
// k_adj_shade runs the replay's vertex for every path of the wave (emission
// with its MIS weight, the light sample and its derivatives, the BSDF sample
// and its derivatives, Russian roulette) and stores the vertex record; the
// light sample's shadow ray goes to k_adj_shadow, which marks the sample
// visible; k_extend traces the continuations.  After the last level
// k_adj_sweep sums each sample's radiance and runs its reverse sweep.  The
// arithmetic of every vertex is adjoint_items' (the records megakernel, kept
// for the frozen-path records).

__device__ __forceinline__ float3 xyz3(float4 v) { return make_float3(v.x, v.y, v.z); }

__global__ void __launch_bounds__(PATH_BLOCK, 6) k_adj_shade(FrameParams F, AdjParams A, int level, long long wave0) {
    constexpr int MV = ADJ_MAX_VERTICES;
    const SceneView& s = F.scene;
    const SkyParams& P = F.sky;
    const int order = F.rng_order;
    const int nl = s.nlights;
    const bool first = level == 0;
    const float3 sun_rad = *F.sun_radiance;
    const int cap = F.cap;
    int n;
    if (first) {
        const long long left = (long long)F.counts[0] * F.nsamples - wave0;
        n = (int)(left < 0 ? 0 : (left < cap ? left : cap));
    } else {
        n = F.level_counts[LEVEL_WORDS * level];
    }
    const PathRec* in = F.paths[level & 1];
    PathRec* out = F.paths[(level + 1) & 1];
    int* here = F.level_counts + LEVEL_WORDS * level;
    int* next = F.level_counts + LEVEL_WORDS * (level + 1);
    if (first && blockIdx.x == 0 && threadIdx.x == 0) here[0] = n;   // read back by kpt_get_level_counts
    float4* const vr0 = A.vr + (size_t)level * cap * AV_FIELDS;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float3 o, d, beta, prev;
        float p_b;
        uint32_t seed;
        int loc;   // the path's slot in the wave
        PrimaryRec h;
        if (first) {
            const long long item = wave0 + i;   // pixel-major, as in the forward
            const int hj = (int)(item / F.nsamples);
            const int k = (int)(item - (long long)hj * F.nsamples);
            const int p = F.hit_list[hj];
            const int x = p % F.W, y = p / F.W;
            Sampler S0;
            S0.init(x, y, F.W, F.sample0 + k);
            S0.get1D();   // BoxFilter::sample, result discarded (kernels.cu:397-402)
            S0.get1D();
            const XRay cam = camera_ray(F, x, y);
            o = cam.o;
            d = cam.d;
            beta = make_float3(1.0f, 1.0f, 1.0f);
            prev = make_float3(0.0f, 0.0f, 0.0f);
            p_b = 1.0f;
            seed = S0.seed;
            h = F.primary[p];
            loc = i;
        } else {
            const PathRec pr = in[i];
            o = make_float3(pr.o_pb.x, pr.o_pb.y, pr.o_pb.z);
            p_b = pr.o_pb.w;
            d = make_float3(pr.d_seed.x, pr.d_seed.y, pr.d_seed.z);
            seed = __float_as_uint(pr.d_seed.w);
            beta = make_float3(pr.beta_item.x, pr.beta_item.y, pr.beta_item.z);
            loc = __float_as_int(pr.beta_item.w);
            prev = make_float3(pr.prev.x, pr.prev.y, pr.prev.z);
            h = F.hits[i];
        }
        auto end_path = [&](bool escaped, int nv, float3 de, float3 be) {
            A.vend[2 * (size_t)loc] = make_float4(de.x, de.y, de.z, __int_as_float(nv));
            A.vend[2 * (size_t)loc + 1] = make_float4(be.x, be.y, be.z, __int_as_float(escaped ? 1 : 0));
        };
        if (h.inst < 0) {   // the path leaves the scene: k_adj_sky evaluates the sky
            end_path(true, level, d, beta);
            A.esc[group_append(A.esc_count)] = loc;
            continue;
        }
        Sampler S;
        S.seed = seed + (uint32_t)level;
        Surf si = surface_at(s, h.inst, h.tri, h.t, h.u, h.v, o, d);
        float3 c = make_float3(0.0f, 0.0f, 0.0f);
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
            c = Le * w_l;
        }
        Bsdf bsdf = bsdf_at(s, si);
        const MatFactors mf = mat_factors(s, si);
        const float3 dalb = first ? make_float3(0.0f, 0.0f, 0.0f) : mf.alb_tex;
        if (first) bsdf.albedo = make_float3(1.0f, 1.0f, 1.0f);
        float dal = 2.0f * mf.rough_eff * mf.rough_tex;
        if (!first && bsdf.alpha < 0.3f) {
            float a2 = 2.0f * bsdf.alpha;
            dal *= (a2 > 0.1f && a2 < 0.3f) ? 2.0f : 0.0f;
            bsdf.alpha = clampf(2.0f * bsdf.alpha, 0.1f, 0.3f);
        }
        const float3 wo = -d;
        const float3 zero = make_float3(0.0f, 0.0f, 0.0f);
        float3 fcos = zero, kk = zero, dat = zero, dalt = zero;
        int nee = 0;   // 1: sun, 2: area light, with a shadow ray sent
        if (!(bsdf.alpha < 0.001f)) {
            // the light sample: each branch sets up its direction, the BSDF
            // and its derivatives are evaluated once for the warp
            const bool sun = S.get1D() < 0.5f;
            const float dsun = 149.597e9f;
            const float3 sun_pos = make_float3(__fmul_rn(P.sun_dir.x, dsun), __fmul_rn(P.sun_dir.y, dsun),
                                               __fmul_rn(P.sun_dir.z, dsun));
            float3 wi = P.sun_dir, target = sun_pos, Lem = zero;
            float pdf = 0.0f, prob = 0.0f;
            bool eval = false;
            if (sun) {
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
                target = make_float3(__fadd_rn(sun_pos.x, __fmul_rn(off.x, P.sun_radius_m)),
                                     __fadd_rn(sun_pos.y, __fmul_rn(off.y, P.sun_radius_m)),
                                     __fadd_rn(sun_pos.z, __fmul_rn(off.z, P.sun_radius_m)));
                eval = true;
            } else {
                float X = S.get1D();
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
                    float3 lp = (lt.p0 * bx) + (lt.p1 * by) + (lt.p2 * bz);
                    lp = row3(model, lp, 1.0f);
                    float3 gn = row3(model, lt.gn, 0.0f);
                    pdf = 1.0f / lt.tri_area;
                    pdf *= Sqr(length(lp - si.pos));
                    pdf /= AbsDot(normalize(lp - si.pos), gn);
                    wi = normalize(lp - si.pos);
                    Lem = emission_of(s, lt.material, luv);
                    target = lp;
                    eval = !(pdf <= 0.0f || !nonzero(Lem));
                }
            }
            float cf = 0.0f;
            FGrad fg;
            float3 fc = zero;
            if (eval) {
                cf = fmaxf(0.0f, dot(wi, (si.backface ? -1.0f : 1.0f) * si.ng));
                fc = bsdf_f_grad(bsdf, wo, wi, fg) * cf;
            }
            if (eval && nonzero(fc) && (!sun || nonzero(sun_rad))) {
                if (sun) {
                    float area = PI_F * Sqr(P.sun_radius_m);
                    float3 sn = normalize(target - sun_pos), wt = normalize(target - si.pos);
                    float th = AbsDot(sn, -wt);
                    float spdf = (1.0f / area) / (th / Sqr(dsun));
                    const float k = 6.0e5f / spdf / 0.5f;
                    kk = make_float3(k, k, k);
                    nee = 1;
                } else {
                    float p_l = prob * pdf;
                    float pb = bsdf.pdf(wo, wi);
                    float w_l = Sqr(p_l) / (Sqr(p_l) + Sqr(pb));
                    kk = Lem * (w_l / p_l / (1.0f - 0.5f));
                    nee = 2;
                }
                fcos = fc;
                dat = fg.da * dalb * cf;
                dalt = fg.dal * dal * cf;
                // the shadow ray of Integrator::unoccluded (integrator.cuh:124-131)
                const float3 so = si.backface ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
                const float3 sd = normalize(target - so);
                const float tmax = length(target - so) - 0.11f;
                // sun rays from the front of the buffer, light rays from the
                // back (one append per kind: the group shares one counter)
                int j;
                if (nee == 1) j = group_append(here + 1);
                else j = cap - 1 - group_append(here + 2);
                ShadowRec r;
                r.o_tmax = make_float4(so.x, so.y, so.z, tmax);
                r.d_item = make_float4(sd.x, sd.y, sd.z, __int_as_float(loc));
                r.contrib = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                F.shadow[j] = r;
            }
        }
        vr0[(size_t)loc * AV_FIELDS + AV_BETA] = make_float4(beta.x, beta.y, beta.z, __int_as_float(si.material));
        vr0[(size_t)loc * AV_FIELDS + AV_EMIT] = make_float4(c.x, c.y, c.z, __int_as_float(nee));
        vr0[(size_t)loc * AV_FIELDS + AV_FCOS] = make_float4(fcos.x, fcos.y, fcos.z, 0.0f);
        vr0[(size_t)loc * AV_FIELDS + AV_K] = make_float4(kk.x, kk.y, kk.z, 0.0f);
        vr0[(size_t)loc * AV_FIELDS + AV_DA] = make_float4(dat.x, dat.y, dat.z, 0.0f);
        vr0[(size_t)loc * AV_FIELDS + AV_DAL] = make_float4(dalt.x, dalt.y, dalt.z, 0.0f);
        const int nv = level + 1;
        float3 w = zero, dwa = zero, dwr = zero;
        bool go = false;
        if (level < F.max_depth && nv < MV) {
            float2 uu, X;
            if ((order & RNG_BSDF) == 0) { uu = S.get2D(order); X = S.get2D(order); }
            else { X = S.get2D(order); uu = S.get2D(order); }
            FGrad sg;
            SampleInfo sinfo;
            BsdfSample bs = bsdf_sample_grad(bsdf, wo, uu, X, sg, sinfo);
            if (!(bs.scatter == SC_ABSORBED || !nonzero(bs.f))) {
                const float cw = AbsDot(si.ng, bs.wi);
                w = bs.f * cw / bs.pdf;
                dwa = sg.da * dalb * cw / bs.pdf;
                dwr = sg.dal * dal * cw / bs.pdf;
                beta = beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
                p_b = bsdf.pdf(wo, bs.wi);
                o = (bs.scatter & SC_TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
                float rr = 1.0f;
                bool killed = false;
                float mx = fmaxf(beta.x, fmaxf(beta.y, beta.z));
                if (mx < 1.0f && level >= 1) {
                    float q = fmaxf(0.0f, 1.0f - mx);
                    if (S.get1D() < q) killed = true;
                    else {
                        beta = beta / (1.0f - q);
                        rr = 1.0f / (1.0f - q);
                    }
                }
                w = w * rr;
                dwa = dwa * rr;
                dwr = dwr * rr;
                go = !(killed || !nonzero(beta));
                d = bs.wi;
            }
        }
        vr0[(size_t)loc * AV_FIELDS + AV_W] = make_float4(w.x, w.y, w.z, 0.0f);
        vr0[(size_t)loc * AV_FIELDS + AV_DWA] = make_float4(dwa.x, dwa.y, dwa.z, 0.0f);
        vr0[(size_t)loc * AV_FIELDS + AV_DWR] = make_float4(dwr.x, dwr.y, dwr.z, 0.0f);
        if (!go) {
            end_path(false, nv, zero, zero);
            continue;
        }
        const int j = group_append(next);
        PathRec pr;
        pr.o_pb = make_float4(o.x, o.y, o.z, p_b);
        pr.d_seed = make_float4(d.x, d.y, d.z, __uint_as_float(S.seed));
        pr.beta_item = make_float4(beta.x, beta.y, beta.z, __int_as_float(loc));
        pr.prev = make_float4(si.pos.x, si.pos.y, si.pos.z, 0.0f);
        out[j] = pr;
    }
}

// The replay's shadow rays of `level`: an unoccluded ray marks its vertex's
// light sample visible.
struct AdjShadowQueue {
    const ShadowRec* rec;
    unsigned char* vis;
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
        if (!occluded) vis[__float_as_int(rec[slot(i)].d_item.w)] = 1;
    }
};

__global__ void __launch_bounds__(TRACE_BLOCK, TRACE_MIN_BLOCKS) k_adj_shadow(FrameParams F, AdjParams A, int level) {
    int stack[STACK_WORDS];
    TraceStats st = {0, 0, 0, 0};
    int* lc = F.level_counts + LEVEL_WORDS * level;
    AdjShadowQueue q{F.shadow, A.vis + (size_t)level * F.cap, lc[1], F.cap};
    trace_queue<true>(F.scene, lc[1] + lc[2], lc + 4, q, st, stack);
}

// An escape's sky Jacobian evaluated where it occurs (its queue is full):
// weight . J added to the block's sky gradient slots.
static __device__ __noinline__ void sky_jacobian_now(const SkyParams& P, float3 obs, float3 d, bool band, float3 w,
                                                     double* slots) {
    float3 J[SKY_PARAMS];
    if (band) nishita_jacobian_d(P, obs, d, J);
    else nishita_grad(P, obs, d, J);
    for (int q = 0; q < SKY_PARAMS; ++q) atomicAdd(slots + q, (double)wdot(w, J[q]));
}

// The sky radiance at the end of every escaped path of the wave (the
// forward's march), for k_adj_sweep.
__global__ void __launch_bounds__(PATH_BLOCK) k_adj_sky(FrameParams F, AdjParams A, long long) {
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const int n = *A.esc_count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int i = A.esc[q];
        const float3 s = nishita(P, obs, xyz3(A.vend[2 * (size_t)i]));
        A.vsky[i] = make_float4(s.x, s.y, s.z, 0.0f);
    }
}

// Every sample of the wave: its radiance from the vertex records (the
// forward's sum), clamp, image, and the reverse sweep into the gradients.
// the sweep and the vertex replay are held to 64 and 85 registers: left to
// 193 and 110 they keep 8 and 16 warps per SM on latency-bound loads (the
// sweep's spills cost less than the warps it gains)
__global__ void __launch_bounds__(PATH_BLOCK, 8) k_adj_sweep(FrameParams F, AdjParams A, long long wave0) {
    extern __shared__ double sg[];
    const int ng = 4 * A.nmat + ADJ_SKY_PARAMS;
    grad_begin(sg, ng);
    GradAcc acc{sg};
    double gsky[SKY_PARAMS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    // the sun light samples' weights, summed: their sky gradient is linear in
    // the sun's Jacobian, applied once at the end
    double cs0 = 0.0, cs1 = 0.0, cs2 = 0.0;
    const SkyParams& P = F.sky;
    const float3 obs = make_float3(0.0f, P.earth_r + 1.0f, 0.0f);
    const float3 sun_rad = *F.sun_radiance;
    const int cap = F.cap;
    const int nhit = F.counts[0];
    const long long left = (long long)nhit * F.nsamples - wave0;
    const int n = (int)(left < 0 ? 0 : (left < cap ? left : cap));
    const float inv_n = 1.0f / (float)F.nsamples;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long item = wave0 + i;
        const int p = F.hit_list[item / F.nsamples];
        const float4 e0 = A.vend[2 * (size_t)i], e1 = A.vend[2 * (size_t)i + 1];
        const int nv = __float_as_int(e0.w);
        const bool escaped = __float_as_int(e1.w) != 0;
        const float3 d_end = xyz3(e0), b_end = xyz3(e1);
        const float3 s_end = escaped ? xyz3(A.vsky[i]) : make_float3(0.0f, 0.0f, 0.0f);
        // c of vertex k: its emission, plus its light sample where visible
        auto vertex_c = [&](int k, float4 emit, bool* vis_nee) {
            const float3 c = xyz3(emit);
            const int nee = __float_as_int(emit.w);
            *vis_nee = nee != 0 && A.vis[(size_t)k * cap + i] != 0;
            if (!*vis_nee) return c;
            const float3 fcos = xyz3(A.vr[((size_t)k * cap + i) * AV_FIELDS + AV_FCOS]);
            const float3 kk = xyz3(A.vr[((size_t)k * cap + i) * AV_FIELDS + AV_K]);
            return nee == 1 ? c + fcos * sun_rad * kk.x : c + fcos * kk;
        };
        // the path's radiance: summed over its vertices, or (the backward
        // half of a split adjoint) as the forward half stored it
        float3 L = make_float3(0.0f, 0.0f, 0.0f);
        if (A.lpath_ready) {
            L = xyz3(A.lpath[i]);
        } else {
#pragma unroll 1
            for (int k = 0; k < nv; ++k) {
                bool v;
                const float3 b = xyz3(A.vr[((size_t)k * cap + i) * AV_FIELDS + AV_BETA]);
                L = L + b * vertex_c(k, A.vr[((size_t)k * cap + i) * AV_FIELDS + AV_EMIT], &v);
            }
            if (escaped) L = L + b_end * s_end;
            if (A.lpath) A.lpath[i] = make_float4(L.x, L.y, L.z, 0.0f);
        }
        float3 msk;
        const float3 Lc = make_float3(clamp_out(L.x, &msk.x), clamp_out(L.y, &msk.y), clamp_out(L.z, &msk.z));
        if (A.image) {
            atomicAdd(&A.image[p].x, Lc.x * inv_n);
            atomicAdd(&A.image[p].y, Lc.y * inv_n);
            atomicAdd(&A.image[p].z, Lc.z * inv_n);
        }
        if (!A.adjoint) continue;   // the forward half of a split adjoint: the image only
        const float4 a = A.adjoint[p];
        const float3 g = make_float3(a.x, a.y, a.z) * msk * inv_n;
        if (!nonzero(g)) continue;
        float3 R = escaped ? s_end : make_float3(0.0f, 0.0f, 0.0f);
        if (escaped) {
            const float3 gb = wmul(g, b_end);
            const bool band = sky_in_band(P, d_end);
            const bool done = band ? sky_defer(A, d_end, gb)
                                   : sky_push(A.skyqf, A.skyqf_count, A.skyqf_cap, d_end, gb);
            if (!done) sky_jacobian_now(P, obs, d_end, band, gb, sg + 4 * A.nmat);
        }
#pragma unroll 1
        for (int k = nv - 1; k >= 0; --k) {
            const size_t o = (size_t)k * cap + i;
            const float4 b4 = A.vr[o * AV_FIELDS + AV_BETA];
            bool v;
            const float3 ck = vertex_c(k, A.vr[o * AV_FIELDS + AV_EMIT], &v);
            float3 dca = make_float3(0.0f, 0.0f, 0.0f), dcr = dca, cs = dca;
            if (v) {
                const int nee = __float_as_int(A.vr[o * AV_FIELDS + AV_EMIT].w);
                const float3 kk = xyz3(A.vr[o * AV_FIELDS + AV_K]);
                const float3 da = xyz3(A.vr[o * AV_FIELDS + AV_DA]), dl = xyz3(A.vr[o * AV_FIELDS + AV_DAL]);
                if (nee == 1) {
                    dca = da * sun_rad * kk.x;
                    dcr = dl * sun_rad * kk.x;
                    cs = xyz3(A.vr[o * AV_FIELDS + AV_FCOS]) * kk.x;
                } else {
                    dca = da * kk;
                    dcr = dl * kk;
                }
            }
            const float3 gb = wmul(g, xyz3(b4));
            const float3 dwa = xyz3(A.vr[o * AV_FIELDS + AV_DWA]), dwr = xyz3(A.vr[o * AV_FIELDS + AV_DWR]);
            const float3 ta = wmul(gb, dca + wmul(dwa, R));
            const int m4 = 4 * __float_as_int(b4.w);
            acc.add(m4 + 0, ta.x);
            acc.add(m4 + 1, ta.y);
            acc.add(m4 + 2, ta.z);
            acc.add(m4 + 3, wdot(gb, dcr + wmul(dwr, R)));
            if (nonzero(cs)) {
                const float3 gs = wmul(gb, cs);
                cs0 += gs.x;
                cs1 += gs.y;
                cs2 += gs.z;
            }
            R = ck + xyz3(A.vr[o * AV_FIELDS + AV_W]) * R;
        }
    }
    if (!A.adjoint) return;   // uniform over the block: the image only, no gradient
    for (int q = 0; q < SKY_PARAMS; ++q) {   // one shared add per warp per sky parameter
        const float3 J = A.sun_J[q];
        double v = gsky[q] + cs0 * J.x + cs1 * J.y + cs2 * J.z;
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(sg + 4 * A.nmat + q, v);
    }
    grad_end(sg, ng, A.grad);
}

}  // namespace kpt
