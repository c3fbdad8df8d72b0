// kpt_shade.cuh -- unified BSDF, lights and the Nishita sky on the device.
//
// Follows shaders/bsdf.cuh (GGX, Fresnel, UnifiedBSDF), shaders/light.cu,
// shaders/light_sampler.cuh, shaders/triangle.cuh:104-122 (area light
// sampling), shaders/material.cu:17-70 and shaders/atmosphere.cuh:30-311.
// Arithmetic is the reference GPU build's (fast maths).  Where the reference
// evaluates a float expression with a double literal (GGX D), it is kept in
// double.
#pragma once
#include "kpt_device.cuh"

// KPT_BSDF_CALL: the BSDF's f / pdf / sample are compiled as one out-of-line
// copy each (the shading kernel calls f and pdf twice per vertex; inlined it
// is large enough to stall on instruction fetch: measured 4.34 -> 3.72 ms per
// 1080p16 frame); KPT_BSDF_INLINE inlines them at every call site
#ifdef KPT_BSDF_INLINE
#define KPT_BSDF_CALL __forceinline__
#else
#define KPT_BSDF_CALL __noinline__
#endif

namespace kpt {

struct M3 { float3 c0, c1, c2; };   // column-major 3x3

__device__ __forceinline__ float3 mul(const M3& m, float3 v) {
    return make_float3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z,
                       m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
                       m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
// transpose(m) * v
__device__ __forceinline__ float3 mul_t(const M3& m, float3 v) {
    return make_float3(m.c0.x * v.x + m.c0.y * v.y + m.c0.z * v.z,
                       m.c1.x * v.x + m.c1.y * v.y + m.c1.z * v.z,
                       m.c2.x * v.x + m.c2.y * v.y + m.c2.z * v.z);
}
// generateONBFrisvad (maths/matrix_maths.cuh:375-396)
__device__ __forceinline__ M3 onb_frisvad(float3 n) {
    M3 r;
    if (n.z < -0.999805696f) {
        r.c0 = make_float3(0.0f, -1.0f, 0.0f);
        r.c1 = make_float3(-1.0f, 0.0f, 0.0f);
    } else {
        float a = 1.0f / (1.0f + n.z);
        float b = -n.x * n.y * a;
        r.c0 = make_float3(1.0f - n.x * n.x * a, b, -n.x);
        r.c1 = make_float3(b, 1.0f - n.y * n.y * a, -n.y);
    }
    r.c2 = n;
    return r;
}

// ---------------------------------------------------------------------------
// GGX (bsdf.cuh:18-88)

__device__ __forceinline__ float ggx_D(float alpha, float3 wm) {
    float a = alpha;
    if (alpha < 0.001f) a = fmaxf(a, 1.0e-3f);
    float a2 = Sqr(a);
    float ndh = Sqr(saturatef_(wm.z));
    float b = (float)((double)ndh * ((double)a2 - 1.0) + 1.0);
    return a2 / (PI_F * Sqr(b));
}
__device__ __forceinline__ float ggx_G(float alpha, float3 wo, float3 wi) {
    float nv = fmaxf(wo.z, 0.0f);
    float nl = fabsf(wi.z);
    float tv = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nv));
    float tl = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nl));
    return ((2.0f * nv) / (nv + tv)) * ((2.0f * nl) / (nl + tl));
}
__device__ __forceinline__ float3 ggx_sample_wm(float alpha, float2 u) {
    float a2 = Sqr(alpha);
    float theta = acosf(sqrtf((1.0f - u.x) / ((a2 - 1.0f) * u.x + 1.0f)));
    float phi = 2.0f * PI_F * u.y;
    float st = sinf(theta);
    return normalize(make_float3(st * cosf(phi), st * sinf(phi), cosf(theta)));
}

__device__ __forceinline__ float fresnel_dielectric(float c, float ior) {  // bsdf.cuh:122-141
    c = clampf(c, -1.0f, 1.0f);
    if (c < 0.0f) { ior = 1.0f / ior; c = -c; }
    float s2 = 1.0f - c * c;
    float s2t = s2 / (ior * ior);
    if (s2t >= 1.0f) return 1.0f;
    float ct = sqrtf(1.0f - s2t);
    float rp = (ior * c - ct) / (ior * c + ct);
    float rs = (c - ior * ct) / (c + ior * ct);
    return (rp * rp + rs * rs) * 0.5f;
}
__device__ __forceinline__ float microfacet_brdf(float alpha, float3 wo, float3 wi, float3 wm) {  // bsdf.cuh:151-164
    float nv = saturatef_(wo.z), nl = saturatef_(wi.z);
    float f = (ggx_D(alpha, wm) * ggx_G(alpha, wo, wi)) / (4.0f * fmaxf(nv, 1.0e-3f) * nl);
    if (wi.z <= 0.0f || dot(wi, wm) <= 0.0f) f = 0.0f;
    return f;
}
__device__ __forceinline__ bool refract3(float3 wi, float3 n, float ior, float3* wt) {  // vector_maths.cuh:46-65
    float c = dot(wi, n);
    if (c < 0.0f) { ior = 1.0f / ior; c *= -1.0f; n = n * -1.0f; }
    float s2 = 1.0f - c * c;
    float s2t = s2 / (ior * ior);
    if (s2t >= 1.0f) return false;
    float ct = sqrtf(1.0f - s2t);
    *wt = (-1.0f * wi) / ior + (c / ior - ct) * n;
    return true;
}

enum { SC_ABSORBED = 0, SC_REFLECTED = 2, SC_TRANSMITTED = 4, SC_DIFFUSE = 8, SC_GLOSSY = 16 };

struct BsdfSample { int scatter; float3 f, wi; float pdf; };

struct Bsdf {   // UnifiedBSDF (bsdf.cuh:166-624)
    M3 basis;
    float3 albedo;
    float alpha, metallic, transmission, ior;
    bool backface;

    __device__ __forceinline__ float pdf_glossy(float3 wo, float3 wm) const {
        float voh = fmaxf(dot(wo, wm), 0.0f);
        float noh = fmaxf(wm.z, 0.0f);
        return (ggx_D(alpha, wm) * noh) / (4.0f * voh);
    }
    __device__ __forceinline__ float f_glossy(float3 wo, float3 wi, float3 wm) const {
        return fresnel_dielectric(dot(wo, wm), ior) * microfacet_brdf(alpha, wo, wi, wm);
    }
    __device__ __forceinline__ float3 f_opaque(float3 wo, float3 wi) const {
        float3 wm = normalize(wo + wi);
        float g = f_glossy(wo, wi, wm);
        float fd = ((wo.z * wi.z > 0) ? 1.0f : 0.0f) * INV_PI_F;
        return make_float3(1.0f - g, 1.0f - g, 1.0f - g) * (albedo * fd) + make_float3(g, g, g);
    }
    __device__ __forceinline__ float pdf_opaque(float3 wo, float3 wi) const {
        float3 wm = normalize(wo + wi);
        return 0.5f * (pdf_glossy(wo, wm) + wi.z * INV_PI_F);
    }
    __device__ __forceinline__ float3 f_conductor(float3 wo, float3 wi) const {
        float3 wm = normalize(wo + wi);
        float nv = clampf(wo.z, 0.0f, 1.0f), nl = clampf(wi.z, 0.0f, 1.0f);
        if (nv == 0.0f || nl == 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
        float voh = clampf(dot(wo, wm), 0.0f, 1.0f);
        float3 M = make_float3(0.0f, 0.0f, 0.0f);
        if (nl > 0.0f && voh > 0.0f) {
            float p5 = 1.0f - voh;
            p5 = p5 * p5 * p5 * p5 * p5;
            float3 F = albedo + (make_float3(1.0f, 1.0f, 1.0f) - albedo) * p5;
            F = make_float3(clampf(F.x, 0.0f, 1.0f), clampf(F.y, 0.0f, 1.0f), clampf(F.z, 0.0f, 1.0f));
            M = F * microfacet_brdf(alpha, wo, wi, wm);
        }
        return M;
    }
    __device__ __forceinline__ float btdf_pdf(float3 wo, float3 wi, float3 ht, float eta) const {
        float temp = dot(wi, ht) * eta + dot(wo, ht);
        float dwm = AbsDot(wi, ht) / (temp * temp);
        float F = fresnel_dielectric(AbsDot(wo, ht), eta);
        return (ggx_D(alpha, ht) * fabsf(ht.z)) * dwm * (1.0f - F);
    }
    __device__ __forceinline__ float3 btdf_f(float3 wo, float3 wi, float3 ht, float eta) const {
        float temp = dot(wi, ht) * eta + dot(wo, ht);
        float F = fresnel_dielectric(AbsDot(wo, ht), eta);
        float T = ggx_D(alpha, ht) * ggx_G(alpha, wo, wi) * fabsf(dot(wi, ht) * dot(wo, ht) / (wi.z * wo.z * temp * temp));
        return (albedo * (1.0f - F)) * T;
    }
    __device__ __forceinline__ float3 f_transparent(float3 wo, float3 wi) const {
        float co = wo.z, ci = wi.z;
        bool refl = (co * ci) > 0.0f;
        float eta = 1.0f;
        if (!refl) eta = !backface ? ior : (1.0f / ior);
        float3 wm = eta * wi + wo;
        wm = normalize((wm.z > 0) ? wm : -wm);
        if ((dot(wm, wi) * ci < 0.0f) || (dot(wm, wo) * co < 0.0f)) return make_float3(0.0f, 0.0f, 0.0f);
        float F = fresnel_dielectric(fabsf(dot(wo, wm)), ior);
        if (refl) {
            float v = F * microfacet_brdf(alpha, wo, wi, wm);
            return make_float3(v, v, v);
        }
        float temp = dot(wi, wm) * eta + dot(wo, wm);
        float dwm = fabsf(dot(wi, wm)) * fabsf(dot(wo, wm)) / (temp * temp);
        float Tss = ggx_D(alpha, wm) * ggx_G(alpha, wo, wi) * dwm / (fabsf(ci * co));
        return ((1.0f - F) * albedo) * Tss;
    }
    __device__ __forceinline__ float pdf_transparent(float3 wo, float3 wi) const {
        float co = wo.z, ci = wi.z;
        bool refl = co * ci > 0.0f;
        float eta = 1.0f;
        if (!refl) eta = !backface ? ior : 1.0f / ior;
        float3 wm = eta * wi + wo;
        wm = normalize((wm.z > 0) ? wm : -wm);
        if (dot(wm, wi) * ci < 0.0f || dot(wm, wo) * co < 0.0f) return 0.0f;
        float F = fresnel_dielectric(fabsf(dot(wo, wm)), ior);
        if (refl) return pdf_glossy(wo, wm) * F;
        float temp = dot(wi, wm) + dot(wo, wm) / eta;
        float dwm = fabsf(dot(wo, wm)) / (temp * temp);
        return ggx_D(alpha, wm) * fmaxf(wm.z, 0.0f) * dwm * (1.0f - F);
    }

    // UnifiedBSDF::f (bsdf.cuh:191-216)
    __device__ KPT_BSDF_CALL float3 f(float3 w_wo, float3 w_wi) const {
        float3 wo = mul_t(basis, w_wo), wi = mul_t(basis, w_wi);
        float wt = (1.0f - metallic) * transmission;
        float wd = (1.0f - metallic) * (1.0f - transmission);
        float3 F = make_float3(0.0f, 0.0f, 0.0f);
        if (metallic > 0.0f) F = F + f_conductor(wo, wi) * metallic;
        if (wt > 0.0f) F = F + f_transparent(wo, wi) * wt;
        if (wd > 0.0f) F = F + f_opaque(wo, wi) * wd;
        return F;
    }
    // UnifiedBSDF::pdf (bsdf.cuh:218-241)
    __device__ KPT_BSDF_CALL float pdf(float3 w_wo, float3 w_wi) const {
        float3 wi = mul_t(basis, w_wi), wo = mul_t(basis, w_wo);
        float wt = (1.0f - metallic) * transmission;
        float wd = (1.0f - metallic) * (1.0f - transmission);
        float p = 0.0f;
        if (metallic > 0.0f) p += metallic * pdf_glossy(wo, normalize(wo + wi));
        if (wt > 0.0f) p += wt * pdf_transparent(wo, wi);
        if (wd > 0.0f) p += wd * pdf_opaque(wo, wi);
        return p;
    }
    // UnifiedBSDF::sampleF (bsdf.cuh:243-268) with the three lobe samplers
    __device__ KPT_BSDF_CALL BsdfSample sample(float3 w_wo, float2 u, float2 X) const {
        float3 wo = mul_t(basis, w_wo);
        BsdfSample bs;
        bs.scatter = SC_ABSORBED;
        bs.f = make_float3(0.0f, 0.0f, 0.0f);
        bs.wi = make_float3(0.0f, 0.0f, 0.0f);
        bs.pdf = 0.0f;
        float pt = (1.0f - metallic) * transmission;
        if (X.x < metallic) {                         // sampleConductor
            float3 wm = ggx_sample_wm(alpha, u);
            float3 wi = reflect3(-wo, wm);
            bs.scatter = SC_GLOSSY | SC_REFLECTED;
            bs.f = f_conductor(wo, wi);
            bs.wi = wi;
            bs.pdf = pdf_glossy(wo, wm);
        } else if (X.x < pt) {                        // sampleTransparentDielectric
            bool inside = backface;
            float eta = inside ? (1.0f / ior) : ior;
            float3 ht = ggx_sample_wm(alpha, u);
            float3 wi = make_float3(0.0f, 0.0f, 0.0f);
            bool tir = !refract3(wo, ht, eta, &wi);
            if ((X.y < 0.5f && !inside) || (tir && inside)) {
                wi = reflect3(-wo, ht);
                if ((wi.z * wo.z) > 0.0f) {
                    float v = fresnel_dielectric(dot(wo, ht), eta) * microfacet_brdf(alpha, wo, wi, ht);
                    if (!tir) v = v * 2.0f;
                    bs.scatter = SC_REFLECTED | SC_GLOSSY;
                    bs.f = make_float3(v, v, v);
                    bs.wi = wi;
                    bs.pdf = pdf_glossy(wo, ht);
                }
            } else if (!(tir || (wi.z * wo.z) > 0.0f || wi.z == 0.0f)) {
                float3 f = btdf_f(wo, wi, ht, eta);
                if (!inside) f = f * 2.0f;
                bs.scatter = SC_TRANSMITTED | SC_GLOSSY;
                bs.f = f;
                bs.wi = wi;
                bs.pdf = btdf_pdf(wo, wi, ht, eta);
            }
        } else if (X.y < 0.5f) {                      // sampleOpaqueDielectric, glossy
            float3 wm = ggx_sample_wm(alpha, u);
            float3 wi = reflect3(-wo, wm);
            float v = f_glossy(wo, wi, wm) * 2.0f;
            bs.scatter = SC_GLOSSY | SC_REFLECTED;
            bs.f = make_float3(v, v, v);
            bs.wi = wi;
            bs.pdf = pdf_glossy(wo, wm);
        } else {                                      // sampleOpaqueDielectric, diffuse
            float phi = 2.0f * PI_F * u.x;
            float ct = sqrtf(u.y), st = sqrtf(1.0f - u.y);
            float3 wi = make_float3(st * cosf(phi), st * sinf(phi), ct);
            float fd = ((wo.z * wi.z > 0) ? 1.0f : 0.0f) * INV_PI_F;
            bs.scatter = SC_DIFFUSE | SC_REFLECTED;
            bs.f = (albedo * fd) * 2.0f;
            bs.wi = wi;
            bs.pdf = wi.z * INV_PI_F;
        }
        bs.wi = mul(basis, bs.wi);
        return bs;
    }
};

// ---------------------------------------------------------------------------
// textures (shaders/texture.cuh:34-66)

__device__ __forceinline__ float3 texture_eval(const SceneView& s, int id, float2 uv) {
    const TexRec t = s.textures[id];
    if (t.offset < 0 || t.offset >= s.npixels) return make_float3(0.0f, 0.0f, 0.0f);
    long long px = t.ch, row = (long long)t.w * px;
    float sx = uv.x - floorf(uv.x), sy = uv.y - floorf(uv.y);
    int x = (int)(sx * t.w) % t.w, y = (int)(sy * t.h) % t.h;
    if (x < 0) x += t.w;
    if (y < 0) y += t.h;
    long long off = (long long)y * row + (long long)x * px;
    if (off + 3 >= s.npixels) return make_float3(0.0f, 0.0f, 0.0f);
    const uint8_t* p = s.pixels + t.offset + off;
    const float k = 0.00392156862f;
    return make_float3(p[0] * k, p[1] * k, p[2] * k);
}
__device__ __forceinline__ float srgb_decode(float v) {
    return (v <= 0.04045f) ? (v / 12.92f) : powf((v + 0.055f) / (1 + 0.055f), 2.4f);
}

// ---------------------------------------------------------------------------
// Nishita single scattering (shaders/atmosphere.cuh:30-223)

// The geometry of the sky model works with vectors of length ~6.4e6 m, where
// one float ulp is 0.5 m of altitude and a 1 m altitude error is 1e-3 of Mie
// density (scale height 1200 m).  It therefore runs in IEEE arithmetic
// without contraction; the exponentials use the fast exp and their arguments
// the reciprocal scale heights (relative error ~1e-6 for these arguments,
// like the reference's fast-math division).
__device__ __forceinline__ bool sphere_hit(float3 o, float3 d, float radius, float* t0, float* t1) {
    float3 oc = make_float3(-o.x, -o.y, -o.z);
    float a = xdot(d, d);
    float b = xm(-2.0f, xdot(d, oc));
    float c = xs(xdot(oc, oc), xm(radius, radius));
    float disc = xs(xm(b, b), xm(xm(4.0f, a), c));
    if (disc < 0.0f) return false;
    float sq = __fsqrt_rn(disc);
    float a2 = xm(2.0f, a);
    float x0 = __fdiv_rn(xs(-b, sq), a2), x1 = __fdiv_rn(xa(-b, sq), a2);
    if (x0 > x1) { float t = x0; x0 = x1; x1 = t; }
    *t0 = x0;
    *t1 = x1;
    return !(x1 < 0.0f);
}

__device__ __forceinline__ float3 xpoint(float3 o, float t, float3 d) {
    return make_float3(xa(o.x, xm(t, d.x)), xa(o.y, xm(t, d.y)), xa(o.z, xm(t, d.z)));
}

// The same model in the arithmetic of the reference's GPU build: plain
// single-precision operators under fast maths (approximate square root,
// division and exponential, contracted products), written with the
// reference's expression structure (intersectSphere, atmosphere.cuh:30-57;
// sampleLi, :132-223) so that the compiler forms the same operations.  Its
// altitudes carry that build's rounding (one ulp of a ~6.4e6 m length is
// 0.5 m), so its sky agrees with that build's rather than with IEEE
// arithmetic.
__device__ __forceinline__ bool sphere_hit_gpu(float3 o, float3 d, float radius, float* t0, float* t1) {
    float3 oc = make_float3(0.0f - o.x, 0.0f - o.y, 0.0f - o.z);
    float a = dot(d, d);
    float b = -2.0f * dot(d, oc);
    float c = dot(oc, oc) - Sqr(radius);
    float disc = Sqr(b) - 4.0f * a * c;
    if (disc < 0.0f) return false;
    float sq = sqrtf(disc);
    *t0 = (-b - sq) / (2.0f * a);
    *t1 = (-b + sq) / (2.0f * a);
    if (*t0 > *t1) {
        float t = *t0;
        *t0 = *t1;
        *t1 = t;
    }
    return !(*t1 < 0.0f);
}

static __device__ __noinline__ float3 nishita_gpu(const SkyParams& P, float3 o, float3 d) {
    float tmin = 0.0f, tmax = __int_as_float(0x7f800000);
    {
        float te, tx;
        if (!sphere_hit_gpu(o, d, P.atm_r, &te, &tx) || tx < 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
        if (te > tmin && te > 0.0f) tmin = te;
        if (tx < tmax) tmax = tx;
    }
    const float depth = tmax - tmin;
    const float step = depth / 16.0f;
    float t = tmin;
    float3 iR = make_float3(0.0f, 0.0f, 0.0f), iM = make_float3(0.0f, 0.0f, 0.0f);
    float oR = 0.0f, oM = 0.0f;
    const float3 tR = make_float3(P.sigma_r.x + 0.0f, P.sigma_r.y + 0.0f, P.sigma_r.z + 0.0f);
    const float tM = P.sigma_m + P.sigma_am;
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        const float3 sp = o + ((t + (step * 0.5f)) * d);
        const float alt = length(sp) - P.earth_r;
        const float pR = expf(-alt / P.h_r) * step;
        const float pM = expf(-alt / P.h_m) * step;
        oR += pR;
        oM += pM;
        float lte, ltx;
        sphere_hit_gpu(sp, P.sun_dir, P.atm_r, &lte, &ltx);
        const float lstep = ltx / 8.0f;
        float lt = 0.0f, lR = 0.0f, lM = 0.0f;
        int j;
#pragma unroll
        for (j = 0; j < 8; ++j) {
            const float3 spl = sp + ((lt + (lstep * 0.5f)) * P.sun_dir);
            const float altl = length(spl) - P.earth_r;
            if (altl < 0.0f) break;
            lR += expf(-altl / P.h_r) * lstep;
            lM += expf(-altl / P.h_m) * lstep;
            lt += lstep;
        }
        if (j == 8) {
            const float sr = oR + lR, sm = oM + lM;
            const float3 tau = make_float3(tR.x * sr + tM * sm, tR.y * sr + tM * sm, tR.z * sr + tM * sm);
            const float3 Tr = make_float3(expf(-tau.x), expf(-tau.y), expf(-tau.z));
            iR += Tr * pR;
            iM += Tr * pM;
        }
        t += step;
    }
    float mu = dot(d, P.sun_dir);
    float rp = (3.0f * (1.0f + Sqr(mu))) / (16.0f * PI_F);
    const float g = 0.76f;
    float den = (8.0f * PI_F) * ((2.0f + Sqr(g)) * powf(1.0f + Sqr(g) - 2.0f * g * mu, 1.5f));
    float mp = 3.0f * ((1.0f - Sqr(g)) * (1.0f + Sqr(mu))) / den;
    float3 L = P.sigma_r * iR * rp + make_float3(P.sigma_m, P.sigma_m, P.sigma_m) * iM * mp;
    return L * 6.0e5f * P.sun_emission;
}

// Radiance of the sky seen from `o` along `d`, in the arithmetic the frame
// selects (P.gpu_arith).
static __device__ __noinline__ float3 nishita(const SkyParams& P, float3 o, float3 d) {
    if (P.gpu_arith) return nishita_gpu(P, o, d);
    float tmin = 0.0f, tmax = __int_as_float(0x7f800000);
    {
        float te, tx;
        if (!sphere_hit(o, d, P.atm_r, &te, &tx) || tx < 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
        if (te > tmin && te > 0.0f) tmin = te;
        if (tx < tmax) tmax = tx;
    }
    const float step = xm(xs(tmax, tmin), 0.0625f);   // exact: / 16
    const float3 tR = make_float3(xa(P.sigma_r.x, 0.0f), xa(P.sigma_r.y, 0.0f), xa(P.sigma_r.z, 0.0f));
    const float tM = xa(P.sigma_m, P.sigma_am);
    const float half = xm(step, 0.5f);
    float t = tmin;
    float3 iR = make_float3(0.0f, 0.0f, 0.0f), iM = make_float3(0.0f, 0.0f, 0.0f);
    float oR = 0.0f, oM = 0.0f;
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        float3 sp = xpoint(o, xa(t, half), d);
        float alt = xs(__fsqrt_rn(xdot(sp, sp)), P.earth_r);
        float pR = xm(expf(-alt * P.inv_h_r), step);
        float pM = xm(expf(-alt * P.inv_h_m), step);
        oR = xa(oR, pR);
        oM = xa(oM, pM);
        float lte, ltx;
        sphere_hit(sp, P.sun_dir, P.atm_r, &lte, &ltx);
        float lstep = xm(ltx, 0.125f);   // exact: / 8
        float lhalf = xm(lstep, 0.5f);
        float lt = 0.0f, lR = 0.0f, lM = 0.0f;
        int j;
#pragma unroll
        for (j = 0; j < 8; ++j) {
            float3 spl = xpoint(sp, xa(lt, lhalf), P.sun_dir);
            float altl = xs(__fsqrt_rn(xdot(spl, spl)), P.earth_r);
            if (altl < 0.0f) break;
            lR = xa(lR, xm(expf(-altl * P.inv_h_r), lstep));
            lM = xa(lM, xm(expf(-altl * P.inv_h_m), lstep));
            lt = xa(lt, lstep);
        }
        if (j == 8) {
            float sr = xa(oR, lR), sm = xa(oM, lM);
            float tmm = xm(tM, sm);
            float3 tau = make_float3(xa(xm(tR.x, sr), tmm), xa(xm(tR.y, sr), tmm), xa(xm(tR.z, sr), tmm));
            float3 Tr = make_float3(expf(-tau.x), expf(-tau.y), expf(-tau.z));
            iR = make_float3(xa(iR.x, xm(Tr.x, pR)), xa(iR.y, xm(Tr.y, pR)), xa(iR.z, xm(Tr.z, pR)));
            iM = make_float3(xa(iM.x, xm(Tr.x, pM)), xa(iM.y, xm(Tr.y, pM)), xa(iM.z, xm(Tr.z, pM)));
        }
        t = xa(t, step);
    }
    float mu = dot(d, P.sun_dir);
    float rp = (3.0f * (1.0f + Sqr(mu))) / (16.0f * PI_F);
    const float g = 0.76f;
    float den = (8.0f * PI_F) * ((2.0f + Sqr(g)) * powf(1.0f + Sqr(g) - 2.0f * g * mu, 1.5f));
    float mp = 3.0f * ((1.0f - Sqr(g)) * (1.0f + Sqr(mu))) / den;
    float3 L = P.sigma_r * iR * rp + make_float3(P.sigma_m, P.sigma_m, P.sigma_m) * iM * mp;
    return L * 6.0e5f * P.sun_emission;
}

}  // namespace kpt
