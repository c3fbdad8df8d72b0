// kpt_adjoint.cuh -- derivatives of the BSDF and the sky for the path-replay
// adjoint (no counterpart in the reference).
//
// Every function returns the same value as its forward counterpart in
// kpt_shade.cuh (same operations) plus its derivatives:
//   * with respect to the albedo, per channel: every lobe of the unified BSDF
//     (bsdf.cuh:166-624) is affine in the albedo channel by channel (Schlick F0,
//     Lambert, the BTDF's (1 - F) * albedo), so d f_c / d albedo_c is exact;
//   * with respect to alpha (= roughness^2 after texturing and
//     regularisation): through GGX D and the separable Smith G
//     (bsdf.cuh:18-57), the only places alpha enters f;
//   * of the Nishita sky (atmosphere.cuh:132-223) with respect to the Rayleigh
//     coefficients (r, g, b), the Mie coefficient and the two scale heights,
//     by forward-mode differentiation of its 16 x 8-step march.
#pragma once
#include "kpt_shade.cuh"

namespace kpt {

// GGX D and dD/dalpha (ggx_D).
__device__ __forceinline__ float ggx_D_grad(float alpha, float3 wm, float* dD) {
    float a = alpha;
    const bool floor = alpha < 0.001f;
    if (floor) a = fmaxf(a, 1.0e-3f);
    float a2 = Sqr(a);
    float ndh = Sqr(saturatef_(wm.z));
    float b = (float)((double)ndh * ((double)a2 - 1.0) + 1.0);
    float D = a2 / (PI_F * Sqr(b));
    // dD/da2 = (b - 2 a2 ndh) / (pi b^3); a2 = alpha^2 unless floored
    *dD = floor ? 0.0f : ((b - 2.0f * a2 * ndh) / (PI_F * b * b * b)) * (2.0f * a);
    return D;
}

// separable Smith G and dG/dalpha (ggx_G)
__device__ __forceinline__ float ggx_G_grad(float alpha, float3 wo, float3 wi, float* dG) {
    float nv = fmaxf(wo.z, 0.0f);
    float nl = fabsf(wi.z);
    float tv = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nv));
    float tl = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nl));
    float gv = (2.0f * nv) / (nv + tv), gl = (2.0f * nl) / (nl + tl);
    // d t/d alpha = alpha (1 - n^2) / t;  d g/d alpha = -2 n / (n + t)^2 * dt
    float dtv = tv > 0.0f ? alpha * (1.0f - Sqr(nv)) / tv : 0.0f;
    float dtl = tl > 0.0f ? alpha * (1.0f - Sqr(nl)) / tl : 0.0f;
    float dgv = (nv + tv) > 0.0f ? -2.0f * nv / Sqr(nv + tv) * dtv : 0.0f;
    float dgl = (nl + tl) > 0.0f ? -2.0f * nl / Sqr(nl + tl) * dtl : 0.0f;
    *dG = dgv * gl + gv * dgl;
    return gv * gl;
}

// microfacet_brdf and its derivative
__device__ __forceinline__ float micro_grad(float alpha, float3 wo, float3 wi, float3 wm, float* dm) {
    float nv = saturatef_(wo.z), nl = saturatef_(wi.z);
    float dD, dG;
    float D = ggx_D_grad(alpha, wm, &dD), G = ggx_G_grad(alpha, wo, wi, &dG);
    float den = 4.0f * fmaxf(nv, 1.0e-3f) * nl;
    float f = (D * G) / den;
    float d = (dD * G + D * dG) / den;
    if (wi.z <= 0.0f || dot(wi, wm) <= 0.0f) f = d = 0.0f;
    *dm = d;
    return f;
}

// Derivatives of one BSDF evaluation: da (per albedo channel) and dal (alpha).
struct FGrad {
    float3 da, dal;
};

__device__ __forceinline__ float3 conductor_grad(const Bsdf& b, float3 wo, float3 wi, FGrad& g) {
    g.da = g.dal = make_float3(0.0f, 0.0f, 0.0f);
    float3 wm = normalize(wo + wi);
    float nv = clampf(wo.z, 0.0f, 1.0f), nl = clampf(wi.z, 0.0f, 1.0f);
    if (nv == 0.0f || nl == 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
    float voh = clampf(dot(wo, wm), 0.0f, 1.0f);
    float3 M = make_float3(0.0f, 0.0f, 0.0f);
    if (nl > 0.0f && voh > 0.0f) {
        float p5 = 1.0f - voh;
        p5 = p5 * p5 * p5 * p5 * p5;
        float3 F = b.albedo + (make_float3(1.0f, 1.0f, 1.0f) - b.albedo) * p5;
        float3 dF = make_float3(F.x > 0.0f && F.x < 1.0f ? 1.0f - p5 : 0.0f, F.y > 0.0f && F.y < 1.0f ? 1.0f - p5 : 0.0f,
                                F.z > 0.0f && F.z < 1.0f ? 1.0f - p5 : 0.0f);
        F = make_float3(clampf(F.x, 0.0f, 1.0f), clampf(F.y, 0.0f, 1.0f), clampf(F.z, 0.0f, 1.0f));
        float dm;
        float m = micro_grad(b.alpha, wo, wi, wm, &dm);
        M = F * m;
        g.da = dF * m;
        g.dal = F * dm;
    }
    return M;
}

__device__ __forceinline__ float3 opaque_grad(const Bsdf& b, float3 wo, float3 wi, FGrad& g) {
    float3 wm = normalize(wo + wi);
    float dm;
    float fr = fresnel_dielectric(dot(wo, wm), b.ior);
    float gl = fr * micro_grad(b.alpha, wo, wi, wm, &dm);
    float dgl = fr * dm;
    float fd = ((wo.z * wi.z > 0) ? 1.0f : 0.0f) * INV_PI_F;
    g.da = make_float3(1.0f - gl, 1.0f - gl, 1.0f - gl) * fd;
    g.dal = (make_float3(1.0f, 1.0f, 1.0f) - b.albedo * fd) * dgl;
    return make_float3(1.0f - gl, 1.0f - gl, 1.0f - gl) * (b.albedo * fd) + make_float3(gl, gl, gl);
}

__device__ __forceinline__ float3 transparent_grad(const Bsdf& b, float3 wo, float3 wi, FGrad& g) {
    g.da = g.dal = make_float3(0.0f, 0.0f, 0.0f);
    float co = wo.z, ci = wi.z;
    bool refl = (co * ci) > 0.0f;
    float eta = 1.0f;
    if (!refl) eta = !b.backface ? b.ior : (1.0f / b.ior);
    float3 wm = eta * wi + wo;
    wm = normalize((wm.z > 0) ? wm : -wm);
    if ((dot(wm, wi) * ci < 0.0f) || (dot(wm, wo) * co < 0.0f)) return make_float3(0.0f, 0.0f, 0.0f);
    float F = fresnel_dielectric(fabsf(dot(wo, wm)), b.ior);
    if (refl) {
        float dm;
        float v = F * micro_grad(b.alpha, wo, wi, wm, &dm);
        g.dal = make_float3(F * dm, F * dm, F * dm);
        return make_float3(v, v, v);
    }
    float temp = dot(wi, wm) * eta + dot(wo, wm);
    float dwm = fabsf(dot(wi, wm)) * fabsf(dot(wo, wm)) / (temp * temp);
    float dD, dG;
    float D = ggx_D_grad(b.alpha, wm, &dD), G = ggx_G_grad(b.alpha, wo, wi, &dG);
    float Tss = D * G * dwm / (fabsf(ci * co));
    float dT = (dD * G + D * dG) * dwm / (fabsf(ci * co));
    g.da = make_float3(1.0f - F, 1.0f - F, 1.0f - F) * Tss;
    g.dal = ((1.0f - F) * b.albedo) * dT;
    return ((1.0f - F) * b.albedo) * Tss;
}

// UnifiedBSDF::f with derivatives
__device__ __forceinline__ float3 bsdf_f_grad(const Bsdf& b, float3 w_wo, float3 w_wi, FGrad& g) {
    float3 wo = mul_t(b.basis, w_wo), wi = mul_t(b.basis, w_wi);
    float wt = (1.0f - b.metallic) * b.transmission;
    float wd = (1.0f - b.metallic) * (1.0f - b.transmission);
    float3 F = make_float3(0.0f, 0.0f, 0.0f);
    g.da = g.dal = make_float3(0.0f, 0.0f, 0.0f);
    FGrad l;
    if (b.metallic > 0.0f) {
        F = F + conductor_grad(b, wo, wi, l) * b.metallic;
        g.da = g.da + l.da * b.metallic;
        g.dal = g.dal + l.dal * b.metallic;
    }
    if (wt > 0.0f) {
        F = F + transparent_grad(b, wo, wi, l) * wt;
        g.da = g.da + l.da * wt;
        g.dal = g.dal + l.dal * wt;
    }
    if (wd > 0.0f) {
        F = F + opaque_grad(b, wo, wi, l) * wd;
        g.da = g.da + l.da * wd;
        g.dal = g.dal + l.dal * wd;
    }
    return F;
}

// The sampled lobe and its local geometry (for the frozen-path records).
enum { LOBE_NONE = 0, LOBE_CONDUCTOR, LOBE_T_REFLECT, LOBE_T_TRANSMIT, LOBE_O_GLOSSY, LOBE_O_DIFFUSE };
struct SampleInfo {
    int lobe, tir, inside;
    float eta;
    float3 wo, wi, wm;   // local frame
};

// UnifiedBSDF::sampleF (Bsdf::sample) with the derivatives of the sampled
// lobe's f at the sampled direction (the direction itself is held fixed).
__device__ __forceinline__ BsdfSample bsdf_sample_grad(const Bsdf& b, float3 w_wo, float2 u, float2 X, FGrad& g,
                                                       SampleInfo& info) {
    float3 wo = mul_t(b.basis, w_wo);
    info.lobe = LOBE_NONE;
    info.tir = info.inside = 0;
    info.eta = 1.0f;
    info.wo = wo;
    info.wi = info.wm = make_float3(0.0f, 0.0f, 0.0f);
    BsdfSample bs;
    bs.scatter = SC_ABSORBED;
    bs.f = make_float3(0.0f, 0.0f, 0.0f);
    bs.wi = make_float3(0.0f, 0.0f, 0.0f);
    bs.pdf = 0.0f;
    g.da = g.dal = make_float3(0.0f, 0.0f, 0.0f);
    float pt = (1.0f - b.metallic) * b.transmission;
    if (X.x < b.metallic) {                         // sampleConductor
        float3 wm = ggx_sample_wm(b.alpha, u);
        float3 wi = reflect3(-wo, wm);
        bs.scatter = SC_GLOSSY | SC_REFLECTED;
        bs.f = conductor_grad(b, wo, wi, g);
        bs.wi = wi;
        bs.pdf = b.pdf_glossy(wo, wm);
        info.lobe = LOBE_CONDUCTOR;
        info.wi = wi;
        info.wm = wm;
    } else if (X.x < pt) {                          // sampleTransparentDielectric
        bool inside = b.backface;
        float eta = inside ? (1.0f / b.ior) : b.ior;
        float3 ht = ggx_sample_wm(b.alpha, u);
        float3 wi = make_float3(0.0f, 0.0f, 0.0f);
        bool tir = !refract3(wo, ht, eta, &wi);
        info.tir = tir;
        info.inside = inside;
        info.eta = eta;
        info.wm = ht;
        if ((X.y < 0.5f && !inside) || (tir && inside)) {
            wi = reflect3(-wo, ht);
            if ((wi.z * wo.z) > 0.0f) {
                float dm;
                float fr = fresnel_dielectric(dot(wo, ht), eta);
                float v = fr * micro_grad(b.alpha, wo, wi, ht, &dm);
                float dv = fr * dm;
                if (!tir) {
                    v = v * 2.0f;
                    dv = dv * 2.0f;
                }
                bs.scatter = SC_REFLECTED | SC_GLOSSY;
                bs.f = make_float3(v, v, v);
                g.dal = make_float3(dv, dv, dv);
                bs.wi = wi;
                bs.pdf = b.pdf_glossy(wo, ht);
                info.lobe = LOBE_T_REFLECT;
                info.wi = wi;
            }
        } else if (!(tir || (wi.z * wo.z) > 0.0f || wi.z == 0.0f)) {
            // btdf_f with derivatives
            float temp = dot(wi, ht) * eta + dot(wo, ht);
            float F = fresnel_dielectric(AbsDot(wo, ht), eta);
            float dD, dG;
            float D = ggx_D_grad(b.alpha, ht, &dD), G = ggx_G_grad(b.alpha, wo, wi, &dG);
            float k = fabsf(dot(wi, ht) * dot(wo, ht) / (wi.z * wo.z * temp * temp));
            float T = D * G * k, dT = (dD * G + D * dG) * k;
            float3 f = (b.albedo * (1.0f - F)) * T;
            float3 da = make_float3(1.0f - F, 1.0f - F, 1.0f - F) * T;
            float3 dal = (b.albedo * (1.0f - F)) * dT;
            if (!inside) {
                f = f * 2.0f;
                da = da * 2.0f;
                dal = dal * 2.0f;
            }
            bs.scatter = SC_TRANSMITTED | SC_GLOSSY;
            bs.f = f;
            g.da = da;
            g.dal = dal;
            bs.wi = wi;
            bs.pdf = b.btdf_pdf(wo, wi, ht, eta);
            info.lobe = LOBE_T_TRANSMIT;
            info.wi = wi;
        }
    } else if (X.y < 0.5f) {                        // sampleOpaqueDielectric, glossy
        float3 wm = ggx_sample_wm(b.alpha, u);
        float3 wi = reflect3(-wo, wm);
        float dm;
        float fr = fresnel_dielectric(dot(wo, wm), b.ior);
        float v = fr * micro_grad(b.alpha, wo, wi, wm, &dm) * 2.0f;
        bs.scatter = SC_GLOSSY | SC_REFLECTED;
        bs.f = make_float3(v, v, v);
        g.dal = make_float3(fr * dm * 2.0f, fr * dm * 2.0f, fr * dm * 2.0f);
        bs.wi = wi;
        bs.pdf = b.pdf_glossy(wo, wm);
        info.lobe = LOBE_O_GLOSSY;
        info.wi = wi;
        info.wm = wm;
    } else {                                        // sampleOpaqueDielectric, diffuse
        float phi = 2.0f * PI_F * u.x;
        float ct = sqrtf(u.y), st = sqrtf(1.0f - u.y);
        float3 wi = make_float3(st * cosf(phi), st * sinf(phi), ct);
        float fd = ((wo.z * wi.z > 0) ? 1.0f : 0.0f) * INV_PI_F;
        bs.scatter = SC_DIFFUSE | SC_REFLECTED;
        bs.f = (b.albedo * fd) * 2.0f;
        g.da = make_float3(fd * 2.0f, fd * 2.0f, fd * 2.0f);
        bs.wi = wi;
        bs.pdf = wi.z * INV_PI_F;
        info.lobe = LOBE_O_DIFFUSE;
        info.wi = wi;
    }
    bs.wi = mul(b.basis, bs.wi);
    return bs;
}

// a * b per channel, 0 where a is 0: a transmittance that underflowed to 0
// (the optical depth of a march through the earth is infinite) has
// derivative 0, whatever the optical depth's derivative is
__device__ __forceinline__ float3 zmul(float3 a, float3 b) {
    return make_float3(a.x != 0.0f ? a.x * b.x : 0.0f, a.y != 0.0f ? a.y * b.y : 0.0f, a.z != 0.0f ? a.z * b.z : 0.0f);
}

// Sky parameters the adjoint differentiates, in this order.
enum { SKY_RAYLEIGH_R = 0, SKY_RAYLEIGH_G, SKY_RAYLEIGH_B, SKY_MIE, SKY_RAYLEIGH_H, SKY_MIE_H, SKY_PARAMS };

// The Jacobian of the sky in double precision (one evaluation per frame: the
// radiance towards the sun).  At the sun the Rayleigh derivatives are a
// near-cancellation of terms ~30x larger than the result, where the single-
// precision march's own error (~1e-4 of the value) would show as percent-level
// error; the value itself stays the single-precision nishita() the forward
// uses.
struct D3 { double x, y, z; };
__device__ __forceinline__ D3 d3(float3 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ bool sphere_hit_d(D3 o, D3 d, double radius, double* t0, double* t1) {
    double a = ddot(d, d), b = 2.0 * ddot(d, o), c = ddot(o, o) - radius * radius;
    double disc = b * b - 4.0 * a * c;
    if (disc < 0.0) return false;
    double sq = sqrt(disc);
    double x0 = (-b - sq) / (2.0 * a), x1 = (-b + sq) / (2.0 * a);
    if (x0 > x1) { double t = x0; x0 = x1; x1 = t; }
    *t0 = x0;
    *t1 = x1;
    return !(x1 < 0.0);
}
static __device__ __noinline__ void nishita_jacobian_d(const SkyParams& P, float3 of, float3 df, float3* J) {
    for (int i = 0; i < SKY_PARAMS; ++i) J[i] = make_float3(0.0f, 0.0f, 0.0f);
    const D3 o = d3(of), d = d3(df), sun = d3(P.sun_dir);
    double te, tx, tmin = 0.0, tmax = 1.0e300;
    if (!sphere_hit_d(o, d, P.atm_r, &te, &tx) || tx < 0.0) return;
    if (te > tmin && te > 0.0) tmin = te;
    if (tx < tmax) tmax = tx;
    const double sR[3] = {P.sigma_r.x, P.sigma_r.y, P.sigma_r.z}, sM = P.sigma_m, tM = (double)P.sigma_m + P.sigma_am;
    const double hr = P.h_r, hm = P.h_m, er = P.earth_r;
    const double step = (tmax - tmin) / 16.0, half = 0.5 * step;
    double t = tmin, oR = 0.0, oM = 0.0, doR = 0.0, doM = 0.0;
    double iR[3] = {0, 0, 0}, iM[3] = {0, 0, 0}, diR[4][3] = {}, diM[4][3] = {};
    for (int i = 0; i < 16; ++i) {
        const double s = t + half;
        const D3 sp = {o.x + s * d.x, o.y + s * d.y, o.z + s * d.z};
        const double alt = sqrt(ddot(sp, sp)) - er;
        const double pR = exp(-alt / hr) * step, pM = exp(-alt / hm) * step;
        const double dpR = pR * alt / (hr * hr), dpM = pM * alt / (hm * hm);
        oR += pR;
        oM += pM;
        doR += dpR;
        doM += dpM;
        double lte, ltx;
        sphere_hit_d(sp, sun, P.atm_r, &lte, &ltx);
        const double lstep = ltx / 8.0;
        double lR = 0.0, lM = 0.0, dlR = 0.0, dlM = 0.0;
        int j;
        for (j = 0; j < 8; ++j) {
            const double ls = (j + 0.5) * lstep;
            const D3 q = {sp.x + ls * sun.x, sp.y + ls * sun.y, sp.z + ls * sun.z};
            const double altl = sqrt(ddot(q, q)) - er;
            if (altl < 0.0) break;
            const double eR = exp(-altl / hr) * lstep, eM = exp(-altl / hm) * lstep;
            lR += eR;
            lM += eM;
            dlR += eR * altl / (hr * hr);
            dlM += eM * altl / (hm * hm);
        }
        if (j == 8) {
            const double sr = oR + lR, sm = oM + lM, dsr = doR + dlR, dsm = doM + dlM;
            for (int c = 0; c < 3; ++c) {
                const double Tr = exp(-(sR[c] * sr + tM * sm));
                iR[c] += Tr * pR;
                iM[c] += Tr * pM;
                const double dtau[4] = {sr, sm, sR[c] * dsr, tM * dsm};
                for (int k = 0; k < 4; ++k) {
                    const double dTr = Tr == 0.0 ? 0.0 : -Tr * dtau[k];
                    diR[k][c] += dTr * pR;
                    diM[k][c] += dTr * pM;
                }
                diR[2][c] += Tr * dpR;
                diM[3][c] += Tr * dpM;
            }
        }
        t += step;
    }
    const double mu = ddot(d, sun);
    const double rp = 3.0 * (1.0 + mu * mu) / (16.0 * 3.14159265358979323846);
    const double g = 0.76;
    const double den = (8.0 * 3.14159265358979323846) * ((2.0 + g * g) * pow(1.0 + g * g - 2.0 * g * mu, 1.5));
    const double mp = 3.0 * ((1.0 - g * g) * (1.0 + mu * mu)) / den;
    const double K = 6.0e5 * (double)P.sun_emission;
    double j[SKY_PARAMS][3] = {};
    for (int c = 0; c < 3; ++c) {
        j[SKY_RAYLEIGH_R + c][c] = ((iR[c] + sR[c] * diR[0][c]) * rp + sM * diM[0][c] * mp) * K;
        j[SKY_MIE][c] = (sR[c] * diR[1][c] * rp + (iM[c] + sM * diM[1][c]) * mp) * K;
        j[SKY_RAYLEIGH_H][c] = (sR[c] * diR[2][c] * rp + sM * diM[2][c] * mp) * K;
        j[SKY_MIE_H][c] = (sR[c] * diR[3][c] * rp + sM * diM[3][c] * mp) * K;
    }
    for (int i = 0; i < SKY_PARAMS; ++i) J[i] = make_float3((float)j[i][0], (float)j[i][1], (float)j[i][2]);
}

// nishita_jacobian_d in single precision, with the geometry rewritten so
// that nothing cancels: the altitude of o + s d is h / (sqrt(R^2 + h) + R)
// with h = |o + s d|^2 - R^2 = (|o|^2 - R^2) + s (2 o.d + s d.d) formed from
// small terms (|o|^2 - R^2 = o.x^2 + o.z^2 + (o.y - R)(o.y + R)), likewise
// along the sun ray from each view sample, and the far root of each sphere
// intersection in its stable form; sample positions are tmin + (i + 1/2)
// step, not a running sum.  The altitudes are then good to ~1e-2 m (one
// float ulp of a 6.4e6 m vector is 0.5 m), and the Rayleigh derivatives'
// near-cancellation at the sun (terms ~30x the result) keeps ~1e-5 of the
// result; the float and FP64 pipes differ ~60x in rate on this part.
__device__ __forceinline__ float sphere_exit_s(float b, float a, float c) {   // far root of a t^2 + 2 b t + c
    const float disc = b * b - a * c;
    if (disc < 0.0f) return -1.0f;
    const float sq = sqrtf(disc);
    return b >= 0.0f ? -c / (b + sq) : (sq - b) / a;
}
static __device__ __noinline__ void nishita_jacobian_s(const SkyParams& P, float3 o, float3 d, float3* J) {
    for (int i = 0; i < SKY_PARAMS; ++i) J[i] = make_float3(0.0f, 0.0f, 0.0f);
    const float3 sun = P.sun_dir;
    const float R = P.earth_r, A = P.atm_r;
    const float dA = (A - R) * (A + R);                                   // A^2 - R^2
    const float h0 = o.x * o.x + o.z * o.z + (o.y - R) * (o.y + R);       // |o|^2 - R^2
    const float dd = dot(d, d), od = dot(o, d), ss = dot(sun, sun), osun = dot(o, sun), dsun = dot(d, sun);
    const float tmax = sphere_exit_s(od, dd, h0 - dA);
    if (!(tmax >= 0.0f)) return;
    const float disc0 = od * od - dd * (h0 - dA);
    const float te = (-od - sqrtf(fmaxf(disc0, 0.0f))) / dd;
    const float tmin = te > 0.0f ? te : 0.0f;
    const float sR[3] = {P.sigma_r.x, P.sigma_r.y, P.sigma_r.z}, sM = P.sigma_m, tM = P.sigma_m + P.sigma_am;
    const float hr = P.h_r, hm = P.h_m, ihr2 = 1.0f / (hr * hr), ihm2 = 1.0f / (hm * hm);
    const float step = (tmax - tmin) / 16.0f;
    const float R2 = R * R;
    float oR = 0.0f, oM = 0.0f, doR = 0.0f, doM = 0.0f;
    float iR[3] = {0, 0, 0}, iM[3] = {0, 0, 0}, diR[4][3] = {}, diM[4][3] = {};
    for (int i = 0; i < 16; ++i) {
        const float s = tmin + ((float)i + 0.5f) * step;
        const float h = h0 + s * (2.0f * od + s * dd);
        const float alt = h / (sqrtf(R2 + h) + R);
        const float pR = expf(-alt / hr) * step, pM = expf(-alt / hm) * step;
        const float dpR = pR * alt * ihr2, dpM = pM * alt * ihm2;
        oR += pR;
        oM += pM;
        doR += dpR;
        doM += dpM;
        const float b = osun + s * dsun;                                  // (o + s d) . sun
        const float ltx = sphere_exit_s(b, ss, h - dA);
        const float lstep = ltx / 8.0f;
        float lR = 0.0f, lM = 0.0f, dlR = 0.0f, dlM = 0.0f;
        int j;
        for (j = 0; j < 8; ++j) {
            const float ls = ((float)j + 0.5f) * lstep;
            const float hl = h + ls * (2.0f * b + ls * ss);
            const float altl = hl / (sqrtf(R2 + hl) + R);
            if (altl < 0.0f) break;
            const float eR = expf(-altl / hr) * lstep, eM = expf(-altl / hm) * lstep;
            lR += eR;
            lM += eM;
            dlR += eR * altl * ihr2;
            dlM += eM * altl * ihm2;
        }
        if (j == 8) {
            const float sr = oR + lR, sm = oM + lM, dsr = doR + dlR, dsm = doM + dlM;
            for (int c = 0; c < 3; ++c) {
                const float Tr = expf(-(sR[c] * sr + tM * sm));
                iR[c] += Tr * pR;
                iM[c] += Tr * pM;
                const float dtau[4] = {sr, sm, sR[c] * dsr, tM * dsm};
                for (int k = 0; k < 4; ++k) {
                    const float dTr = Tr == 0.0f ? 0.0f : -Tr * dtau[k];
                    diR[k][c] += dTr * pR;
                    diM[k][c] += dTr * pM;
                }
                diR[2][c] += Tr * dpR;
                diM[3][c] += Tr * dpM;
            }
        }
    }
    const float mu = dot(d, sun);
    const float rp = 3.0f * (1.0f + mu * mu) / (16.0f * 3.14159265f);
    const float g = 0.76f;
    const float den = (8.0f * 3.14159265f) * ((2.0f + g * g) * powf(1.0f + g * g - 2.0f * g * mu, 1.5f));
    const float mp = 3.0f * ((1.0f - g * g) * (1.0f + mu * mu)) / den;
    const float K = 6.0e5f * P.sun_emission;
    for (int c = 0; c < 3; ++c) {
        float* jr = &J[SKY_RAYLEIGH_R + c].x;
        jr[c] = ((iR[c] + sR[c] * diR[0][c]) * rp + sM * diM[0][c] * mp) * K;
        (&J[SKY_MIE].x)[c] = (sR[c] * diR[1][c] * rp + (iM[c] + sM * diM[1][c]) * mp) * K;
        (&J[SKY_RAYLEIGH_H].x)[c] = (sR[c] * diR[2][c] * rp + sM * diM[2][c] * mp) * K;
        (&J[SKY_MIE_H].x)[c] = (sR[c] * diR[3][c] * rp + sM * diM[3][c] * mp) * K;
    }
}

// nishita() with its derivatives: J[i] = dL/d(parameter i), i < SKY_PARAMS.
static __device__ __noinline__ float3 nishita_grad(const SkyParams& P, float3 o, float3 d, float3* J) {
    for (int i = 0; i < SKY_PARAMS; ++i) J[i] = make_float3(0.0f, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = __int_as_float(0x7f800000);
    {
        float te, tx;
        if (!sphere_hit(o, d, P.atm_r, &te, &tx) || tx < 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
        if (te > tmin && te > 0.0f) tmin = te;
        if (tx < tmax) tmax = tx;
    }
    const float step = xm(xs(tmax, tmin), 0.0625f);
    const float3 tR = make_float3(xa(P.sigma_r.x, 0.0f), xa(P.sigma_r.y, 0.0f), xa(P.sigma_r.z, 0.0f));
    const float tM = xa(P.sigma_m, P.sigma_am);
    const float half = xm(step, 0.5f);
    const float ihr2 = 1.0f / (P.h_r * P.h_r), ihm2 = 1.0f / (P.h_m * P.h_m);
    float t = tmin;
    float3 iR = make_float3(0.0f, 0.0f, 0.0f), iM = make_float3(0.0f, 0.0f, 0.0f);
    // derivatives of iR, iM: [0] d/d sigma_r (own channel), [1] d/d sigma_m, [2] d/d h_r, [3] d/d h_m
    float3 diR[4], diM[4];
    for (int k = 0; k < 4; ++k) diR[k] = diM[k] = make_float3(0.0f, 0.0f, 0.0f);
    float oR = 0.0f, oM = 0.0f, doR = 0.0f, doM = 0.0f;   // doR = d oR / d h_r, doM = d oM / d h_m
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        float3 sp = xpoint(o, xa(t, half), d);
        float alt = xs(__fsqrt_rn(xdot(sp, sp)), P.earth_r);
        float pR = xm(expf(-alt * P.inv_h_r), step);
        float pM = xm(expf(-alt * P.inv_h_m), step);
        float dpR = pR * alt * ihr2, dpM = pM * alt * ihm2;   // d/d h of exp(-alt / h) * step
        oR = xa(oR, pR);
        oM = xa(oM, pM);
        doR += dpR;
        doM += dpM;
        float lte, ltx;
        sphere_hit(sp, P.sun_dir, P.atm_r, &lte, &ltx);
        float lstep = xm(ltx, 0.125f);
        float lhalf = xm(lstep, 0.5f);
        float lt = 0.0f, lR = 0.0f, lM = 0.0f, dlR = 0.0f, dlM = 0.0f;
        int j;
#pragma unroll
        for (j = 0; j < 8; ++j) {
            float3 spl = xpoint(sp, xa(lt, lhalf), P.sun_dir);
            float altl = xs(__fsqrt_rn(xdot(spl, spl)), P.earth_r);
            if (altl < 0.0f) break;
            float eR = xm(expf(-altl * P.inv_h_r), lstep), eM = xm(expf(-altl * P.inv_h_m), lstep);
            lR = xa(lR, eR);
            lM = xa(lM, eM);
            dlR += eR * altl * ihr2;
            dlM += eM * altl * ihm2;
            lt = xa(lt, lstep);
        }
        if (j == 8) {
            float sr = xa(oR, lR), sm = xa(oM, lM);
            float dsr = doR + dlR, dsm = doM + dlM;
            float tmm = xm(tM, sm);
            float3 tau = make_float3(xa(xm(tR.x, sr), tmm), xa(xm(tR.y, sr), tmm), xa(xm(tR.z, sr), tmm));
            float3 Tr = make_float3(expf(-tau.x), expf(-tau.y), expf(-tau.z));
            iR = make_float3(xa(iR.x, xm(Tr.x, pR)), xa(iR.y, xm(Tr.y, pR)), xa(iR.z, xm(Tr.z, pR)));
            iM = make_float3(xa(iM.x, xm(Tr.x, pM)), xa(iM.y, xm(Tr.y, pM)), xa(iM.z, xm(Tr.z, pM)));
            // d tau: sigma_r (own channel) sr; sigma_m sm; h_r sigma_r dsr; h_m tM dsm; dTr = -Tr dtau
            const float3 dtau[4] = {make_float3(sr, sr, sr), make_float3(sm, sm, sm), tR * dsr,
                                    make_float3(tM * dsm, tM * dsm, tM * dsm)};
            for (int k = 0; k < 4; ++k) {
                float3 dTr = -zmul(Tr, dtau[k]);
                diR[k] = diR[k] + dTr * pR;
                diM[k] = diM[k] + dTr * pM;
            }
            diR[2] = diR[2] + zmul(Tr, make_float3(dpR, dpR, dpR));
            diM[3] = diM[3] + zmul(Tr, make_float3(dpM, dpM, dpM));
        }
        t = xa(t, step);
    }
    float mu = dot(d, P.sun_dir);
    float rp = (3.0f * (1.0f + Sqr(mu))) / (16.0f * PI_F);
    const float g = 0.76f;
    float den = (8.0f * PI_F) * ((2.0f + Sqr(g)) * powf(1.0f + Sqr(g) - 2.0f * g * mu, 1.5f));
    float mp = 3.0f * ((1.0f - Sqr(g)) * (1.0f + Sqr(mu))) / den;
    const float K = 6.0e5f * P.sun_emission;
    float3 L = P.sigma_r * iR * rp + make_float3(P.sigma_m, P.sigma_m, P.sigma_m) * iM * mp;
    const float3 sM = make_float3(P.sigma_m, P.sigma_m, P.sigma_m);
    // L_c = (sigma_r_c iR_c rp + sigma_m iM_c mp) K; sigma_r_c enters only channel c
    float3 dLr = (iR + P.sigma_r * diR[0]) * rp + sM * diM[0] * mp;
    J[SKY_RAYLEIGH_R] = make_float3(dLr.x * K, 0.0f, 0.0f);
    J[SKY_RAYLEIGH_G] = make_float3(0.0f, dLr.y * K, 0.0f);
    J[SKY_RAYLEIGH_B] = make_float3(0.0f, 0.0f, dLr.z * K);
    J[SKY_MIE] = (P.sigma_r * diR[1] * rp + (iM + sM * diM[1]) * mp) * K;
    J[SKY_RAYLEIGH_H] = (P.sigma_r * diR[2] * rp + sM * diM[2] * mp) * K;
    J[SKY_MIE_H] = (P.sigma_r * diR[3] * rp + sM * diM[3] * mp) * K;
    return L * 6.0e5f * P.sun_emission;   // nishita()'s own rounding
}

}  // namespace kpt
