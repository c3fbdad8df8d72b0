// adjoint_oracle.cpp -- FP64 host oracle for the path-replay adjoint.
//
// TEST INFRASTRUCTURE, not part of the library: only tests/ call it.
//
// Given the frozen path records written by kpt_adjoint_records_device (every
// vertex of every replayed sample with what the adjoint holds fixed: local
// directions, pdfs, roulette factors, light-sample factors, emission, the
// sample's adjoint weight), orc_adjoint_estimate evaluates in double precision
//     E(theta) = sum over samples of g . L(theta)
// where L is the path's radiance rebuilt vertex by vertex with the BSDF
// values and the sky evaluated at theta = (per material albedo, roughness;
// Rayleigh r, g, b, Mie, Rayleigh and Mie scale heights).  Central
// differences of E give the gradient the adjoint must return.  The BSDF lobes
// restate the reference's formulas (shaders/bsdf.cuh:18-624: GGX D and Smith
// G, dielectric Fresnel, conductor Schlick, opaque and transparent
// dielectric) and the sky its Nishita march (shaders/atmosphere.cuh:132-223),
// all in double.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>

namespace {

// the layout of AdjRec (kittlespt_gb300/csrc/kpt_internal.h), 192 bytes
struct Rec {
    int32_t item, vertex, material, flags;
    int32_t lobe, nee, pixel, pad0;
    float alb_tex[3], rough_tex;
    float metallic, transmission, ior, eta;
    float wo[3], cosw;
    float wi[3], pdf;
    float wm[3], rr;
    float nwi[3], ncos;
    float nfac[3], pad1;
    float emit[3], pad2;
    float g[3], pad3;
    float miss[3], pad4;
};
static_assert(sizeof(Rec) == 192, "record layout");

enum { FIRST = 1, BACKFACE = 2, LAST = 4, ESCAPED = 8, NEE_VIS = 16 };
enum { L_NONE = 0, L_CONDUCTOR, L_T_REFLECT, L_T_TRANSMIT, L_O_GLOSSY, L_O_DIFFUSE };

constexpr double PI = 3.14159265358979323846;

struct V3 {
    double x, y, z;
};
V3 v3(const float* p) { return {p[0], p[1], p[2]}; }
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 normalize(V3 v) { return v * (1.0 / std::sqrt(dot(v, v))); }
double sqr(double v) { return v * v; }
double clampd(double v, double a, double b) { return std::fmax(a, std::fmin(v, b)); }

// GGX (bsdf.cuh:18-57)
double ggx_D(double alpha, V3 wm) {
    double a = alpha < 0.001 ? std::fmax(alpha, 1.0e-3) : alpha;
    double a2 = a * a;
    double ndh = sqr(clampd(wm.z, 0.0, 1.0));
    double b = ndh * (a2 - 1.0) + 1.0;
    return a2 / (PI * b * b);
}
double ggx_G(double alpha, V3 wo, V3 wi) {
    double nv = std::fmax(wo.z, 0.0), nl = std::fabs(wi.z);
    double tv = std::sqrt(alpha * alpha + (1.0 - alpha * alpha) * nv * nv);
    double tl = std::sqrt(alpha * alpha + (1.0 - alpha * alpha) * nl * nl);
    return ((2.0 * nv) / (nv + tv)) * ((2.0 * nl) / (nl + tl));
}
double fresnel_dielectric(double c, double ior) {   // bsdf.cuh:122-141
    c = clampd(c, -1.0, 1.0);
    if (c < 0.0) {
        ior = 1.0 / ior;
        c = -c;
    }
    double s2 = 1.0 - c * c, s2t = s2 / (ior * ior);
    if (s2t >= 1.0) return 1.0;
    double ct = std::sqrt(1.0 - s2t);
    double rp = (ior * c - ct) / (ior * c + ct), rs = (c - ior * ct) / (c + ior * ct);
    return (rp * rp + rs * rs) * 0.5;
}
double micro(double alpha, V3 wo, V3 wi, V3 wm) {   // bsdf.cuh:151-164
    double nv = clampd(wo.z, 0.0, 1.0), nl = clampd(wi.z, 0.0, 1.0);
    if (wi.z <= 0.0 || dot(wi, wm) <= 0.0) return 0.0;
    return ggx_D(alpha, wm) * ggx_G(alpha, wo, wi) / (4.0 * std::fmax(nv, 1.0e-3) * nl);
}

struct Mat {
    V3 albedo;
    double alpha, metallic, transmission, ior;
    bool backface;
};

V3 f_conductor(const Mat& m, V3 wo, V3 wi) {
    V3 wm = normalize(wo + wi);
    double nv = clampd(wo.z, 0.0, 1.0), nl = clampd(wi.z, 0.0, 1.0);
    if (nv == 0.0 || nl == 0.0) return {0, 0, 0};
    double voh = clampd(dot(wo, wm), 0.0, 1.0);
    if (!(nl > 0.0 && voh > 0.0)) return {0, 0, 0};
    double p5 = std::pow(1.0 - voh, 5.0);
    V3 F = {clampd(m.albedo.x + (1.0 - m.albedo.x) * p5, 0.0, 1.0), clampd(m.albedo.y + (1.0 - m.albedo.y) * p5, 0.0, 1.0),
            clampd(m.albedo.z + (1.0 - m.albedo.z) * p5, 0.0, 1.0)};
    return F * micro(m.alpha, wo, wi, wm);
}
V3 f_opaque(const Mat& m, V3 wo, V3 wi) {
    V3 wm = normalize(wo + wi);
    double g = fresnel_dielectric(dot(wo, wm), m.ior) * micro(m.alpha, wo, wi, wm);
    double fd = (wo.z * wi.z > 0 ? 1.0 : 0.0) / PI;
    return m.albedo * ((1.0 - g) * fd) + V3{g, g, g};
}
V3 f_transparent(const Mat& m, V3 wo, V3 wi) {
    double co = wo.z, ci = wi.z;
    bool refl = co * ci > 0.0;
    double eta = refl ? 1.0 : (!m.backface ? m.ior : 1.0 / m.ior);
    V3 wm = wi * eta + wo;
    wm = normalize(wm.z > 0 ? wm : wm * -1.0);
    if (dot(wm, wi) * ci < 0.0 || dot(wm, wo) * co < 0.0) return {0, 0, 0};
    double F = fresnel_dielectric(std::fabs(dot(wo, wm)), m.ior);
    if (refl) {
        double v = F * micro(m.alpha, wo, wi, wm);
        return {v, v, v};
    }
    double temp = dot(wi, wm) * eta + dot(wo, wm);
    double dwm = std::fabs(dot(wi, wm)) * std::fabs(dot(wo, wm)) / (temp * temp);
    double T = ggx_D(m.alpha, wm) * ggx_G(m.alpha, wo, wi) * dwm / std::fabs(ci * co);
    return m.albedo * ((1.0 - F) * T);
}
// UnifiedBSDF::f (bsdf.cuh:191-216), local directions
V3 bsdf_f(const Mat& m, V3 wo, V3 wi) {
    double wt = (1.0 - m.metallic) * m.transmission, wd = (1.0 - m.metallic) * (1.0 - m.transmission);
    V3 F = {0, 0, 0};
    if (m.metallic > 0.0) F = F + f_conductor(m, wo, wi) * m.metallic;
    if (wt > 0.0) F = F + f_transparent(m, wo, wi) * wt;
    if (wd > 0.0) F = F + f_opaque(m, wo, wi) * wd;
    return F;
}
// f of the sampled lobe at the recorded sample (UnifiedBSDF::sampleF, bsdf.cuh:243-624)
V3 lobe_f(const Mat& m, const Rec& r) {
    V3 wo = v3(r.wo), wi = v3(r.wi), wm = v3(r.wm);
    const bool tir = r.pad0 & 1, inside = (r.pad0 >> 1) & 1;
    switch (r.lobe) {
    case L_CONDUCTOR:
        return f_conductor(m, wo, wi);
    case L_T_REFLECT: {
        double v = fresnel_dielectric(dot(wo, wm), r.eta) * micro(m.alpha, wo, wi, wm) * (tir ? 1.0 : 2.0);
        return {v, v, v};
    }
    case L_T_TRANSMIT: {
        double temp = dot(wi, wm) * r.eta + dot(wo, wm);
        double F = fresnel_dielectric(std::fabs(dot(wo, wm)), r.eta);
        double T = ggx_D(m.alpha, wm) * ggx_G(m.alpha, wo, wi) *
                   std::fabs(dot(wi, wm) * dot(wo, wm) / (wi.z * wo.z * temp * temp));
        return m.albedo * ((1.0 - F) * T * (inside ? 1.0 : 2.0));
    }
    case L_O_GLOSSY: {
        double v = fresnel_dielectric(dot(wo, wm), m.ior) * micro(m.alpha, wo, wi, wm) * 2.0;
        return {v, v, v};
    }
    case L_O_DIFFUSE: {
        double fd = (wo.z * wi.z > 0 ? 1.0 : 0.0) / PI;
        return m.albedo * (fd * 2.0);
    }
    default:
        return {0, 0, 0};
    }
}

struct Sky {
    V3 sigma_r, sun_dir;
    double sigma_m, sigma_am, h_r, h_m, earth_r, atm_r, sun_emission;
};

bool sphere_hit(V3 o, V3 d, double radius, double* t0, double* t1) {   // atmosphere.cuh ray-sphere
    V3 oc = o * -1.0;
    double a = dot(d, d), b = -2.0 * dot(d, oc), c = dot(oc, oc) - radius * radius;
    double disc = b * b - 4.0 * a * c;
    if (disc < 0.0) return false;
    double sq = std::sqrt(disc);
    double x0 = (-b - sq) / (2.0 * a), x1 = (-b + sq) / (2.0 * a);
    if (x0 > x1) std::swap(x0, x1);
    *t0 = x0;
    *t1 = x1;
    return !(x1 < 0.0);
}

// NishitaAtmosphereModel::sampleLi (atmosphere.cuh:132-223) in double
V3 nishita(const Sky& P, V3 o, V3 d) {
    double tmin = 0.0, tmax = INFINITY, te, tx;
    if (!sphere_hit(o, d, P.atm_r, &te, &tx) || tx < 0.0) return {0, 0, 0};
    if (te > tmin && te > 0.0) tmin = te;
    if (tx < tmax) tmax = tx;
    const double step = (tmax - tmin) / 16.0, half = step * 0.5, tM = P.sigma_m + P.sigma_am;
    double t = tmin, oR = 0.0, oM = 0.0;
    V3 iR = {0, 0, 0}, iM = {0, 0, 0};
    for (int i = 0; i < 16; ++i) {
        V3 sp = o + d * (t + half);
        double alt = std::sqrt(dot(sp, sp)) - P.earth_r;
        double pR = std::exp(-alt / P.h_r) * step, pM = std::exp(-alt / P.h_m) * step;
        oR += pR;
        oM += pM;
        double lte, ltx;
        sphere_hit(sp, P.sun_dir, P.atm_r, &lte, &ltx);
        double lstep = ltx / 8.0, lhalf = lstep * 0.5, lt = 0.0, lR = 0.0, lM = 0.0;
        int j;
        for (j = 0; j < 8; ++j) {
            V3 spl = sp + P.sun_dir * (lt + lhalf);
            double altl = std::sqrt(dot(spl, spl)) - P.earth_r;
            if (altl < 0.0) break;
            lR += std::exp(-altl / P.h_r) * lstep;
            lM += std::exp(-altl / P.h_m) * lstep;
            lt += lstep;
        }
        if (j == 8) {
            double sr = oR + lR, sm = oM + lM;
            V3 Tr = {std::exp(-(P.sigma_r.x * sr + tM * sm)), std::exp(-(P.sigma_r.y * sr + tM * sm)),
                     std::exp(-(P.sigma_r.z * sr + tM * sm))};
            iR = iR + Tr * pR;
            iM = iM + Tr * pM;
        }
        t += step;
    }
    double mu = dot(d, P.sun_dir);
    double rp = 3.0 * (1.0 + mu * mu) / (16.0 * PI);
    const double g = 0.76;
    double den = (8.0 * PI) * ((2.0 + g * g) * std::pow(1.0 + g * g - 2.0 * g * mu, 1.5));
    double mp = 3.0 * ((1.0 - g * g) * (1.0 + mu * mu)) / den;
    V3 L = P.sigma_r * iR * rp + iM * (P.sigma_m * mp);
    return L * (6.0e5 * P.sun_emission);
}

}  // namespace

extern "C" {

// The sky radiance in double for n directions (sky, fixed as below).
void orc_sky_double(int n, const float* dirs, const double* sky, const double* fixed, double* out) {
    Sky P;
    P.sigma_r = {sky[0], sky[1], sky[2]};
    P.sigma_m = sky[3];
    P.h_r = sky[4];
    P.h_m = sky[5];
    P.sun_dir = {fixed[0], fixed[1], fixed[2]};
    P.sun_emission = fixed[3];
    P.sigma_am = fixed[4];
    P.earth_r = fixed[5];
    P.atm_r = fixed[6];
    const V3 obs = {0.0, P.earth_r + 1.0, 0.0};
    for (int i = 0; i < n; ++i) {
        V3 L = nishita(P, obs, v3(dirs + 3 * i));
        out[3 * i] = L.x;
        out[3 * i + 1] = L.y;
        out[3 * i + 2] = L.z;
    }
}

// E(theta) over n frozen vertex records (an item's vertices are contiguous,
// its last one flagged).  albedo[3 m + c], roughness[m]; sky = (Rayleigh r,
// g, b, Mie, Rayleigh height, Mie height); fixed = (sun direction xyz, sun
// emission factor, Mie absorption, earth radius, atmosphere radius).
// Returns the number of items.
int orc_adjoint_estimate(const void* records, int n, const double* albedo, const double* roughness,
                         const double* sky, const double* fixed, double* out) {
    const Rec* rec = static_cast<const Rec*>(records);
    Sky P;
    P.sigma_r = {sky[0], sky[1], sky[2]};
    P.sigma_m = sky[3];
    P.h_r = sky[4];
    P.h_m = sky[5];
    P.sun_dir = {fixed[0], fixed[1], fixed[2]};
    P.sun_emission = fixed[3];
    P.sigma_am = fixed[4];
    P.earth_r = fixed[5];
    P.atm_r = fixed[6];
    const V3 obs = {0.0, P.earth_r + 1.0, 0.0};
    const V3 sun_rad = nishita(P, obs, P.sun_dir);
    double E = 0.0;
    int items = 0;
    V3 beta = {1, 1, 1}, L = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const Rec& r = rec[i];
        const bool first = r.flags & FIRST;
        Mat M;
        const int m = r.material;
        M.albedo = first ? V3{1, 1, 1}
                         : V3{albedo[3 * m] * r.alb_tex[0], albedo[3 * m + 1] * r.alb_tex[1], albedo[3 * m + 2] * r.alb_tex[2]};
        double re = roughness[m] * r.rough_tex;
        M.alpha = re * re;
        if (!first && M.alpha < 0.3) M.alpha = clampd(2.0 * M.alpha, 0.1, 0.3);
        M.metallic = r.metallic;
        M.transmission = r.transmission;
        M.ior = r.ior;
        M.backface = r.flags & BACKFACE;
        V3 c = v3(r.emit);
        if (r.flags & NEE_VIS) {
            V3 f = bsdf_f(M, v3(r.wo), v3(r.nwi)) * r.ncos;
            c = c + f * (r.nee == 1 ? sun_rad * v3(r.nfac) : v3(r.nfac));
        }
        L = L + beta * c;
        if (r.lobe != L_NONE && r.rr > 0.0f) beta = beta * (lobe_f(M, r) * (r.cosw / r.pdf * r.rr));
        if (r.flags & LAST) {
            if (r.flags & ESCAPED) L = L + beta * nishita(P, obs, v3(r.miss));
            // channels the clamp removed carry weight 0 (and may be infinite here)
            const V3 g = v3(r.g);
            E += (g.x != 0.0 ? g.x * L.x : 0.0) + (g.y != 0.0 ? g.y * L.y : 0.0) + (g.z != 0.0 ? g.z * L.z : 0.0);
            ++items;
            beta = {1, 1, 1};
            L = {0, 0, 0};
        }
    }
    *out = E;
    return items;
}

}  // extern "C"
