// kpt_fsr.cu -- the reference's FSR 1.0 upscale path: EASU (edge-adaptive
// spatial upsampling of the render to the output size) and RCAS (robust
// contrast-adaptive sharpening of that image).  The reference compiles this
// path only with USE_FSR defined (kernels.cuh:3; launchUpscaleComputeKernel,
// kernels.cu:84-104, runs the upscale kernel's FSR branch, upscale.cuh:
// 271-283, then the sharpen kernel, upscale.cuh:415-433); here it is
// kpt_settings.upscale = 2.
//
// The unit is compiled without fast maths and without contraction
// (-fmad=false): every float operation rounds once, in the reference's order,
// and the reference's double-precision literals (0.5, .4, 1.5625, .29, 1. /
// lob, 4. * lobe + 1., the RCAS limit) keep their double results, so the
// images are bit for bit those of the reference compiled for the host.  FP64
// is slow on this GPU, so where a float form provably rounds to the same
// float it replaces the double one (each case says why); the rest stays in
// double.
// Reads go through textureReadBilinear's rule (device_texture_buffer.cuh:
// 42-80): the pixel position truncated toward zero, texels clamped to the
// image, lerps with the remainder (negative at the top and left edges).
#include "kpt_post.h"

namespace kpt {
namespace {

__device__ __forceinline__ float3 texel3(const float4* img, int w, int h, int x, int y) {
    x = min(max(x, 0), w - 1);
    y = min(max(y, 0), h - 1);
    const float4 v = __ldg(img + (size_t)y * w + x);
    return make_float3(v.x, v.y, v.z);
}

__device__ __forceinline__ float3 lerp3(float3 a, float3 b, float t) {
    return make_float3(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z));
}

// textureReadBilinear at pixel position (px, py), colour channels only
__device__ __forceinline__ float3 bilinear3(const float4* img, int w, int h, float px, float py) {
    const int ix = (int)px, iy = (int)py;
    const float ws = px - (float)ix, wt = py - (float)iy;
    const float3 top = lerp3(texel3(img, w, h, ix, iy), texel3(img, w, h, ix + 1, iy), ws);
    const float3 bot = lerp3(texel3(img, w, h, ix, iy + 1), texel3(img, w, h, ix + 1, iy + 1), ws);
    return lerp3(top, bot, wt);
}

// luma times two of the reference, y + 0.5 * (x + z), evaluated there in
// double and rounded to float.  When halving s = x + z is exact in float, the
// float sum y + s/2 is the same float: the exact sum rounded once, and where
// double cannot hold the exact sum (exponents more than 29 apart) the
// smaller term is below half a float ulp of the larger either way.  A
// subnormal s takes the double form.
__device__ __forceinline__ float luma2(float3 c) {
    const float s = c.x + c.z, h = 0.5f * s;
    if (h + h == s) return c.y + h;
    return (float)((double)c.y + 0.5 * (double)s);
}

// clamp(q, 0, 1) of helper_math, fmaxf(0, fminf(q, 1)), which gives 1 for a
// NaN q (0 / 0 on a flat row or column of lumas); spelled out so that the
// NaN case cannot become a saturation (which gives 0)
__device__ __forceinline__ float clamp01(float q) {
    return isnan(q) ? 1.0f : fmaxf(0.0f, fminf(q, 1.0f));
}

// FsrEasuSetF (upscale.cuh:101-130): gradient direction and edge length of
// one bilinear corner from its '+' of lumas  a / b c d / e
__device__ __forceinline__ void easu_set(float2& dir, float& len, float w, float lA, float lB, float lC, float lD,
                                         float lE) {
    float lenX = fmaxf(fabsf(lD - lC), fabsf(lC - lB));
    const float dirX = lD - lB;
    dir.x += dirX * w;
    lenX = clamp01(fabsf(dirX) / lenX);
    lenX *= lenX;
    len += lenX * w;
    float lenY = fmaxf(fabsf(lE - lC), fabsf(lC - lA));
    const float dirY = lE - lA;
    dir.y += dirY * w;
    lenY = clamp01(fabsf(dirY) / lenY);
    lenY *= lenY;
    len += lenY * w;
}

// 0.4 (double) - 0.4f, rounded to float: the low part of 0.4
constexpr float CL4 = -0x1.99999ap-28f;

struct EasuKernel {
    float2 dir, len2;
    float lob, clp, ppx, ppy;
    float3 aC;
    float aW;
    // FsrEasuTapF (upscale.cuh:65-98): the tap at (tx, ty) from the texel
    // grid's origin, weighted by a windowed Lanczos-2 approximation along the
    // rotated, stretched offset
    __device__ __forceinline__ void tap(float tx, float ty, float3 c) {
        const float ox = tx - ppx, oy = ty - ppy;
        float vx = ox * dir.x + oy * dir.y;
        float vy = ox * -dir.y + oy * dir.x;
        vx *= len2.x;
        vy *= len2.y;
        const float d2 = fminf(vx * vx + vy * vy, clp);
        // 0.4 * d2 - 1.0 in double rounded to float, from floats: the
        // product with 0.4 split as 0.4f + CL4 (an exact product and its
        // error by fma), then a two-sum with -1.  After the squaring and
        // the fused step below it gives the double form's wB for every float
        // d2 in [0, 4.8] (d2 <= clp <= 1 / 0.21), checked exhaustively; the
        // one input where the two differ before squaring is 2.5 (0 against
        // -2^-52).
        const float ph = 0.4f * d2, pl = fmaf(0.4f, d2, -ph), tt = fmaf(CL4, d2, pl);
        const float sm = ph + -1.0f, bb = sm - ph, er = (ph - (sm - bb)) + (-1.0f - bb);
        float wB = sm + (er + tt);
        // (double)(lob * d2) - 1.0 rounded to float: p = lob * d2 lies in
        // [0, 2] (d2 <= clp = 1 / lob); for p >= 2^-29 the difference is
        // exact in double, so one float subtraction rounds it the same, and
        // below that both give -1
        float wA = lob * d2 - 1.0f;
        wB *= wB;
        wA *= wA;
        // 1.5625 * wB - 0.5625 in double, wB in [0, 1]: the product (29
        // bits) is exact and the difference either exact or, for wB < 2^-26,
        // rounded far from a float tie, so one fused rounding is the same
        wB = fmaf(1.5625f, wB, -0.5625f);
        const float w = wB * wA;
        aC.x += c.x * w;
        aC.y += c.y * w;
        aC.z += c.z * w;
        aW += w;
    }
};

}  // namespace

// FsrEasuCon (upscale.cuh:18-62) with the render size as viewport and
// input size, on the host (IEEE float divisions and the reference's double
// expressions, the same on x86-64 and aarch64 hosts)
EasuCon easu_constants(int sw, int sh, int dw, int dh) {
    const float inw = (float)sw, inh = (float)sh, ow = (float)dw, oh = (float)dh;
    EasuCon c;
    c.c0x = inw / ow;
    c.c0y = inh / oh;
    c.c0z = (float)(0.5 * (double)inw / (double)ow - 0.5);
    c.c0w = (float)(0.5 * (double)inh / (double)oh - 0.5);
    c.c1x = 1.0f / inw;
    c.c1y = 1.0f / inh;
    c.c1z = 1.0f / inw;
    c.c1w = -1.0f / inh;
    c.c2x = -1.0f / inw;
    c.c2y = 2.0f / inh;
    c.c2z = 1.0f / inw;
    c.c2w = 2.0f / inh;
    c.c3x = 0.0f / inw;
    c.c3y = 4.0f / inh;
    return c;
}

// EASU (FsrEasuF, upscale.cuh:133-254) of the render [sh][sw] into dst
// [dh][dw], one thread per output pixel
__global__ void k_easu(const float4* src, int sw, int sh, float4* dst, int dw, int dh, EasuCon con) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const float inw = (float)sw, inh = (float)sh;
    const float c0x = con.c0x, c0y = con.c0y, c0z = con.c0z, c0w = con.c0w;
    const float c1x = con.c1x, c1y = con.c1y, c1z = con.c1z, c1w = con.c1w;
    const float c2x = con.c2x, c2y = con.c2y, c2z = con.c2z, c2w = con.c2w;
    const float c3x = con.c3x, c3y = con.c3y;
    const float offx = -0.5f * c1x, offy = 0.5f * c1x, offz = -0.5f * c1y, offw = 0.5f * c1y;

    float ppx = (float)x * c0x + c0z, ppy = (float)y * c0y + c0w;
    const float fpx = floorf(ppx), fpy = floorf(ppy);
    ppx -= fpx;
    ppy -= fpy;
    const float p0x = fpx * c1x + c1z, p0y = fpy * c1y + c1w;
    const float p1x = p0x + c2x, p1y = p0y + c2y;
    const float p2x = p0x + c2z, p2y = p0y + c2w;
    const float p3x = p0x + c3x, p3y = p0y + c3y;
    // the 12 taps  b c / e f g h / i j k l / n o, each a bilinear read at a
    // normalised position scaled back to pixels
    auto tap = [&](float px, float py, float ox, float oy) {
        return bilinear3(src, sw, sh, (px + ox) * inw, (py + oy) * inh);
    };
    const float3 bC = tap(p0x, p0y, offx, offw), cC = tap(p0x, p0y, offy, offw);
    const float3 iC = tap(p1x, p1y, offx, offw), jC = tap(p1x, p1y, offy, offw);
    const float3 fC = tap(p1x, p1y, offy, offz), eC = tap(p1x, p1y, offx, offz);
    const float3 kC = tap(p2x, p2y, offx, offw), lC = tap(p2x, p2y, offy, offw);
    const float3 hC = tap(p2x, p2y, offy, offz), gC = tap(p2x, p2y, offx, offz);
    const float3 oC = tap(p3x, p3y, offy, offz), nC = tap(p3x, p3y, offx, offz);
    const float bL = luma2(bC), cL = luma2(cC), iL = luma2(iC), jL = luma2(jC), fL = luma2(fC), eL = luma2(eC);
    const float kL = luma2(kC), lL = luma2(lC), hL = luma2(hC), gL = luma2(gC), oL = luma2(oC), nL = luma2(nC);

    float2 dir = make_float2(0.0f, 0.0f);
    float len = 0.0f;
    easu_set(dir, len, (float)((1.0 - (double)ppx) * (1.0 - (double)ppy)), bL, eL, fL, gL, jL);
    easu_set(dir, len, (float)((double)ppx * (1.0 - (double)ppy)), cL, fL, gL, hL, kL);
    easu_set(dir, len, (float)((1.0 - (double)ppx) * (double)ppy), fL, iL, jL, kL, nL);
    easu_set(dir, len, ppx * ppy, gL, jL, kL, lL, oL);

    // normalise the direction (1 / sqrt, both correctly rounded), shape the
    // length, set the anisotropic window
    const float d2x = dir.x * dir.x, d2y = dir.y * dir.y;
    float dirR = d2x + d2y;
    const bool zro = dirR < 1.0f / 32768.0f;
    dirR = 1.0f / sqrtf(dirR);
    dirR = zro ? 1.0f : dirR;
    dir.x = zro ? 1.0f : dir.x;
    dir.x *= dirR;
    dir.y *= dirR;
    len = (float)((double)len * 0.5);
    len *= len;
    const float stretch = (dir.x * dir.x + dir.y * dir.y) / fmaxf(fabsf(dir.x), fabsf(dir.y));
    EasuKernel K;
    K.dir = dir;
    // 1. - .5 * len and 1. / lob in double give the float forms' results for
    // every float len in [0, 1] and lob in [0.2, 0.51] (checked
    // exhaustively); .29 * len and the stretch term stay in double
    K.len2 = make_float2((float)(1.0 + ((double)stretch - 1.0) * (double)len), 1.0f - 0.5f * len);
    K.lob = (float)(0.5 - 0.29 * (double)len);
    K.clp = 1.0f / K.lob;
    K.ppx = ppx;
    K.ppy = ppy;
    K.aC = make_float3(0.0f, 0.0f, 0.0f);
    K.aW = 0.0f;
    K.tap(0.0f, -1.0f, bC);
    K.tap(1.0f, -1.0f, cC);
    K.tap(-1.0f, 1.0f, iC);
    K.tap(0.0f, 1.0f, jC);
    K.tap(0.0f, 0.0f, fC);
    K.tap(-1.0f, 0.0f, eC);
    K.tap(1.0f, 1.0f, kC);
    K.tap(2.0f, 1.0f, lC);
    K.tap(2.0f, 0.0f, hC);
    K.tap(1.0f, 0.0f, gC);
    K.tap(1.0f, 2.0f, oC);
    K.tap(0.0f, 2.0f, nC);
    // deringing: clamp to the range of the four nearest texels
    const float mnx = fminf(fminf(fC.x, gC.x), fminf(jC.x, kC.x)), mxx = fmaxf(fmaxf(fC.x, gC.x), fmaxf(jC.x, kC.x));
    const float mny = fminf(fminf(fC.y, gC.y), fminf(jC.y, kC.y)), mxy = fmaxf(fmaxf(fC.y, gC.y), fmaxf(jC.y, kC.y));
    const float mnz = fminf(fminf(fC.z, gC.z), fminf(jC.z, kC.z)), mxz = fmaxf(fmaxf(fC.z, gC.z), fmaxf(jC.z, kC.z));
    const float rx = fminf(mxx, fmaxf(mnx, K.aC.x / K.aW));
    const float ry = fminf(mxy, fmaxf(mny, K.aC.y / K.aW));
    const float rz = fminf(mxz, fmaxf(mnz, K.aC.z / K.aW));
    dst[(size_t)y * dw + x] = make_float4(rx, ry, rz, 1.0f);
}

// RCAS (FsrRcasF with sharpness 0, upscale.cuh:316-375; the sharpen kernel,
// :415-433) of the EASU image [h][w] into dst, one thread per pixel
__global__ void k_rcas(const float4* src, int w, int h, float4* dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float fw = (float)w, fh = (float)h;
    // FsrRcasLoadF: textureReadBilinearUV(p / size), i.e. a bilinear read at
    // (p / size) * size
    auto load = [&](float px, float py) { return bilinear3(src, w, h, (px / fw) * fw, (py / fh) * fh); };
    const float sx = (float)x, sy = (float)y;
    const float3 b = load(sx + 0.0f, sy + -1.0f), d = load(sx + -1.0f, sy + 0.0f), e = load(sx, sy);
    const float3 f = load(sx + 1.0f, sy + 0.0f), hh = load(sx + 0.0f, sy + 1.0f);
    const float3 mn4 = make_float3(fminf(b.x, fminf(f.x, hh.x)), fminf(b.y, fminf(f.y, hh.y)), fminf(b.z, fminf(f.z, hh.z)));
    const float3 mx4 = make_float3(fmaxf(b.x, fmaxf(f.x, hh.x)), fmaxf(b.y, fmaxf(f.y, hh.y)), fmaxf(b.z, fmaxf(f.z, hh.z)));
    // limiters: the lobe that keeps the ring within [0, 1]
    const float hminx = mn4.x / (4.0f * mx4.x), hmaxx = (1.0f - mx4.x) / (4.0f * mn4.x + -4.0f);
    const float hminy = mn4.y / (4.0f * mx4.y), hmaxy = (1.0f - mx4.y) / (4.0f * mn4.y + -4.0f);
    const float hminz = mn4.z / (4.0f * mx4.z), hmaxz = (1.0f - mx4.z) / (4.0f * mn4.z + -4.0f);
    const float lx = fmaxf(-hminx, hmaxx), ly = fmaxf(-hminy, hmaxy), lz = fmaxf(-hminz, hmaxz);
    // lobe = max(-(0.25 - 1/16), min(peak, 0.)) * con in double, con =
    // exp2(-sharpness) = 1 (FsrRcasCon, sharpness 0): every operand is a
    // float, so float min/max give the same value; 4. * lobe + 1. lies in
    // [0.25, 1], exact in double unless |4 * lobe| < 2^-29, where both forms
    // give 1, so one float rounding is the same
    const float lobe = fmaxf(-0.1875f, fminf(fmaxf(lx, fmaxf(ly, lz)), 0.0f));
    const float den = 4.0f * lobe + 1.0f;
    const float ox = (lobe * (((b.x + d.x) + hh.x) + f.x) + e.x) / den;
    const float oy = (lobe * (((b.y + d.y) + hh.y) + f.y) + e.y) / den;
    const float oz = (lobe * (((b.z + d.z) + hh.z) + f.z) + e.z) / den;
    dst[(size_t)y * w + x] = make_float4(ox, oy, oz, 1.0f);
}

}  // namespace kpt
