// kpt_post.cu -- post chain of one frame (IEEE arithmetic, no fast maths).
//
//   k_resolve    addSample + modulateSamples (integrator.cuh:406-415,
//                kernels.cu:453-472): render = sum / n * 8-bit albedo;
//   k_histogram  histogramComputeKernel (histogram.cu:55-90): 256-bin
//                log-luminance histogram with centre-weighted metering,
//                accumulated as 2^-24 fixed point with warp-aggregated
//                integer atomics, so the result does not depend on the order
//                of the atomics; the bins the reference drops at the image
//                edge (a bin is flushed by the thread of the same index,
//                which exits when its pixel is outside the image) are
//                dropped here too;
//   k_exposure   histogramAverageLuminanceComputeKernel (histogram.cu:
//                93-154) + AutoExposureProgram (autoexposure_program.hpp:
//                18-94) + the exposure scalar of Renderer::setExposure
//                (renderer.cu:312-329), on the device in double precision:
//                no host round trip per frame;
//   k_bloom_down / k_bloom_up   downSample / upSampleCombine
//                (bloom.cu:90-146) over the mip chain (mipchain.cuh:17-59);
//   k_tonemap    computePostProcess (kernels.cu:475-504): bloom blend, Yxy
//                exposure, AgX (film.cuh:79-194).
// Every kernel but k_tonemap is bit-identical to the CPU oracle; k_tonemap
// differs only through CUDA's log2f/exp2f/powf.
#include "kpt_internal.h"
#include "kpt_post.h"

namespace kpt {

// RGBSpectrum::clampOutput (color.cuh:295-302) of every sample, added to the
// pixel's accumulation in sample order (integrator.cuh:406-415), as the
// reference accumulates one frame per sample.  Samples of a pixel whose camera
// ray misses all equal the pixel's sky radiance.
__global__ void k_accumulate(FrameParams F) {
    const int npix = F.W * F.H;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int j = F.hit_index[p];   // radiance is pixel-major: hit j's samples are contiguous
    float4 acc = F.acc ? F.acc[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int k = 0; k < F.nsamples; ++k) {
        float4 L = j < 0 ? F.pixel_sky[p] : F.radiance[(size_t)j * F.nsamples + k];
        if (isnan(L.x) || isnan(L.y) || isnan(L.z) || isinf(L.x) || isinf(L.y) || isinf(L.z))
            L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        else
            L = make_float4(fmaxf(0.0f, fminf(L.x, 1.0e8f)), fmaxf(0.0f, fminf(L.y, 1.0e8f)),
                            fmaxf(0.0f, fminf(L.z, 1.0e8f)), 0.0f);
        acc.x = __fadd_rn(acc.x, L.x);
        acc.y = __fadd_rn(acc.y, L.y);
        acc.z = __fadd_rn(acc.z, L.z);
        if (F.sample_out) F.sample_out[(size_t)k * npix + p] = L;
    }
    if (F.acc) F.acc[p] = make_float4(acc.x, acc.y, acc.z, 1.0f);
}

// --- temporal accumulation (kernels.cu:164-327) ------------------------------
// IEEE single precision in the reference's order of operations throughout.

// Mat4 row r times (x, y, z, w): c0[r]*x + c1[r]*y + c2[r]*z + c3[r]*w
// (matrix_maths.cuh:258-267)
__device__ __forceinline__ float trow(float4 r, float x, float y, float z, float w) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.x, x), __fmul_rn(r.y, y)), __fmul_rn(r.z, z)), __fmul_rn(r.w, w));
}

// RGBSpectrum::clampOutput (color.cuh:295-302), as k_accumulate applies it
__device__ __forceinline__ float4 clamp_sample(float4 L) {
    if (isnan(L.x) || isnan(L.y) || isnan(L.z) || isinf(L.x) || isinf(L.y) || isinf(L.z))
        return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return make_float4(fmaxf(0.0f, fminf(L.x, 1.0e8f)), fmaxf(0.0f, fminf(L.y, 1.0e8f)),
                       fmaxf(0.0f, fminf(L.z, 1.0e8f)), 0.0f);
}

__device__ __forceinline__ float4 tex_nearest(const float4* t, int W, int H, int x, int y) {   // cudaBoundaryModeClamp
    x = min(max(x, 0), W - 1);
    y = min(max(y, 0), H - 1);
    return t[(size_t)y * W + x];
}
__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {   // a + t * (b - a)
    return make_float4(__fadd_rn(a.x, __fmul_rn(t, __fsub_rn(b.x, a.x))), __fadd_rn(a.y, __fmul_rn(t, __fsub_rn(b.y, a.y))),
                       __fadd_rn(a.z, __fmul_rn(t, __fsub_rn(b.z, a.z))), __fadd_rn(a.w, __fmul_rn(t, __fsub_rn(b.w, a.w))));
}

// computeVelocity, then reprojectAccumulate without SUPER_SAMPLE: the pixel
// moves back by velocity * resolution; off screen, or when the depth of the
// previous frame there (nearest texel) differs from the reprojected
// distance by 4.5% or more, the history restarts; otherwise the previous
// image is read bilinearly (its history count from the nearest texel) and
// blended with weight 1 / min(history + 1, 16).
__global__ void k_temporal(TemporalParams T) {
    const int npix = T.W * T.H;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int x = p % T.W, y = p / T.W;
    const int j = T.hit_index[p];
    const float4 curr = clamp_sample(j < 0 ? T.pixel_sky[p] : T.radiance[(size_t)j * T.nsamples + T.sample]);
    const float4 vs = T.vis[p];
    if (T.depth_out) T.depth_out[p] = vs.w;
    float4 out = make_float4(curr.x, curr.y, curr.z, 0.0f);
    if (j >= 0) {
        const TemporalInst& I = T.inst[T.primary[p].inst];
        // computeVelocity (kernels.cu:164-192)
        const float lx = trow(I.inv[0], vs.x, vs.y, vs.z, 1.0f), ly = trow(I.inv[1], vs.x, vs.y, vs.z, 1.0f),
                    lz = trow(I.inv[2], vs.x, vs.y, vs.z, 1.0f);
        const float cw = trow(T.vp[3], vs.x, vs.y, vs.z, 1.0f);
        const float cx = __fdiv_rn(trow(T.vp[0], vs.x, vs.y, vs.z, 1.0f), cw);
        const float cy = __fdiv_rn(trow(T.vp[1], vs.x, vs.y, vs.z, 1.0f), cw);
        const float pw = trow(I.pm[3], lx, ly, lz, 1.0f);
        const float px = __fdiv_rn(trow(I.pm[0], lx, ly, lz, 1.0f), pw);
        const float py = __fdiv_rn(trow(I.pm[1], lx, ly, lz, 1.0f), pw);
        const float vx = __fsub_rn(__fdiv_rn(__fadd_rn(cx, 1.0f), 2.0f), __fdiv_rn(__fadd_rn(px, 1.0f), 2.0f));
        const float vy = __fsub_rn(__fdiv_rn(__fadd_rn(cy, 1.0f), 2.0f), __fdiv_rn(__fadd_rn(py, 1.0f), 2.0f));
        // reprojectAccumulate (kernels.cu:299-327)
        const float qx = __fsub_rn((float)x, __fmul_rn(vx, (float)T.W));
        const float qy = __fsub_rn((float)y, __fmul_rn(vy, (float)T.H));
        if (!(qx < 0.0f || qx >= (float)T.W || qy < 0.0f || qy >= (float)T.H)) {
            // testReprojection (kernels.cu:206-223)
            const int ix = (int)qx, iy = (int)qy;
            const float d2 = T.prev_depth[(size_t)min(max(iy, 0), T.H - 1) * T.W + min(max(ix, 0), T.W - 1)];
            const float wx = trow(I.prev_model[0], lx, ly, lz, 1.0f), wy = trow(I.prev_model[1], lx, ly, lz, 1.0f),
                        wz = trow(I.prev_model[2], lx, ly, lz, 1.0f);
            const float dx = __fsub_rn(T.prev_origin.x, wx), dy = __fsub_rn(T.prev_origin.y, wy),
                        dz = __fsub_rn(T.prev_origin.z, wz);
            const float d1 = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
            if (fabsf(__fsub_rn(d1, d2)) < __fmul_rn(d2, 0.045f)) {
                // DeviceTextureBuffer::textureReadBilinear (device_texture_buffer.cuh:42-80), alpha point-sampled
                const float ws = __fsub_rn(qx, (float)ix), wt = __fsub_rn(qy, (float)iy);
                const float4 c0 = tex_nearest(T.hist_in, T.W, T.H, ix, iy), c1 = tex_nearest(T.hist_in, T.W, T.H, ix + 1, iy);
                const float4 c2 = tex_nearest(T.hist_in, T.W, T.H, ix, iy + 1),
                             c3 = tex_nearest(T.hist_in, T.W, T.H, ix + 1, iy + 1);
                float4 prev = lerp4(lerp4(c0, c1, ws), lerp4(c2, c3, ws), wt);
                prev.w = c0.w;
                const float alpha = __fdiv_rn(1.0f, fminf(__fadd_rn(prev.w, 1.0f), 16.0f));
                out = make_float4(__fadd_rn(prev.x, __fmul_rn(alpha, __fsub_rn(curr.x, prev.x))),
                                  __fadd_rn(prev.y, __fmul_rn(alpha, __fsub_rn(curr.y, prev.y))),
                                  __fadd_rn(prev.z, __fmul_rn(alpha, __fsub_rn(curr.z, prev.z))),
                                  __fadd_rn(prev.w, 1.0f));
            }
        }
    }
    T.hist_out[p] = out;
}

__device__ __forceinline__ float qbyte(float v) {  // floatToByte then byteToFloat (packing.cuh:10-18)
    v = fmaxf(0.0f, fminf(v, 1.0f));
    uint32_t b = (uint32_t)__fmul_rn(v, 255.0f) & 0xFFu;
    return __fdiv_rn((float)b, 255.0f);
}

__global__ void k_resolve(int npix, const float4* acc, const float4* albedo, float nsamples, float4* render) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    float4 a = acc[i], al = albedo[i];
    render[i] = make_float4(__fmul_rn(__fdiv_rn(a.x, nsamples), qbyte(al.x)),
                            __fmul_rn(__fdiv_rn(a.y, nsamples), qbyte(al.y)),
                            __fmul_rn(__fdiv_rn(a.z, nsamples), qbyte(al.z)), 1.0f);
}

__device__ __forceinline__ float metering(int W, int H, int x, int y) {  // histogram.cu:35-48
    int cx = (int)__fdiv_rn((float)W, 2.0f), cy = (int)__fdiv_rn((float)H, 2.0f);
    float dx = (float)(cx - x), dy = (float)(cy - y);
    float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    dist = __fmul_rn(dist, __fdiv_rn(1.0f, 0.4f));
    float maxd = __fdiv_rn(fminf((float)W, (float)H), 2.0f);
    float nd = __fdiv_rn(dist, maxd);
    float y0 = fmaxf(0.0f, fminf(nd, 1.0f));     // smoothstep(0, 1, nd)
    float ss = __fmul_rn(__fmul_rn(y0, y0), __fsub_rn(3.0f, __fmul_rn(2.0f, y0)));
    return fmaxf(0.0f, fminf(__fsub_rn(1.0f, ss), 1.0f));
}

// One thread per pixel.  thresholds[k], k = 1..254, are the luminances where
// the bin index steps from k to k+1; thresholds[0] is the black cut-off.
__global__ void __launch_bounds__(256) k_histogram(int W, int H, const float4* render, const float* thresholds,
                                                   unsigned long long* hist) {
    __shared__ float thr[256];
    __shared__ unsigned long long sh[256];
    thr[threadIdx.x] = threadIdx.x < 255 ? thresholds[threadIdx.x] : __int_as_float(0x7f800000);
    sh[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int bin = -1;
    unsigned long long w = 0;
    if (i < W * H) {
        int x = i % W, y = i / W;
        float4 c = render[i];
        float Y = __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, c.x), __fmul_rn(0.7152f, c.y)), __fmul_rn(0.0722f, c.z));
        int b = 0;
        if (Y >= thr[0]) {          // binary search: number of thresholds k>=1 with Y >= thr[k]
            int lo = 1, hi = 255;   // first k in [1,255) with Y < thr[k]; thr[255] = inf
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (Y >= thr[mid]) lo = mid + 1; else hi = mid;
            }
            b = lo;                 // = 1 + count
            if (b > 255) b = 255;
        }
        int bx = (x >> 4) * 16 + (b & 15), by = (y >> 4) * 16 + (b >> 4);
        if (bx < W && by < H) {
            bin = b;
            float wf = b > 0 ? metering(W, H, x, y) : 1.0f;
            w = (unsigned long long)__float2ull_rn(__fmul_rn(wf, 16777216.0f));
        }
    }
    // warp aggregation: lanes with the same bin add their integer weights
    unsigned mask = __match_any_sync(0xffffffffu, bin);
    int leader = __ffs(mask) - 1;
    unsigned long long sum = 0;
    for (unsigned m = mask; m; m &= m - 1) sum += __shfl_sync(mask, w, __ffs(m) - 1);
    if (bin >= 0 && (int)(threadIdx.x & 31) == leader) atomicAdd(&sh[bin], sum);
    __syncthreads();
    if (sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

__global__ void k_exposure(const unsigned long long* hist, ExposureState* st, ExposureIn in) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long total = 0, wsum = 0;
    for (int b = 0; b < 256; ++b) { total += hist[b]; wsum += hist[b] * (unsigned long long)b; }
    double nonblack = (double)(total - hist[0]) / 16777216.0;
    if (nonblack < 0.001) nonblack = 0.001;
    double avg_bin = ((double)wsum / 16777216.0) / nonblack;
    double range = (double)in.white_ev - (double)in.black_ev;
    double t = (avg_bin - 1.0) / 254.0;
    t = t < 0 ? 0 : (t > 1 ? 1 : t);
    double avg_lum = exp2(t * range + (double)in.black_ev);
    double k = 1.0 - exp(-(double)in.delta_ms * 0.5);
    double last = (double)st->adapted_lum;
    float adapted = (float)(last + k * (avg_lum - last));
    double ev = log2(((double)adapted * 100.0) / 12.5) - (double)in.ev_comp + 6.0;
    double N = in.aperture;
    double shutter = 1.0 / (0.1 * 1000.0);
    double iso = (N * N * 100.0) / (shutter * exp2(ev));
    iso = fmin(fmax(iso, (double)in.min_iso), (double)in.max_iso);
    double evdiff = ev - log2((N * N * 100.0) / (shutter * iso));
    shutter = shutter * exp2(-evdiff);
    shutter = fmin(fmax(shutter, (double)in.min_shutter), (double)in.max_shutter);
    float isof = (float)iso, shf = (float)shutter;
    double lavg = (10.0 / 0.65) * ((N * N) / ((double)isof * (double)shf));
    st->avg_bin = (float)avg_bin;
    st->avg_lum = (float)avg_lum;
    st->adapted_lum = adapted;
    st->exposure_scalar = (float)(0.18 / lavg);
    st->iso = isof;
    st->shutter = shf;
}

__device__ __forceinline__ float4 f4lerp(float4 a, float4 b, float t) {
    return make_float4(__fadd_rn(a.x, __fmul_rn(t, __fsub_rn(b.x, a.x))), __fadd_rn(a.y, __fmul_rn(t, __fsub_rn(b.y, a.y))),
                       __fadd_rn(a.z, __fmul_rn(t, __fsub_rn(b.z, a.z))), __fadd_rn(a.w, __fmul_rn(t, __fsub_rn(b.w, a.w))));
}
__device__ __forceinline__ float4 at(const float4* img, int w, int h, int x, int y) {  // surf2Dread, clamp
    x = min(max(x, 0), w - 1);
    y = min(max(y, 0), h - 1);
    return __ldg(img + (size_t)y * w + x);
}
// DeviceTextureBuffer::textureReadBilinear (device_texture_buffer.cuh:42-80)
__device__ __forceinline__ float4 bilinear(const float4* img, int w, int h, float px, float py) {
    int dx = (int)px, dy = (int)py;
    float ws = __fsub_rn(px, (float)dx), wt = __fsub_rn(py, (float)dy);
    float4 a = f4lerp(at(img, w, h, dx, dy), at(img, w, h, dx + 1, dy), ws);
    float4 b = f4lerp(at(img, w, h, dx, dy + 1), at(img, w, h, dx + 1, dy + 1), ws);
    return f4lerp(a, b, wt);
}
__device__ __forceinline__ float lum(float4 c) {
    return __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, c.x), __fmul_rn(0.7152f, c.y)), __fmul_rn(0.0722f, c.z));
}
__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4mul(float4 a, float s) {
    return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ float4 karis(float4 a, float4 b, float4 c, float4 d) {  // bloom.cu:6-15
    float w0 = __fdiv_rn(1.0f, lum(a)), w1 = __fdiv_rn(1.0f, lum(b)), w2 = __fdiv_rn(1.0f, lum(c)), w3 = __fdiv_rn(1.0f, lum(d));
    float nw = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(__fadd_rn(w0, w1), w2), w3));
    return f4mul(f4add(f4add(f4add(f4mul(a, w0), f4mul(b, w1)), f4mul(c, w2)), f4mul(d, w3)), nw);
}
__device__ __forceinline__ float4 box4(float4 a, float4 b, float4 c, float4 d, bool ka) {
    return ka ? karis(a, b, c, d) : f4lerp(f4lerp(a, b, 0.5f), f4lerp(c, d, 0.5f), 0.5f);
}
__device__ __forceinline__ float4 clamp_out(float4 c) {  // clampOutput on rgb, alpha 1
    if (isnan(c.x) || isnan(c.y) || isnan(c.z) || isinf(c.x) || isinf(c.y) || isinf(c.z))
        return make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    return make_float4(fmaxf(0.0f, fminf(c.x, 1.0e8f)), fmaxf(0.0f, fminf(c.y, 1.0e8f)), fmaxf(0.0f, fminf(c.z, 1.0e8f)), 1.0f);
}

// 13 bilinear taps (bloom.cu:17-74); optional Karis average.
__global__ void k_bloom_down(const float4* src, int sw, int sh_, float4* dst, int dw, int dh, int karis_avg) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    float px = __fmul_rn(__fdiv_rn((float)x, (float)dw), (float)sw);
    float py = __fmul_rn(__fdiv_rn((float)y, (float)dh), (float)sh_);
    auto T = [&](float ox, float oy) { return bilinear(src, sw, sh_, __fadd_rn(px, ox), __fadd_rn(py, oy)); };
    float4 a = T(-2, 2), b = T(0, 2), c = T(2, 2), d = T(-2, 0), e = bilinear(src, sw, sh_, px, py), f = T(2, 0);
    float4 g = T(-2, -2), h = T(0, -2), i = T(2, -2);
    bool ka = karis_avg != 0;
    float4 hb1 = box4(a, b, d, e, ka), hb2 = box4(b, c, e, f, ka), hb3 = box4(d, e, g, h, ka), hb4 = box4(e, f, h, i, ka);
    float4 j = T(-1, 1), k = T(1, 1), l = T(-1, -1), m = T(1, -1);
    float4 hb5 = box4(j, k, l, m, ka);
    float4 r = f4lerp(hb5, f4lerp(f4lerp(hb1, hb2, 0.5f), f4lerp(hb3, hb4, 0.5f), 0.5f), 0.5f);
    dst[(size_t)y * dw + x] = clamp_out(r);
}

// 3x3 tent of bilinear taps blended into the finer level (bloom.cu:112-146).
__global__ void k_bloom_up(const float4* src, int sw, int sh_, float4* dst, int dw, int dh, float blend) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    float px = __fmul_rn(__fdiv_rn((float)x, (float)dw), (float)sw);
    float py = __fmul_rn(__fdiv_rn((float)y, (float)dh), (float)sh_);
    const float K[3][3] = {{0.0625f, 0.125f, 0.0625f}, {0.125f, 0.25f, 0.125f}, {0.0625f, 0.125f, 0.0625f}};
    float4 m = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int j = -1; j <= 1; ++j)
#pragma unroll
        for (int i = -1; i <= 1; ++i)
            m = f4add(m, f4mul(bilinear(src, sw, sh_, __fadd_rn(px, (float)i), __fadd_rn(py, (float)j)), K[j + 1][i + 1]));
    size_t o = (size_t)y * dw + x;
    dst[o] = clamp_out(f4lerp(dst[o], m, blend));
}

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}
__device__ __forceinline__ float srgb_enc(float v) {  // color.cuh:421-426
    return (v <= 0.0031308f) ? __fmul_rn(12.92f, v) : __fsub_rn(__fmul_rn(__fadd_rn(1.0f, 0.055f), powf(v, __fdiv_rn(1.0f, 2.4f))), 0.055f);
}

// computePostProcess (kernels.cu:475-504) with Film / AgX (film.cuh:79-194).
__global__ void k_tonemap(int W, int H, const float4* render, const float4* bloom, int use_bloom, float final_blend,
                          const ExposureState* st, float fixed_scalar, int auto_exposure, float white_ev, float black_ev,
                          float4* image) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    int sx = (int)__fmul_rn(__fdiv_rn(__fadd_rn((float)x, 0.5f), (float)W), (float)W);
    int sy = (int)__fmul_rn(__fdiv_rn(__fadd_rn((float)y, 0.5f), (float)H), (float)H);
    float4 c = at(render, W, H, sx, sy);
    if (use_bloom) c = f4lerp(c, at(bloom, W, H, sx, sy), final_blend);
    float expo = auto_exposure ? st->exposure_scalar : fixed_scalar;
    // RGB -> XYZ -> Yxy, exposure on Y, back (color.cuh:33-83)
    float X = dot3(0.4124564f, 0.3575761f, 0.1804375f, c.x, c.y, c.z);
    float Yv = dot3(0.2126729f, 0.7151522f, 0.0721750f, c.x, c.y, c.z);
    float Z = dot3(0.0193339f, 0.1191920f, 0.9503041f, c.x, c.y, c.z);
    float inv = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(X, Yv), Z));
    float Y = __fmul_rn(Yv, expo), cx = __fmul_rn(X, inv), cy = __fmul_rn(Yv, inv);
    float X2 = __fdiv_rn(__fmul_rn(Y, cx), cy);
    float Y2 = Y;
    float Z2 = (float)((double)Y * (1.0 - (double)cx - (double)cy) / (double)cy);
    float r = dot3(3.2404542f, -1.5371385f, -0.4985314f, X2, Y2, Z2);
    float g = dot3(-0.9692660f, 1.8760108f, 0.0415560f, X2, Y2, Z2);
    float b = dot3(0.0556434f, -0.2040259f, 1.0572252f, X2, Y2, Z2);
    // AgX (film.cuh:79-172)
    const float mn = log2f(__fmul_rn(exp2f(black_ev), 0.18f)), mx = log2f(__fmul_rn(exp2f(white_ev), 0.18f));
    const float dr = __fsub_rn(mx, mn);
    float r2 = fmaxf(dot3(0.6274f, 0.3293f, 0.0433f, r, g, b), 0.0f);
    float g2 = fmaxf(dot3(0.0691f, 0.9195f, 0.0113f, r, g, b), 0.0f);
    float b2 = fmaxf(dot3(0.0164f, 0.0880f, 0.8956f, r, g, b), 0.0f);
    float ir = dot3(0.856627153315983f, 0.0951212405381588f, 0.0482516061458583f, r2, g2, b2);
    float ig = dot3(0.137318972929847f, 0.761241990602591f, 0.101439036467562f, r2, g2, b2);
    float ib = dot3(0.11189821299995f, 0.0767994186031903f, 0.811302368396859f, r2, g2, b2);
    float v[3] = {ir, ig, ib};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float l = fmaxf(mn, fminf(log2f(v[k]), mx));
        float xx = __fdiv_rn(__fsub_rn(l, mn), dr);
        float x2 = __fmul_rn(xx, xx), x4 = __fmul_rn(x2, x2);
        float p = __fmul_rn(__fmul_rn(15.5f, x4), x2);
        p = __fsub_rn(p, __fmul_rn(__fmul_rn(40.14f, x4), xx));
        p = __fadd_rn(p, __fmul_rn(31.96f, x4));
        p = __fsub_rn(p, __fmul_rn(__fmul_rn(6.868f, x2), xx));
        p = __fadd_rn(p, __fmul_rn(0.4298f, x2));
        p = __fadd_rn(p, __fmul_rn(0.1191f, xx));
        v[k] = __fsub_rn(p, 0.00232f);
    }
    float luma = dot3(v[0], v[1], v[2], 0.2126f, 0.7152f, 0.0722f);
    float lin[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float nv = powf(__fadd_rn(__fmul_rn(v[k], 1.0f), 0.0f), 1.05f);
        float lk = __fadd_rn(luma, __fmul_rn(__fsub_rn(nv, luma), 1.25f));
        lin[k] = powf(lk, 2.4f);
    }
    float o0 = fmaxf(dot3(1.9648846919172409596f, -0.85594737466675834968f, -0.10883731725048386702f, lin[0], lin[1], lin[2]), 0.0f);
    float o1 = fmaxf(dot3(-0.29937618452442253746f, 1.3263980951083531115f, -0.02702191058393112346f, lin[0], lin[1], lin[2]), 0.0f);
    float o2 = fmaxf(dot3(-0.16440106280678278299f, -0.23819967517076844919f, 1.4025007379775505276f, lin[0], lin[1], lin[2]), 0.0f);
    image[(size_t)y * W + x] = make_float4(srgb_enc(o0), srgb_enc(o1), srgb_enc(o2), 1.0f);
}

}  // namespace kpt

namespace kpt {

// textureReadNearestUV (device_texture_buffer.cuh:35-40): texel
// (int)(uv * size), clamped at the edges
__device__ __forceinline__ float4 nearest_uv(const float4* t, int W, int H, float u, float v) {
    int x = (int)__fmul_rn(u, (float)W), y = (int)__fmul_rn(v, (float)H);
    x = min(max(x, 0), W - 1);
    y = min(max(y, 0), H - 1);
    return t[(size_t)y * W + x];
}

// computeEffects with getFishEyeUV (kernels.cu:340-374, 506-527): the pixel's
// fisheye position (power 1.65, radius bound to the corners), then the red
// and blue channels read at +- a chromatic offset that grows with the square
// of the distance from the centre.  IEEE arithmetic in the reference's order;
// rsqrt as 1 / sqrt, tan and pow are CUDA's.
__global__ void k_effects(int W, int H, const float4* src, float4* dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float res_x = (float)W, res_y = (float)H;
    const float px = __fdiv_rn((float)x, res_x), py = __fdiv_rn((float)y, res_x);
    const float prop = __fdiv_rn(res_x, res_y);
    const float mx = 0.5f, my = __fdiv_rn(0.5f, prop);
    const float dx = __fsub_rn(px, mx), dy = __fsub_rn(py, my);
    const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    const float power = 1.65f;
    const float bind = __fsqrt_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)));
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy))));
    const float t1 = tanf(__fmul_rn(r, power)), t2 = tanf(__fmul_rn(bind, power));
    float u = __fadd_rn(mx, __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(dx, inv), t1), bind), t2));
    float v = __fadd_rn(my, __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(dy, inv), t1), bind), t2));
    v = __fmul_rn(v, prop);
    const float ux = __fdiv_rn(__fadd_rn((float)x, 0.5f), res_x), uy = __fdiv_rn(__fadd_rn((float)y, 0.5f), res_y);
    const float ox = __fmul_rn(powf(__fmul_rn(fabsf(__fsub_rn(ux, 0.5f)), 2.0f), 2.0f), 0.01f);
    const float oy = __fmul_rn(powf(__fmul_rn(fabsf(__fsub_rn(uy, 0.5f)), 2.0f), 2.0f), 0.01f);
    const float rr = nearest_uv(src, W, H, __fadd_rn(u, ox), __fadd_rn(v, oy)).x;
    const float gg = nearest_uv(src, W, H, u, v).y;
    const float bb = nearest_uv(src, W, H, __fsub_rn(u, ox), __fsub_rn(v, oy)).z;
    dst[(size_t)y * W + x] = make_float4(rr, gg, bb, 1.0f);
}

}  // namespace kpt

namespace kpt {

// upscale (upscale.cuh:260-291, USE_FSR undefined): destination pixel
// (x, y) / destination size * source size, read with textureReadBilinear
// (device_texture_buffer.cuh:42-80) filtering all four channels.
__global__ void k_upscale(const float4* src, int sw, int sh, float4* dst, int dw, int dh) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const float px = __fmul_rn(__fdiv_rn((float)x, (float)dw), (float)sw);
    const float py = __fmul_rn(__fdiv_rn((float)y, (float)dh), (float)sh);
    const int ix = (int)px, iy = (int)py;
    const float ws = __fsub_rn(px, (float)ix), wt = __fsub_rn(py, (float)iy);
    const float4 c0 = tex_nearest(src, sw, sh, ix, iy), c1 = tex_nearest(src, sw, sh, ix + 1, iy);
    const float4 c2 = tex_nearest(src, sw, sh, ix, iy + 1), c3 = tex_nearest(src, sw, sh, ix + 1, iy + 1);
    dst[(size_t)y * dw + x] = lerp4(lerp4(c0, c1, ws), lerp4(c2, c3, ws), wt);
}

}  // namespace kpt
