// kpt_post.h -- post-chain kernels and their device state.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kpt {

// Exposure state kept on the device between frames.
struct ExposureState {
    float avg_bin, avg_lum, adapted_lum, exposure_scalar, iso, shutter, pad0, pad1;
};

// Camera values read by the exposure program (ExposureValues, pod_types.hpp:9-33).
struct ExposureIn {
    float aperture, ev_comp, white_ev, black_ev;
    float min_iso, max_iso, min_shutter, max_shutter;
    float delta_ms, pad0, pad1, pad2;
};

__global__ void k_resolve(int npix, const float4* acc, const float4* albedo, float nsamples, float4* render);
__global__ void k_histogram(int W, int H, const float4* render, const float* thresholds, unsigned long long* hist);
__global__ void k_exposure(const unsigned long long* hist, ExposureState* st, ExposureIn in);
__global__ void k_bloom_down(const float4* src, int sw, int sh, float4* dst, int dw, int dh, int karis_avg);
__global__ void k_bloom_up(const float4* src, int sw, int sh, float4* dst, int dw, int dh, float blend);
__global__ void k_tonemap(int W, int H, const float4* render, const float4* bloom, int use_bloom, float final_blend,
                          const ExposureState* st, float fixed_scalar, int auto_exposure, float white_ev, float black_ev,
                          float4* image);
// computeEffects (kernels.cu:506-527): fisheye and chromatic aberration of
// the tonemapped image
__global__ void k_effects(int W, int H, const float4* src, float4* dst);
// upscale without FSR (upscale.cuh:260-291): bilinear read of the render at
// the output pixel's position
__global__ void k_upscale(const float4* src, int sw, int sh, float4* dst, int dw, int dh);
// the FSR 1.0 path (kpt_fsr.cu): EASU of the render to the output size, then
// RCAS of that image.  EasuCon holds FsrEasuCon's constants for one pair of
// sizes (upscale.cuh:18-62), computed on the host by easu_constants.
struct EasuCon {
    float c0x, c0y, c0z, c0w, c1x, c1y, c1z, c1w, c2x, c2y, c2z, c2w, c3x, c3y;
};
EasuCon easu_constants(int sw, int sh, int dw, int dh);
__global__ void k_easu(const float4* src, int sw, int sh, float4* dst, int dw, int dh, EasuCon con);
__global__ void k_rcas(const float4* src, int w, int h, float4* dst);

}  // namespace kpt
