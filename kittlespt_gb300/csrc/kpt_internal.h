// kpt_internal.h -- declarations shared by the library's translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "kpt_device.cuh"

namespace kpt {

constexpr int PATH_BLOCK = 128;    // threads per block of the shading kernels
constexpr int SHADE_MAX_BLOCK = 256;   // largest block k_shade is launched with (kpt_tuning.shade_block)
constexpr int SHADE_WINDOW = 2048;     // largest window of paths k_shade regroups by lobe family (kpt_tuning.group_lobes)
constexpr int TRACE_BLOCK = 128;   // threads per block of the ray kernels
// k_primary: a warp traces a TILE_W x (32 / TILE_W) tile of pixels, a
// block of PATH_BLOCK = 128 threads a 2 x 2 arrangement of them
#ifndef KPT_TILE_W
#define KPT_TILE_W 8
#endif
constexpr int TILE_W = KPT_TILE_W, TILE_H = 32 / KPT_TILE_W;
inline int primary_blocks(int W, int H) { return ((W + 2 * TILE_W - 1) / (2 * TILE_W)) * ((H + 2 * TILE_H - 1) / (2 * TILE_H)); }
#ifndef KPT_TRACE_MIN_BLOCKS
#define KPT_TRACE_MIN_BLOCKS 8
#endif
// ray kernels: resident blocks of TRACE_BLOCK threads per SM the register
// budget must allow (8: at most 64 registers, 32 warps per SM)
constexpr int TRACE_MIN_BLOCKS = KPT_TRACE_MIN_BLOCKS;

// Closest hit of a pixel's camera ray (the same for every sample: the
// reference discards its filter jitter, kernels.cu:397-402).
struct __align__(16) PrimaryRec {
    float t, u, v;
    int inst, tri, pad0, pad1, pad2;
};

// A path between two levels of the wave (64 B): the ray of its next segment,
// its throughput, the vertex it leaves and the sampler state.
struct __align__(16) PathRec {
    float4 o_pb;        // ray origin, BSDF pdf of the sampled direction (MIS at a light hit)
    float4 d_seed;      // ray direction, sampler seed (bits)
    float4 beta_item;   // throughput, work item (bits)
    float4 prev;        // previous vertex, unused
};

// A shadow ray and the radiance it carries if nothing blocks it (48 B).
struct __align__(16) ShadowRec {
    float4 o_tmax;      // origin, tmax
    float4 d_item;      // direction, work item (bits)
    float4 contrib;     // radiance added to the item when unoccluded
};

// per-level counters of a wave, LEVEL_WORDS ints per level: paths entering
// the level, sun shadow rays, light shadow rays, then the fetch counters of
// the extension and shadow ray queues
constexpr int LEVEL_WORDS = 8;

// Everything the kernels of one frame read; passed by value.
struct FrameParams {
    SceneView scene;
    SkyParams sky;
    float4 inv_proj[4];        // rows of the inverse projection
    float4 inv_view[3];        // rows 0-2 of the inverse view
    float3 cam_pos;
    int W, H;
    int sample0, nsamples;     // reference frame indices sample0 .. sample0+nsamples-1
    int max_depth, rng_order;
    const float3* sun_radiance;
    float4* acc;               // [H*W] running sum of samples (rgb), may be null
    float4* albedo;            // [H*W] visible-surface albedo, may be null
    int4* first_hit;           // [H*W] (instance, triangle, t bits, 0), may be null
    float4* vis;               // [H*W] visible surface (position, distance; INF distance for a miss), may be null
    float4* sample_out;        // [nsamples][H*W] clamped per-sample radiance, may be null
    unsigned long long* counters;   // [16] box tests, triangle tests, instance transforms, overflows
                                    //      of the extension rays, the camera rays, the shadow rays;
                                    //      then extension rays, shadow rays, camera rays traced
    // work buffers of the frame
    PrimaryRec* primary;       // [H*W]
    int* hit_list;             // [H*W] pixels whose camera ray hits, compacted
    int* hit_index;            // [H*W] position in hit_list, -1 for a miss
    int* miss_list;            // [H*W] pixels whose camera ray misses, compacted
    int* counts;               // [0] hits, [1] misses, [2] queued sky evaluations (zeroed per frame)
    float4* pixel_sky;         // [H*W] sky radiance (times LeSun) of a missing camera ray
    float4* radiance;          // [hits][nsamples] path radiance before clamping (item = hit * nsamples + sample)
    float4* sky_queue;         // [2 per entry] (item bits, direction), (throughput, 0)
    // the wave: up to `cap` paths advanced one level per launch triple
    PathRec* paths[2];         // [cap] paths entering even / odd levels
    PrimaryRec* hits;          // [cap] closest hits of the paths entering a level
    ShadowRec* shadow;         // [cap] shadow rays of a level: sun rays from the front, light rays from the back
    int* level_counts;         // [LEVEL_WORDS * (max_depth + 2)] zeroed per wave; word 5: sky queue
                               // length after level l (of level max_depth + 1: at the wave's start)
    PathRec* unsorted;         // [cap] k_shade's continuations before the octant sort, null: no sort
    int* octants;              // [16 * (max_depth + 2)] per level: paths per direction octant, cursors
    int cap;
    int group_lobes;           // k_shade regroups windows of this many paths by lobe family (levels >= 1); 0 = off
};

// ---------------------------------------------------------------------------
// path-replay adjoint (kpt_adjoint.cu)

constexpr int ADJ_MAX_VERTICES = 17;   // max_depth <= 16
constexpr int ADJ_SKY_PARAMS = 6;      // Rayleigh r, g, b, Mie, Rayleigh height, Mie height

// One path vertex as the replay saw it, everything that is held fixed (for
// the FP64 oracle's finite differences): 192 B.
enum { ADJ_FIRST = 1, ADJ_BACKFACE = 2, ADJ_LAST = 4, ADJ_ESCAPED = 8, ADJ_NEE_UNOCCLUDED = 16 };
struct __align__(16) AdjRec {
    int item, vertex, material, flags;
    int lobe, nee, pixel, pad0;       // sampled lobe (LOBE_*), light sample (0 none, 1 sun, 2 light)
    float alb_tex[3], rough_tex;      // texture factors of albedo and roughness
    float metallic, transmission, ior, eta;
    float wo[3], cosw;                // local wo; |ng . wi| of the sampled direction
    float wi[3], pdf;                 // local sampled direction and its pdf
    float wm[3], rr;                  // local microfacet normal of the sample; roulette factor 1/(1-q)
    float nwi[3], ncos;               // local light-sample direction and its cosine factor
    float nfac[3], pad1;              // light sample: sun 6e5/(pdf 0.5); area light Le w/(p 0.5)
    float emit[3], pad2;              // emission term Le * w (no parameter)
    float g[3], pad3;                 // adjoint weight of the sample (masked by the clamp)
    float miss[3], pad4;              // direction of the escaping ray (ADJ_ESCAPED)
};

struct AdjParams {
    const float4* adjoint;   // [H*W] dLoss/d(mean clamped radiance), rgb
    double* grad;            // [4 * nmat + ADJ_SKY_PARAMS]
    float4* image;           // [H*W] mean clamped radiance, may be null
    float3* sun_J;           // [ADJ_SKY_PARAMS] d(sun radiance)/d(sky parameters)
    AdjRec* rec;             // frozen-path records, may be null
    int* rec_count;
    int max_rec;
    int nmat;
    // escapes whose sky Jacobian is evaluated in double (near the horizon or
    // the sun): (direction, gradient weight) pairs for k_adjoint_sky_d; null:
    // evaluated where they occur
    float4* skyq;
    int* skyq_count;
    int skyq_cap;
    // the other escapes' single-precision Jacobians, the same way, for
    // k_adjoint_sky_f
    float4* skyqf;
    int* skyqf_count;
    int skyqf_cap;
    // the wavefront replay: per vertex AV_FIELDS float4 fields, field f of
    // level l, path slot i at vr[(l * cap + i) * AV_FIELDS + f]; per path slot
    // its end (direction, vertex count; throughput, escaped) at vend[2 i],
    // vend[2 i + 1]; vis[l * cap + i] = 1 when the light sample of vertex l
    // is unoccluded
    float4* vr;
    float4* vend;
    float4* vsky;              // [cap] the sky radiance of an escaped path's last ray
    int* esc;                  // [cap] slots of the wave's escaped paths, esc_count of them
    int* esc_count;
    unsigned char* vis;
    // the split adjoint: each path's radiance, stored by the forward half's
    // sweep (lpath_ready 0) and read by the backward half's (1); null: summed
    float4* lpath;
    int lpath_ready;
};

// fields of the wavefront replay's vertex record
enum AdjVField { AV_BETA, AV_EMIT, AV_FCOS, AV_K, AV_DA, AV_DAL, AV_W, AV_DWA, AV_DWR, AV_FIELDS };

// Frisvad basis applied to l, IEEE arithmetic (maths/matrix_maths.cuh:375-396).
__device__ __forceinline__ float3 onb_apply_exact(float3 n, float3 l) {
    float3 c0, c1;
    if (n.z < -0.999805696f) {
        c0 = make_float3(0.0f, -1.0f, 0.0f);
        c1 = make_float3(-1.0f, 0.0f, 0.0f);
    } else {
        float a = __frcp_rn(xa(1.0f, n.z));
        float b = xm(xm(-n.x, n.y), a);
        c0 = make_float3(xs(1.0f, xm(xm(n.x, n.x), a)), b, -n.x);
        c1 = make_float3(b, xs(1.0f, xm(xm(n.y, n.y), a)), -n.y);
    }
    return make_float3(xa(xa(xm(c0.x, l.x), xm(c1.x, l.y)), xm(n.x, l.z)),
                       xa(xa(xm(c0.y, l.x), xm(c1.y, l.y)), xm(n.y, l.z)),
                       xa(xa(xm(c0.z, l.x), xm(c1.z, l.y)), xm(n.z, l.z)));
}

// One job of a batch whose extension and shadow rays are traced from one
// queue spanning the jobs (kpt_submit_batch): where the job's wave buffers
// are and where its scene sits in the batch's merged scene.
struct __align__(16) BatchJob {
    float4 tlas_lo, tlas_hi;        // root bounds of the job's TLAS
    const PathRec* paths[2];
    PrimaryRec* hits;
    const ShadowRec* shadow;
    float4* radiance;
    int* level_counts;
    const int* counts;              // counts[2]: the job's sky queue length
    int tlas_root;                  // merged TLAS: root node, or -(instance) - 1
    int ninst, inst_base, cap, max_depth, pad[3];
};

// The ray queues of one level of a batch: the prefix sums of the jobs'
// extension rays (paths entering the level) and shadow rays, and their
// fetch counters (written by k_batch_level).
struct BatchQueues {
    int* ext_prefix;    // [njobs + 1]
    int* shd_prefix;    // [njobs + 1]
    int* fetch;         // [2]: extension, shadow
    const BatchJob* jobs;
    int njobs;
};

// kernels (kpt_path.cu, fast maths)
__global__ void k_primary(FrameParams F);
__global__ void k_primary_sky(FrameParams F);
__global__ void k_shade(FrameParams F, int level, long long wave0);        // blocks of <= PATH_BLOCK threads
__global__ void k_shade_wide(FrameParams F, int level, long long wave0);   // blocks of <= SHADE_MAX_BLOCK threads
// levels >= 1 (with F.group_lobes > 0 each window of paths regrouped by lobe family)
__global__ void k_shade_bounce(FrameParams F, int level, long long wave0);
__global__ void k_shade_bounce_wide(FrameParams F, int level, long long wave0);
__global__ void k_extend(FrameParams F, int level);
__global__ void k_count_rays(FrameParams F);   // adds the wave's ray counts to counters[12..13]
__global__ void k_sort_count(FrameParams F, int level);     // octant histogram of the paths entering level
__global__ void k_sort_scatter(FrameParams F, int level);   // paths entering level, grouped by octant
__global__ void k_shadow(FrameParams F, int level);
__global__ void k_sky_queue(FrameParams F, int level);
__global__ void k_sky_constants(FrameParams F, float3* sun_radiance);
// a batch's queues: after every job's k_shade(level), the extension rays of
// level + 1 and the shadow rays of level (one block)
__global__ void k_batch_level(BatchQueues Q, int level);
__global__ void k_extend_batch(SceneView s, BatchQueues Q, int level, unsigned long long* counters);
__global__ void k_shadow_batch(SceneView s, BatchQueues Q, int level, unsigned long long* counters);
// the merged scene of a batch: one job's BLAS / TLAS nodes, meshes and
// instances with their indices moved by the job's offsets
__global__ void k_merge_nodes(const BvhNode* src, int n, BvhNode* dst, int node_add, int leaf_add);
__global__ void k_merge_meshes(const MeshRec* src, int n, MeshRec* dst, int node_add, int tri_add);
__global__ void k_merge_inst(const InstRec* src, int n, InstRec* dst, int mesh_add);
// kpt_adjoint.cu (fast maths)
__global__ void k_adjoint_constants(FrameParams F, AdjParams A);
__global__ void k_sky_grad(SkyParams P, int n, const float3* dirs, float3* out);
__global__ void k_adjoint_miss(FrameParams F, AdjParams A);
__global__ void k_adjoint_rec(FrameParams F, AdjParams A);   // also writes the frozen-path records
__global__ void k_adjoint_sky_d(FrameParams F, AdjParams A);
__global__ void k_adjoint_sky_f(FrameParams F, AdjParams A);
__global__ void k_adj_shade(FrameParams F, AdjParams A, int level, long long wave0);
__global__ void k_adj_shadow(FrameParams F, AdjParams A, int level);
__global__ void k_adj_sweep(FrameParams F, AdjParams A, long long wave0);
__global__ void k_adj_sky(FrameParams F, AdjParams A, long long wave0);
// kpt_post.cu (IEEE): clamp and add the samples of each pixel in sample order
// Temporal accumulation (kernels.cu:164-327): per instance, the matrices of
// computeVelocity and testReprojection for one frame, rows of column-major
// Mat4s (row r = column 0..3 entries r).
struct TemporalInst {
    float4 inv[3];             // curr_inv_model_matrix rows 0..2 (object <- world)
    float4 prev_model[3];      // prev_inv_model_matrix.inverse(), rows 0..2
    float4 pm[4];              // prev view-projection * prev model, rows 0..3
};
// The same matrices for k_temporal_gpu, which inverts them itself: per
// instance the inverse model matrices the host holds (columns).
struct TemporalGpuInst {
    float4 inv_model[4];       // curr_inv_model_matrix
    float4 prev_inv_model[4];  // prev_inv_model_matrix
    int tri_base;              // the instance's mesh: its first triangle in tri_leaf / the leaf-order arrays
    int pad0, pad1, pad2;
};
// One reference frame of the temporal path: the clamped sample `sample` of
// every pixel blended into hist_in reprojected, written to hist_out.
struct TemporalParams {
    int W, H, sample, nsamples;
    const int* counts;         // [0]: camera rays that hit (slots of a sample in `radiance`)
    const int* hit_index;      // pixel -> hit slot, -1: the camera ray missed
    const PrimaryRec* primary; // per pixel: first hit (instance)
    const float4* radiance;    // [nhit][nsamples] path radiance
    const float4* pixel_sky;   // per pixel: the sky of a missing camera ray
    const float4* vis;         // per pixel: visible surface position, distance
    const TemporalInst* inst;
    float4 vp[4];              // current view-projection rows
    float3 prev_origin;        // previous camera position (prev_inv_view column 3)
    const float* prev_depth;   // per pixel: visible-surface distance of the previous frame
    float* depth_out;          // per pixel: this frame's distance for the next frame, may be null
    const float4* hist_in;
    float4* hist_out;
    // k_temporal_gpu: the camera's inverse projection and view matrices of
    // this frame and of the previous one (columns), the instances' inverses
    const TemporalGpuInst* ginst;
    float4 inv_proj[4], inv_view[4], prev_inv_proj[4], prev_inv_view[4];
    // and the visible surface as that build computes it: the hit
    // triangle's vertices (leaf-order triangles: v0, v1 - v0, v2 - v0) and
    // each mesh's triangle id -> leaf-order slot (tri_leaf[tri_base + id])
    const float4* tris;
    const int* tri_leaf;
};
__global__ void k_temporal(TemporalParams T);       // kpt_post.cu, IEEE
__global__ void k_temporal_gpu(TemporalParams T);   // kpt_path.cu, the reference GPU build's arithmetic
__global__ void k_accumulate(FrameParams F);
__global__ void k_sky(SkyParams P, int n, const float3* dirs, float3* out);
__global__ void k_trace(SceneView s, int n, const float3* o, const float3* d, float tmin, float tmax,
                        int* inst, int* tri, float* t, float2* uv, int* next, unsigned long long* counters);
__global__ void k_occluded(SceneView s, int n, const float3* o, const float3* d, float tmin, const float* tmax,
                           uint8_t* out, int* next, unsigned long long* counters);
__global__ void k_sun_constants_gpu(float phi, float theta, float diameter, float* out);
__global__ void k_trace_chains(SceneView s, int n, const float3* o, const float3* d, int nbounces, int* inst,
                               int* tri, float* t, int* next, unsigned long long* counters);

}  // namespace kpt
