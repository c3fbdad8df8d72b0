// ref_gpu_harness.cu -- drives the reference's own CUDA megakernel
// (computePathTraceSamplesMegaKernel through launchPathTraceComputeMegaKernel,
// shaders/kernels.cu:29-41 and :385-451) on the GPU, as the GPU baseline of
// the benchmark and as a GPU oracle for the tests.
//
// TEST INFRASTRUCTURE ONLY.  This is our driver; the code it runs is the
// reference's, compiled unmodified with its GPU build's -use_fast_math by
// oracle/build_ref.sh (gpu) into oracle/_ref/libkpt_ref_gpu.so, never
// committed.  What differs from Renderer::executeRendering
// (renderer.cu:103-195), and why:
//   * the frame surfaces are CUDA arrays created for surface load/store
//     instead of OpenGL textures mapped through interop (no graphics stack
//     here); the kernel reads and writes them through the same surface calls;
//   * the scene buffers are copied to device memory (cudaMalloc) instead of
//     staying in the reference's managed memory, so the kernel reads them
//     from HBM from its first launch;
//   * only the path-tracing megakernel runs: the post launchers are not
//     called, and the TLAS, which the reference rebuilds on the host every
//     frame, is built once (nothing moves between frames here).
//
// Safety guard: the reference's traversal keeps 16-entry node stacks
// (shaders/blas.cuh:37, shaders/tlas.cuh:10) and writes past them if a tree
// needs more.  A pop-one, push-two depth-first traversal holds at most one
// pending node per level above the current one, so an interior node of depth
// d needs at most d + 2 entries.  refgpu_scene_create measures the deepest
// interior node of every BLAS and of the TLAS and refuses (returns null, with
// the depth in refgpu_last_error) any scene with one deeper than 14, before
// any kernel runs.

#include "error_check.cu"
#include "shaders/kernels.cu"
#include "shaders/tlas.cu"
#include "shaders/interaction.cu"
#include "shaders/light.cu"
#include "shaders/material.cu"
#include "shaders/histogram.cu"
#include "shaders/bloom.cu"
#include "shaders/texture.cu"
#include "as_builder.cuh"
#include "pod_types.hpp"
#include "ref_records.h"
#include "ref_scene.h"

#include <array>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_error;

int fail(const std::string& m) {
    g_error = m;
    return -1;
}

#define RG_CUDA(x)                                                                      \
    do {                                                                                \
        cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int REF_STACK = 16;

template <class T>
struct DevArr {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t upload(const thrust::universal_vector<T>& v) {
        n = v.size();
        if (!n) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * n);
        if (e != cudaSuccess) return e;
        return cudaMemcpy(p, thrust::raw_pointer_cast(v.data()), sizeof(T) * n, cudaMemcpyDefault);
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct FrameSurface {
    cudaArray_t arr = nullptr;
    cudaSurfaceObject_t obj = 0;
};

struct GpuScene {
    RefScene host;   // the reference's buffers as its builders left them
    DevArr<TLASNode> tlasnodes;
    DevArr<BLAS2> blas;
    DevArr<BVH2Node> nodes;
    DevArr<int32_t> tri_index;
    DevArr<TriangleMesh> meshes;
    DevArr<Light> lights;
    DevArr<Triangle> tris;
    DevArr<Material> materials;
    DevArr<Texture> textures;
    DevArr<uint8_t> pixels;
    float* histogram = nullptr;        // histogram_buffer, scene_average_luminance: not used by the megakernel
    float* avg_lum = nullptr;
    int W = 0, H = 0;
    FrameSurface surf[9];              // output, render, accumulation, gbuffer, prev_gbuffer, vbuffer, debug, backbuffer, bloom
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ShaderData sd;
    int blas_depth = 0, tlas_depth = 0;
    std::vector<std::array<float, 16>> models;   // each mesh's current model matrix (column-major)
};

// deepest interior node below `root` (root depth 0; -1 for a leaf root)
int blas_interior_depth(const thrust::universal_vector<BVH2Node>& nodes, int root) {
    std::vector<std::pair<int, int>> st{{root, 0}};
    int deepest = -1;
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        const BVH2Node& b = nodes[n];
        if (b.isLeaf()) continue;
        deepest = std::max(deepest, d);
        st.push_back({b.left_child_node_index_or_tris_index_start_index, d + 1});
        st.push_back({b.left_child_node_index_or_tris_index_start_index + 1, d + 1});
    }
    return deepest;
}

int tlas_interior_depth(const thrust::universal_vector<TLASNode>& nodes, int root) {
    if (root < 0) return -1;
    std::vector<std::pair<int, int>> st{{root, 0}};
    int deepest = -1;
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        const TLASNode& t = nodes[n];
        if (t.isleaf()) continue;
        deepest = std::max(deepest, d);
        // the child indices of TLASNode::getChildrenIndex (a device function)
        st.push_back({(int)(t.left_right_index & 0xFFFFu), d + 1});
        st.push_back({(int)((t.left_right_index >> 16) & 0xFFFFu), d + 1});
    }
    return deepest;
}

void free_surfaces(GpuScene& g) {
    for (FrameSurface& s : g.surf) {
        if (s.obj) cudaDestroySurfaceObject(s.obj);
        if (s.arr) cudaFreeArray(s.arr);
        s = FrameSurface();
    }
    g.W = g.H = 0;
}

int clear_surface(const FrameSurface& s, int W, int H) {
    std::vector<float4> zero((size_t)W * H, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    RG_CUDA(cudaMemcpy2DToArray(s.arr, 0, 0, zero.data(), (size_t)W * sizeof(float4), (size_t)W * sizeof(float4), H,
                                cudaMemcpyHostToDevice));
    return 0;
}

// the frame textures of RendererResource (renderer_resource.cuh), as
// RGBA32F surfaces of the render resolution
int ensure_surfaces(GpuScene& g, int W, int H) {
    if (g.W == W && g.H == H) return 0;
    free_surfaces(g);
    cudaChannelFormatDesc cd = cudaCreateChannelDesc<float4>();
    for (FrameSurface& s : g.surf) {
        RG_CUDA(cudaMallocArray(&s.arr, &cd, W, H, cudaArraySurfaceLoadStore));
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = s.arr;
        RG_CUDA(cudaCreateSurfaceObject(&s.obj, &rd));
        if (clear_surface(s, W, H)) return -1;
    }
    g.W = W;
    g.H = H;
    DeviceTextureBuffer* tex[9] = {&g.sd.output_texture, &g.sd.render_texture, &g.sd.accumulation_texture,
                                   &g.sd.gbuffer_texture, &g.sd.prev_gbuffer_texture, &g.sd.vbuffer_texture,
                                   &g.sd.debug_texture, &g.sd.backbuffer_texture, &g.sd.bloom_texture};
    for (int k = 0; k < 9; ++k) {
        tex[k]->dimensions = make_int2(W, H);
        tex[k]->m_surface_object = g.surf[k].obj;
    }
    g.sd.render_resolution = make_int2(W, H);
    g.sd.output_resolution = make_int2(W, H);
    return 0;
}

void set_view(GpuScene& g, const float* inv_proj, const float* inv_view, const void* env, const void* settings) {
    const EnvRecord& e = *(const EnvRecord*)env;
    const SettingsRecord& st = *(const SettingsRecord*)settings;
    ShaderData& sd = g.sd;
    sd.procedural_environment_data.sun_angular_diameter_rad = e.sun_angular_diameter;
    sd.procedural_environment_data.sun_phi_rad = e.sun_phi;
    sd.procedural_environment_data.sun_theta_rad = e.sun_theta;
    sd.procedural_environment_data.sun_emission_factor = e.sun_emission_factor;
    sd.renderer_settings = RendererSettings();
    sd.renderer_settings.integrator_max_ray_depth = st.max_depth;
    Camera cam;
    cam.setView(mat_from(inv_proj), mat_from(inv_view));   // Renderer::setView (renderer.cu:342-354)
    cam.setView(cam.curr_inv_projection_matrix, cam.curr_inv_view_matrix);   // the per-frame update (:186-190)
    sd.scene_camera = cam;
}

// Camera rays of the megakernel (same 8x8 launch, getShadingJob, the
// discarded filter draw is irrelevant here) and their closest hits through
// Integrator::intersect with Li's interval [0, inf) (integrator.cuh:270).
__global__ void k_refgpu_first_hits(const ShaderData sd, int* prim, int* inst, float* t) {
    ShadingJob job = getShadingJob(sd.render_resolution);
    if (job.is_invalid) return;
    float2 ndc = 2.0f * job.uv_coord - 1.0f;
    Ray ray = sd.scene_camera.generateRay(ndc);
    DebugData dbg;
    Intersection h = Integrator::intersect(sd, ray, 0.0f, INFINITY, dbg);
    const size_t p = (size_t)job.pixel_coord.y * sd.render_resolution.x + job.pixel_coord.x;
    prim[p] = h.primitive_id;
    inst[p] = h.instance_id;
    t[p] = h.distance;
}

}  // namespace

extern "C" {

void refgpu_scene_destroy(void* h);

const char* refgpu_last_error(void) { return g_error.c_str(); }

// Scene from the same arrays as ref_scene_create (ref_harness.cpp), on
// `device`.  Null on failure, with the reason in refgpu_last_error; a tree
// too deep for the reference's stacks is a failure (see the guard above).
void* refgpu_scene_create(int device, int ntris, const float* pos, const float* nrm, const float* uv,
                          const int* mat, int nmeshes, const int* mesh_off, const int* mesh_cnt,
                          const float* models, int nmaterials, const void* materials, int ntextures,
                          const int* tex_desc, long long npixels, const unsigned char* pixels) {
    if (cudaSetDevice(device) != cudaSuccess) {
        fail("cudaSetDevice failed");
        return nullptr;
    }
    GpuScene* g = new GpuScene();
    ref_replay_load_scene(&g->host, ntris, pos, nrm, uv, mat, nmeshes, mesh_off, mesh_cnt, models, nmaterials,
                          materials, ntextures, tex_desc, npixels, pixels);
    g->models.resize(nmeshes);
    for (int mi = 0; mi < nmeshes; ++mi) std::memcpy(g->models[mi].data(), models + 16 * mi, 64);
    RefScene& r = g->host;
    for (size_t i = 0; i < r.blas.size(); ++i)
        g->blas_depth = std::max(g->blas_depth, blas_interior_depth(r.nodes, r.blas[i].bvhnode_root_index));
    g->tlas_depth = tlas_interior_depth(r.tlasnodes, r.sd.top_level_acceleration_structure.tlasnode_root_index);
    if (g->blas_depth + 2 > REF_STACK || g->tlas_depth + 2 > REF_STACK) {
        fail("tree depth: deepest interior BLAS node " + std::to_string(g->blas_depth) + ", TLAS node " +
             std::to_string(g->tlas_depth) + "; the reference's 16-entry stacks hold depth <= 14");
        delete g;
        return nullptr;
    }
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = g->tlasnodes.upload(r.tlasnodes);
    if (e == cudaSuccess) e = g->blas.upload(r.blas);
    if (e == cudaSuccess) e = g->nodes.upload(r.nodes);
    if (e == cudaSuccess) e = g->tri_index.upload(r.tri_index);
    if (e == cudaSuccess) e = g->meshes.upload(r.meshes);
    if (e == cudaSuccess) e = g->lights.upload(r.lights);
    if (e == cudaSuccess) e = g->tris.upload(r.tris);
    if (e == cudaSuccess) e = g->materials.upload(r.materials);
    if (e == cudaSuccess) e = g->textures.upload(r.textures);
    if (e == cudaSuccess) e = g->pixels.upload(r.pixels);
    if (e == cudaSuccess) e = cudaMalloc(&g->histogram, 256 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->histogram, 0, 256 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->avg_lum, sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->avg_lum, 0, sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev[1]);
    if (e != cudaSuccess) {
        fail(std::string("scene upload: ") + cudaGetErrorString(e));
        refgpu_scene_destroy(g);
        return nullptr;
    }
    // RendererResource::updateResource (renderer_resource.cuh:28-40), device copies
    ShaderData& sd = g->sd;
    sd.top_level_acceleration_structure = r.sd.top_level_acceleration_structure;
    sd.tlas_nodes_buffer = Buffer<TLASNode>(g->tlasnodes.p, g->tlasnodes.n);
    sd.blas_buffer = Buffer<BLAS2>(g->blas.p, g->blas.n);
    sd.bvh_nodes_buffer = Buffer<BVH2Node>(g->nodes.p, g->nodes.n);
    sd.triangle_index_buffer = Buffer<int32_t>(g->tri_index.p, g->tri_index.n);
    sd.meshes_buffer = Buffer<TriangleMesh>(g->meshes.p, g->meshes.n);
    sd.lights_buffer = Buffer<Light>(g->lights.p, g->lights.n);
    sd.triangles_buffer = Buffer<Triangle>(g->tris.p, g->tris.n);
    sd.materials_buffer = Buffer<Material>(g->materials.p, g->materials.n);
    sd.texture_buffer = Buffer<Texture>(g->textures.p, g->textures.n);
    sd.pixel_buffer = Buffer<uint8_t>(g->pixels.p, g->pixels.n);
    sd.histogram_buffer = Buffer<float>(g->histogram, 256);
    sd.scene_average_luminance = g->avg_lum;
    return g;
}

void refgpu_scene_destroy(void* h) {
    GpuScene* g = (GpuScene*)h;
    if (!g) return;
    free_surfaces(*g);
    g->tlasnodes.release(); g->blas.release(); g->nodes.release(); g->tri_index.release();
    g->meshes.release(); g->lights.release(); g->tris.release(); g->materials.release();
    g->textures.release(); g->pixels.release();
    if (g->histogram) cudaFree(g->histogram);
    if (g->avg_lum) cudaFree(g->avg_lum);
    for (cudaEvent_t e : g->ev) if (e) cudaEventDestroy(e);
    delete g;
}

// deepest interior BLAS node, deepest interior TLAS node
void refgpu_tree_depth(void* h, int* out) {
    GpuScene* g = (GpuScene*)h;
    out[0] = g->blas_depth;
    out[1] = g->tlas_depth;
}

// Renders frames frame0 .. frame0+nframes-1 with the megakernel, one
// launchPathTraceComputeMegaKernel per frame (it synchronises), each timed
// with CUDA events around the launch into ms[f] (may be null).  clear = 1
// zeroes the accumulation surface first.  accum (may be null) receives the
// accumulation surface afterwards: [H][W] RGBA, rgb = the sum of the frames'
// clamped samples since the last clear.
int refgpu_render(void* h, const float* inv_proj, const float* inv_view, const void* env, const void* settings,
                  int W, int H, int frame0, int nframes, int clear, float* accum, float* ms) {
    GpuScene* g = (GpuScene*)h;
    if (!g || W <= 0 || H <= 0 || nframes < 0) return fail("refgpu_render: bad arguments");
    if (ensure_surfaces(*g, W, H)) return -1;
    set_view(*g, inv_proj, inv_view, env, settings);
    if (clear && clear_surface(g->surf[2], W, H)) return -1;
    for (int f = 0; f < nframes; ++f) {
        g->sd.frame_index = frame0 + f;
        RG_CUDA(cudaEventRecord(g->ev[0], 0));
        KittlesPT::launchPathTraceComputeMegaKernel(g->sd);
        RG_CUDA(cudaEventRecord(g->ev[1], 0));
        RG_CUDA(cudaEventSynchronize(g->ev[1]));
        if (ms) RG_CUDA(cudaEventElapsedTime(ms + f, g->ev[0], g->ev[1]));
    }
    if (accum)
        RG_CUDA(cudaMemcpy2DFromArray(accum, (size_t)W * sizeof(float4), g->surf[2].arr, 0, 0,
                                      (size_t)W * sizeof(float4), H, cudaMemcpyDeviceToHost));
    return 0;
}

// Closest hits of the megakernel's camera rays: prim (global triangle index
// in the reference's numbering), inst (mesh) and t, [H][W] each.
int refgpu_first_hits(void* h, const float* inv_proj, const float* inv_view, const void* env, const void* settings,
                      int W, int H, int* prim, int* inst, float* t) {
    GpuScene* g = (GpuScene*)h;
    if (!g || W <= 0 || H <= 0 || !prim || !inst || !t) return fail("refgpu_first_hits: bad arguments");
    if (ensure_surfaces(*g, W, H)) return -1;
    set_view(*g, inv_proj, inv_view, env, settings);
    const size_t n = (size_t)W * H;
    int *dp = nullptr, *di = nullptr;
    float* dt = nullptr;
    RG_CUDA(cudaMalloc(&dp, n * 4));
    RG_CUDA(cudaMalloc(&di, n * 4));
    RG_CUDA(cudaMalloc(&dt, n * 4));
    dim3 block(8, 8, 1), grid(W / 8 + 1, H / 8 + 1, 1);   // launchPathTraceComputeMegaKernel's shape
    k_refgpu_first_hits<<<grid, block>>>(g->sd, dp, di, dt);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(prim, dp, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(inst, di, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(t, dt, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dp);
    cudaFree(di);
    cudaFree(dt);
    if (e != cudaSuccess) return fail(std::string("refgpu_first_hits: ") + cudaGetErrorString(e));
    return 0;
}

// One frame of Renderer::executeRendering (renderer.cu:103-195) with
// temporal accumulation on (integrator_use_temporal_accumulation), for the
// parts the path stage touches: Renderer::setView (:342-354) when the camera
// is given, Renderer::setMeshTransform (:250-269) for every mesh whose model
// matrix differs from its current one (models: column-major, one per mesh,
// may be null) and the TLAS rebuild of updateTLAS, the megakernel (which
// computes the velocity and reprojects, kernels.cu:165-338), the copy of the
// render into the accumulation texture, modulateSamples, the G-buffer copy
// into the previous G-buffer and the camera's per-frame update.  reset = 1
// starts a sequence: accumulation and previous G-buffer zeroed and the given
// camera as both previous and current.  render_out receives the modulated
// render and accum_out the accumulation texture ([H][W] RGBA each; alpha of
// the accumulation = the history length), either may be null.
int refgpu_temporal_frame(void* h, const float* inv_proj, const float* inv_view, const void* env, const void* settings,
                          int W, int H, int frame_index, const float* models, int reset, float* render_out,
                          float* accum_out) {
    GpuScene* g = (GpuScene*)h;
    if (!g || W <= 0 || H <= 0) return fail("refgpu_temporal_frame: bad arguments");
    if (ensure_surfaces(*g, W, H)) return -1;
    const EnvRecord& e = *(const EnvRecord*)env;
    const SettingsRecord& st = *(const SettingsRecord*)settings;
    ShaderData& sd = g->sd;
    sd.procedural_environment_data.sun_angular_diameter_rad = e.sun_angular_diameter;
    sd.procedural_environment_data.sun_phi_rad = e.sun_phi;
    sd.procedural_environment_data.sun_theta_rad = e.sun_theta;
    sd.procedural_environment_data.sun_emission_factor = e.sun_emission_factor;
    sd.renderer_settings = RendererSettings();
    sd.renderer_settings.integrator_max_ray_depth = st.max_depth;
    sd.renderer_settings.integrator_use_temporal_accumulation = true;
    if (reset) {
        if (clear_surface(g->surf[2], W, H) || clear_surface(g->surf[4], W, H)) return -1;
        Camera cam;
        cam.setView(mat_from(inv_proj), mat_from(inv_view));
        cam.setView(cam.curr_inv_projection_matrix, cam.curr_inv_view_matrix);
        sd.scene_camera = cam;
    } else if (inv_proj && inv_view) {
        sd.scene_camera.setView(mat_from(inv_proj), mat_from(inv_view));
    }
    if (models) {
        RefScene& r = g->host;
        bool moved = false;
        for (size_t mi = 0; mi < g->models.size(); ++mi) {
            if (std::memcmp(g->models[mi].data(), models + 16 * mi, 64) == 0) continue;
            std::memcpy(g->models[mi].data(), models + 16 * mi, 64);
            Mat4 model = mat_from(models + 16 * mi);
            TriangleMesh tm = r.meshes[mi];
            tm.setTransform(model.inverse());
            r.meshes[mi] = tm;
            BLAS2 b = r.blas[tm.blas_index];
            b.setTransform(model);
            r.blas[tm.blas_index] = b;
            moved = true;
        }
        if (moved) {   // updateTLAS (renderer_resource.cuh:24-26)
            TLASBuilder tb(&r.blas, &r.tlasnodes);   // rebuilt in place, as updateTLAS does
            r.sd.top_level_acceleration_structure = tb.build();
            if (tlas_interior_depth(r.tlasnodes, r.sd.top_level_acceleration_structure.tlasnode_root_index) + 2 >
                REF_STACK)
                return fail("refgpu_temporal_frame: TLAS deeper than the reference's stack allows");
            sd.top_level_acceleration_structure = r.sd.top_level_acceleration_structure;
            if (r.tlasnodes.size() > g->tlasnodes.n) return fail("refgpu_temporal_frame: TLAS grew");
            RG_CUDA(cudaMemcpy(g->tlasnodes.p, thrust::raw_pointer_cast(r.tlasnodes.data()),
                               sizeof(TLASNode) * r.tlasnodes.size(), cudaMemcpyDefault));
            RG_CUDA(cudaMemcpy(g->blas.p, thrust::raw_pointer_cast(r.blas.data()), sizeof(BLAS2) * r.blas.size(),
                               cudaMemcpyDefault));
            RG_CUDA(cudaMemcpy(g->meshes.p, thrust::raw_pointer_cast(r.meshes.data()),
                               sizeof(TriangleMesh) * r.meshes.size(), cudaMemcpyDefault));
            sd.tlas_nodes_buffer = Buffer<TLASNode>(g->tlasnodes.p, r.tlasnodes.size());
        }
    }
    sd.frame_index = frame_index;
    KittlesPT::launchPathTraceComputeMegaKernel(sd);
    const size_t pitch = (size_t)W * sizeof(float4);
    RG_CUDA(cudaMemcpy2DArrayToArray(g->surf[2].arr, 0, 0, g->surf[1].arr, 0, 0, pitch, H, cudaMemcpyDeviceToDevice));
    KittlesPT::launchModulateComputeKernel(sd);
    if (render_out)
        RG_CUDA(cudaMemcpy2DFromArray(render_out, pitch, g->surf[1].arr, 0, 0, pitch, H, cudaMemcpyDeviceToHost));
    if (accum_out)
        RG_CUDA(cudaMemcpy2DFromArray(accum_out, pitch, g->surf[2].arr, 0, 0, pitch, H, cudaMemcpyDeviceToHost));
    RG_CUDA(cudaMemcpy2DArrayToArray(g->surf[4].arr, 0, 0, g->surf[3].arr, 0, 0, pitch, H, cudaMemcpyDeviceToDevice));
    sd.scene_camera.setView(sd.scene_camera.curr_inv_projection_matrix, sd.scene_camera.curr_inv_view_matrix);
    return 0;
}

// The reference's lens effects (computeEffects through launchFxComputeKernel,
// kernels.cu:120-132 and :506-528) on an image: `in` ([H][W] RGBA) is the
// backbuffer, `out` receives the output texture.
int refgpu_effects(int W, int H, const float* in, float* out) {
    if (W <= 0 || H <= 0 || !in || !out) return fail("refgpu_effects: bad arguments");
    FrameSurface src, dst;
    cudaChannelFormatDesc cd = cudaCreateChannelDesc<float4>();
    cudaError_t e = cudaMallocArray(&src.arr, &cd, W, H, cudaArraySurfaceLoadStore);
    if (e == cudaSuccess) e = cudaMallocArray(&dst.arr, &cd, W, H, cudaArraySurfaceLoadStore);
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    if (e == cudaSuccess) {
        rd.res.array.array = src.arr;
        e = cudaCreateSurfaceObject(&src.obj, &rd);
    }
    if (e == cudaSuccess) {
        rd.res.array.array = dst.arr;
        e = cudaCreateSurfaceObject(&dst.obj, &rd);
    }
    const size_t pitch = (size_t)W * sizeof(float4);
    if (e == cudaSuccess) e = cudaMemcpy2DToArray(src.arr, 0, 0, in, pitch, pitch, H, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        ShaderData sd;
        sd.output_resolution = make_int2(W, H);
        sd.render_resolution = make_int2(W, H);
        sd.backbuffer_texture.dimensions = make_int2(W, H);
        sd.backbuffer_texture.m_surface_object = src.obj;
        sd.output_texture.dimensions = make_int2(W, H);
        sd.output_texture.m_surface_object = dst.obj;
        KittlesPT::launchFxComputeKernel(sd);
        e = cudaMemcpy2DFromArray(out, pitch, dst.arr, 0, 0, pitch, H, cudaMemcpyDeviceToHost);
    }
    for (FrameSurface* f : {&src, &dst}) {
        if (f->obj) cudaDestroySurfaceObject(f->obj);
        if (f->arr) cudaFreeArray(f->arr);
    }
    if (e != cudaSuccess) return fail(std::string("refgpu_effects: ") + cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
