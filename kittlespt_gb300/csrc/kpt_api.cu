// kpt_api.cu -- the C ABI (include/kpt.h): context, scene commit, frame graph.
//
// Host-side counterpart of KittlesPT::Renderer (renderer.cu) and
// RendererResource (renderer_resource.cuh): the context owns every device
// buffer; a frame is one CUDA graph (sky constants, camera rays, the path
// wave level by level, sky queue, accumulation, resolve, histogram, exposure,
// bloom chain, tonemap) re-captured and updated in place each frame, with no
// host synchronisation inside it.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "kpt.h"
#include "kpt_internal.h"
#include "kpt_post.h"
#include "kpt_scene.h"

using namespace kpt;

namespace {

thread_local std::string g_error;

kpt_status fail(kpt_status code, const std::string& msg) {
    g_error = msg;
    return code;
}

#define KPT_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? KPT_ERR_NOMEM : KPT_ERR_CUDA,             \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    cudaError_t upload(const T* src, size_t count, cudaStream_t s) {
        cudaError_t e = ensure(count);
        if (e != cudaSuccess || count == 0) return e;
        return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

std::atomic<unsigned long long> g_scene_versions{0};

void rows_of(const float* cm, float4* rows, int nrows) {   // column-major Mat4 -> rows
    for (int r = 0; r < nrows; ++r) rows[r] = make_float4(cm[r], cm[4 + r], cm[8 + r], cm[12 + r]);
}

}  // namespace

struct kpt_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    // second stream of the frame graph: the shadow rays of a level run on it
    // while the next level's extension rays run on `stream`
    cudaStream_t side = nullptr;
    // third stream: the sky of the paths that left the scene at level l runs
    // on it once k_shadow(l) has ended, beside the later levels
    cudaStream_t sky = nullptr;
    cudaEvent_t ev_sky = nullptr;
    std::vector<cudaEvent_t> ev_fork, ev_join;
    uint64_t launches = 0;

    // host scene
    std::vector<kpt_material> materials;
    std::vector<HostMesh> meshes;
    std::vector<HostInstance> instances;
    std::vector<TexRec> textures;
    std::vector<uint8_t> pixels;
    bool committed = false, tlas_dirty = true;
    int nlights = 0;

    // device scene
    DBuf<BvhNode> d_nodes, d_tlas;
    DBuf<float4> d_tris;
    DBuf<int> d_tri_leaf;   // per mesh, triangle id -> leaf-order slot (tri_base + id)
    DBuf<TriShade> d_shade;
    DBuf<MeshRec> d_meshes;
    DBuf<InstRec> d_inst;
    DBuf<LightRec> d_lights;
    DBuf<MatRec> d_materials;
    DBuf<TexRec> d_textures;
    DBuf<uint8_t> d_pixels;
    SceneView view{};
    std::vector<int> mesh_node_base, mesh_tri_base;   // per mesh: first node / triangle in the device arrays
    std::vector<LightRec> h_lights;
    std::vector<InstRec> h_inst;

    // camera and settings
    float inv_proj[16], inv_view[16];
    float prev_inv_proj[16], prev_inv_view[16];   // Camera::prev_* (camera.cuh:27-35)
    bool has_camera = false;
    kpt_environment env;
    kpt_settings settings;
    kpt_exposure exposure;

    // frame buffers: W x H is the render resolution, OW x OH the output's
    // (smaller by 2.5 with upscaling, resizeResolution renderer.cu:55-101)
    int W = 0, H = 0, OW = 0, OH = 0;
    DBuf<float4> output;        // the render upscaled to the output resolution (upscale)
    int frame_index = 0;
    int levels_depth = -1;      // max depth of the last wave whose level counts are kept (-1: none)
    DBuf<float4> acc, albedo, render, image;
    // temporal accumulation: visible surface, distances of the previous frame
    // and this one, history images (color, frames), per-instance matrices
    DBuf<float4> vis, thist[2];
    DBuf<float4> backbuf;       // the tonemapped image before the effects (postprocess_effects)
    DBuf<float4> easu;          // the EASU image before sharpening (upscale = 2)
    DBuf<float> tdepth[2];
    int tdepth_prev = 0;
    DBuf<TemporalInst> tinst;
    std::vector<TemporalInst> h_tinst;
    DBuf<TemporalGpuInst> tginst;   // the inverse model matrices for k_temporal_gpu
    std::vector<TemporalGpuInst> h_tginst;
    float4 tvp[2][4];           // current view-projection rows (the same for both)
    float3 torigin[2];          // previous camera position: first sample, later samples
    DBuf<int4> first_hit;
    std::vector<DBuf<float4>> mips;
    std::vector<int2> mip_dims;
    DBuf<unsigned long long> hist, counters;
    DBuf<float> thresholds;
    float thr_black = NAN, thr_white = NAN;
    DBuf<ExposureState> expo_state;
    DBuf<float3> sun_radiance;
    // the sun's constants in the reference GPU build's arithmetic (direction,
    // LeSun threshold, disc radius), computed on the device for sun_env
    DBuf<float> sun_gpu_dev;
    float sun_gpu[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool sun_gpu_valid = false;
    kpt_environment sun_env{};
    cudaGraphExec_t graph_exec = nullptr;
    // work buffers of the path stage
    DBuf<PrimaryRec> primary, hits;
    DBuf<int> hit_list, hit_index, miss_list, counts, level_counts;
    DBuf<int> fetch;   // queue counter of the ray-batch entry points
    // adjoint: d(sun radiance)/d(sky), host-call staging, record counter
    DBuf<float3> sun_J;
    DBuf<float> adj_in, adj_image;
    DBuf<double> adj_grad;
    DBuf<int> rec_count;
    DBuf<float4> adj_skyq;      // deferred double-precision sky Jacobians: (direction, weight)
    DBuf<int> adj_skyq_count;
    DBuf<float4> adj_skyqf;     // deferred single-precision sky Jacobians
    DBuf<int> adj_skyqf_count;
    DBuf<float4> adj_vr, adj_vend, adj_vsky;   // the wavefront replay's vertex and end records, escape skies
    DBuf<float4> adj_lpath;                    // the split adjoint's per-path radiance
    // the records kept by kpt_adjoint_forward_device for the backward call,
    // and the state they were replayed in
    struct AdjForward {
        bool valid = false;
        FrameParams F;
        AdjParams A;
        unsigned long long version = 0;
        std::vector<kpt_material> materials;
        kpt_environment env;
        kpt_settings settings;
        float inv_proj[16], inv_view[16];
        int W = 0, H = 0;
    } adj_fwd;
    DBuf<int> adj_esc;                          // the wavefront replay's escaped paths, then their count
    DBuf<unsigned char> adj_vis;     // the wavefront replay's light-sample visibility
    DBuf<float4> pixel_sky, radiance, sky_queue;
    DBuf<PathRec> paths[2], unsorted;
    DBuf<int> octants;
    DBuf<ShadowRec> shadow;
    int wave_cap = 0;
    bool device_blas = false;   // kpt_set_blas_build
    // the device scene's version (a value no other scene state of any
    // context has had: a batch's merged scene is rebuilt when one changes)
    unsigned long long scene_version = 0;
    int n_nodes = 0, n_tris = 0;   // BLAS nodes and triangles on the device
    kpt_tuning tuning{};   // launch parameters of the path stage (kpt_set_tuning)

    // stage timing inside the frame graph: per frame, event-record nodes
    // between the launches and the stage each interval belongs to
    static constexpr int EV_FRAMES = 32, EV_PER_FRAME = 96;
    struct TimedFrame {
        cudaEvent_t ev[EV_PER_FRAME] = {};
        unsigned char stage[EV_PER_FRAME] = {};
        int n = 0;
    };
    TimedFrame tframes[EV_FRAMES];
    bool timing = false;
    int frames_rendered = 0, last_slot = 0;
    TimedFrame* tf = nullptr;   // frame being captured with timing, else null
};

// Wave capacity: paths advanced together, level by level (208 B of work
// buffers each; 2^25 paths hold a 1080p frame of 16 samples in one wave).
static constexpr long long WAVE_CAP = 1LL << 25;
// device memory for one wave of the wavefront adjoint's vertex records
static constexpr size_t ADJ_WAVE_BYTES = (size_t)12 << 30;
// finished lanes of a warp that store results and fetch rays together
// (kpt_tuning.fetch_batch): 7 measured best on the 1080p16 frame with
// pixel-major waves and shading blocks of 256 (20.51 ms; 6: 20.55-20.60, 8:
// 20.53, 5: 20.65, 4: 20.83)
static constexpr int FETCH_BATCH = 7;
// threads per block of the shading kernel unless tuned (256: 22.48 ms on the
// 1080p16 frame against 22.51 with 128 and 64)
static constexpr int SHADE_BLOCK = SHADE_MAX_BLOCK;

extern "C" {

const char* kpt_last_error(void) { return g_error.c_str(); }

void kpt_environment_default(kpt_environment* e) {   // pod_types.hpp:37-44, atmosphere.cuh:292-310
    e->sun_angular_diameter = 0.0087f;
    e->sun_phi = 4.18879f;
    e->sun_theta = 17.0f * 3.14159265358979323846f / 180.0f;
    e->sun_emission_factor = 1.0f;
    e->rayleigh[0] = 3.8e-6f;
    e->rayleigh[1] = 13.5e-6f;
    e->rayleigh[2] = 33.1e-6f;
    e->mie = 21e-6f;
    e->mie_absorption = 21e-6f * 0.1f;
    e->rayleigh_height = 7994.0f;
    e->mie_height = 1200.0f;
    e->pad = 0.0f;
}

void kpt_settings_default(kpt_settings* s) {   // pod_types.hpp:46-57
    s->max_depth = 3;
    s->bloom = 0;
    s->karis = 0;
    s->auto_exposure = 0;
    s->bloom_final_blend = 0.175f;
    s->bloom_internal_blend = 0.65f;
    s->frame_delta_ms = 16.0f;
    s->rng_order = 0;
    s->temporal_accumulation = 0;
    s->postprocess_effects = 0;
    s->upscale = 0;
    s->sky_arith = 1;
    s->temporal_arith = 1;
}

void kpt_exposure_default(kpt_exposure* e) {   // SampleApp camera_controller.hpp:55-60
    e->aperture = 11.0f;
    e->iso = 100.0f;
    e->shutter = 0.004f;
    e->ev_comp = 0.0f;
    e->white_ev = 6.5f;
    e->black_ev = -10.0f;
    e->max_iso = 6400.0f;
    e->min_iso = 100.0f;
    e->max_shutter = 1.0f / 30.0f;
    e->min_shutter = 1.0f / 400.0f;
    e->pad0 = e->pad1 = 0.0f;
}

static kpt_status sun_constants_gpu(kpt_context* c);

kpt_status kpt_create(int device, kpt_context** out) {
    if (!out) return fail(KPT_ERR_INVALID, "kpt_create: null output");
    int n = 0;
    KPT_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(KPT_ERR_INVALID, "kpt_create: no such device");
    KPT_CUDA(cudaSetDevice(device));
    kpt_context* c = new kpt_context();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->sky, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_sky, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete c;
        return fail(KPT_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    kpt_environment_default(&c->env);
    kpt_settings_default(&c->settings);
    kpt_exposure_default(&c->exposure);
    kpt_tuning_default(&c->tuning);
    c->view.fetch_batch = c->tuning.fetch_batch;
    if (c->expo_state.ensure(1) != cudaSuccess || c->sun_radiance.ensure(1) != cudaSuccess ||
        c->counters.ensure(16) != cudaSuccess ||
        c->counts.ensure(4) != cudaSuccess || c->fetch.ensure(1) != cudaSuccess ||
        c->hist.ensure(256) != cudaSuccess || c->thresholds.ensure(256) != cudaSuccess) {
        kpt_destroy(c);
        return fail(KPT_ERR_NOMEM, "kpt_create: device allocation failed");
    }
    cudaMemsetAsync(c->expo_state.p, 0, sizeof(ExposureState), c->stream);
    cudaMemsetAsync(c->counters.p, 0, 16 * sizeof(unsigned long long), c->stream);
    if (sun_constants_gpu(c) != KPT_OK) {
        std::string why = kpt_last_error();
        kpt_destroy(c);
        return fail(KPT_ERR_CUDA, "kpt_create: " + why);
    }
    *out = c;
    return KPT_OK;
}

kpt_status kpt_destroy(kpt_context* c) {
    if (!c) return KPT_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    for (auto& f : c->tframes)
        for (cudaEvent_t e : f.ev)
            if (e) cudaEventDestroy(e);
    c->d_nodes.release(); c->d_tlas.release(); c->d_tris.release(); c->d_tri_leaf.release(); c->d_shade.release();
    c->d_meshes.release(); c->d_inst.release(); c->d_lights.release(); c->d_materials.release();
    c->d_textures.release(); c->d_pixels.release();
    c->acc.release(); c->albedo.release(); c->render.release(); c->image.release(); c->first_hit.release();
    c->vis.release(); c->tinst.release(); c->tginst.release(); c->backbuf.release(); c->output.release(); c->easu.release();
    for (int k = 0; k < 2; ++k) { c->thist[k].release(); c->tdepth[k].release(); }
    for (auto& m : c->mips) m.release();
    c->hist.release(); c->counters.release(); c->thresholds.release(); c->expo_state.release();
    c->sun_radiance.release();
    c->primary.release(); c->hits.release(); c->hit_list.release(); c->hit_index.release();
    c->miss_list.release(); c->counts.release(); c->level_counts.release(); c->pixel_sky.release();
    c->radiance.release(); c->sky_queue.release(); c->paths[0].release(); c->paths[1].release();
    c->unsorted.release(); c->octants.release();
    c->shadow.release(); c->fetch.release();
    c->sun_J.release(); c->adj_in.release(); c->adj_image.release(); c->adj_grad.release(); c->rec_count.release();
    c->adj_skyq.release(); c->adj_skyq_count.release(); c->adj_skyqf.release(); c->adj_skyqf_count.release();
    c->adj_vr.release(); c->adj_vend.release(); c->adj_vsky.release(); c->adj_lpath.release(); c->adj_vis.release(); c->adj_esc.release();
    for (auto* v : {&c->ev_fork, &c->ev_join})
        for (cudaEvent_t e : *v) cudaEventDestroy(e);
    if (c->ev_sky) cudaEventDestroy(c->ev_sky);
    if (c->sky) cudaStreamDestroy(c->sky);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return KPT_OK;
}

static kpt_status clear_accumulation(kpt_context* c) {
    c->frame_index = 0;
    if (c->acc.p) KPT_CUDA(cudaMemsetAsync(c->acc.p, 0, sizeof(float4) * (size_t)c->W * c->H, c->stream));
    // Renderer::resetAccumulation (renderer.cu:336-340) clears the history
    // image in temporal mode; the previous frame's depth stays
    if (c->thist[0].p) KPT_CUDA(cudaMemsetAsync(c->thist[0].p, 0, sizeof(float4) * c->thist[0].n, c->stream));
    return KPT_OK;
}

// Buffers of the temporal mode, allocated when it is first used (zeroed).
static kpt_status ensure_temporal(kpt_context* c) {
    const size_t np = (size_t)c->W * c->H;
    if (c->vis.n >= np && c->thist[0].n >= np) return KPT_OK;
    KPT_CUDA(c->vis.ensure(np));
    for (int k = 0; k < 2; ++k) {
        KPT_CUDA(c->thist[k].ensure(np));
        KPT_CUDA(c->tdepth[k].ensure(np));
        KPT_CUDA(cudaMemsetAsync(c->thist[k].p, 0, sizeof(float4) * np, c->stream));
        KPT_CUDA(cudaMemsetAsync(c->tdepth[k].p, 0, sizeof(float) * np, c->stream));
    }
    return KPT_OK;
}

// Renderer::resizeResolution (renderer.cu:55-101): output w x h, render
// resolution the output's / 2.5 with upscaling; an existing camera gets the
// projection of its field of view at the render aspect (near 0.1, far 100).
static kpt_status apply_resolution(kpt_context* c, int w, int h) {
    const bool up = c->settings.upscale != 0;
    const float scale_factor = 2.5f;
    const int rw = up ? std::max(1, (int)((float)w / scale_factor)) : w;
    const int rh = up ? std::max(1, (int)((float)h / scale_factor)) : h;
    if (w == c->OW && h == c->OH && rw == c->W && rh == c->H) return KPT_OK;
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    size_t np = (size_t)rw * rh, no = (size_t)w * h;
    KPT_CUDA(c->acc.ensure(np));
    KPT_CUDA(c->albedo.ensure(np));
    KPT_CUDA(c->render.ensure(np));
    KPT_CUDA(c->first_hit.ensure(np));
    KPT_CUDA(c->image.ensure(no));
    if (up) KPT_CUDA(c->output.ensure(no));
    // bloom mip chain at the output resolution (mipchain.cuh:17-36): levels below mip 0, at most 6
    int levels = std::min((int)std::log2((double)w), (int)std::log2((double)h));
    levels = std::min(levels, 6);
    for (auto& m : c->mips) m.release();
    c->mips.assign(levels + 1, DBuf<float4>());
    c->mip_dims.assign(levels + 1, make_int2(0, 0));
    for (int l = 0; l <= levels; ++l) {
        c->mip_dims[l] = make_int2(w >> l, h >> l);
        KPT_CUDA(c->mips[l].ensure((size_t)(w >> l) * (h >> l)));
    }
    c->W = rw;
    c->H = rh;
    c->OW = w;
    c->OH = h;
    if (c->has_camera) {
        // recompute projection for new screen size (renderer.cu:77-83)
        float proj[16];
        inverse4(c->inv_proj, proj);
        const float fov = 2.0f * atanf(1.0f / proj[5]);
        const float hh = cosf(0.5f * fov) / sinf(0.5f * fov);
        const float ww = hh * (float)rh / (float)rw;
        const float zn = 0.1f, zf = 100.0f;
        float p[16] = {0};
        p[0] = ww;
        p[5] = hh;
        p[10] = (zf + zn) / (zf - zn);
        p[11] = 1.0f;
        p[14] = -(2.0f * zf * zn) / (zf - zn);
        inverse4(p, c->inv_proj);
    }
    c->vis.release();   // the temporal buffers are re-created (zeroed) at the new size
    for (int k = 0; k < 2; ++k) {
        c->thist[k].release();
        c->tdepth[k].release();
    }
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    return clear_accumulation(c);
}

kpt_status kpt_resize(kpt_context* c, int w, int h) {
    if (!c || w <= 0 || h <= 0) return fail(KPT_ERR_INVALID, "kpt_resize: bad size");
    KPT_CUDA(cudaSetDevice(c->device));
    return apply_resolution(c, w, h);
}

kpt_status kpt_get_render_size(kpt_context* c, int* w, int* h) {
    if (!c || !w || !h) return fail(KPT_ERR_INVALID, "kpt_get_render_size: null argument");
    *w = c->W;
    *h = c->H;
    return KPT_OK;
}

kpt_status kpt_set_materials(kpt_context* c, int n, const kpt_material* m) {
    if (!c || n < 0 || (n > 0 && !m)) return fail(KPT_ERR_INVALID, "kpt_set_materials: bad arguments");
    c->materials.assign(m, m + n);
    c->committed = false;
    return KPT_OK;
}

kpt_status kpt_set_textures(kpt_context* c, int n, const int32_t* desc, size_t nbytes, const uint8_t* pixels) {
    if (!c || n < 0 || (n > 0 && !desc) || (nbytes > 0 && !pixels)) return fail(KPT_ERR_INVALID, "kpt_set_textures: bad arguments");
    c->textures.resize(n);
    for (int i = 0; i < n; ++i) {
        c->textures[i].w = desc[4 * i];
        c->textures[i].h = desc[4 * i + 1];
        c->textures[i].ch = desc[4 * i + 2];
        c->textures[i].offset = desc[4 * i + 3];
        c->textures[i].pad = 0;
        if (c->textures[i].w <= 0 || c->textures[i].h <= 0 || c->textures[i].ch < 3)
            return fail(KPT_ERR_INVALID, "kpt_set_textures: bad texture descriptor");
    }
    c->pixels.assign(pixels, pixels + nbytes);
    c->committed = false;
    return KPT_OK;
}

kpt_status kpt_upload_mesh(kpt_context* c, int ntris, const float* pos, const float* nrm, const float* uv,
                           const int32_t* mat, int* mesh_out) {
    if (!c || ntris <= 0 || !pos || !mat) return fail(KPT_ERR_INVALID, "kpt_upload_mesh: bad arguments");
    HostMesh m;
    m.pos.assign(pos, pos + 9 * (size_t)ntris);
    if (nrm) m.nrm.assign(nrm, nrm + 9 * (size_t)ntris);
    else m.nrm.assign(9 * (size_t)ntris, 0.0f);
    if (uv) m.uv.assign(uv, uv + 6 * (size_t)ntris);
    else m.uv.assign(6 * (size_t)ntris, 0.0f);
    m.material.assign(mat, mat + ntris);
    for (int i = 0; i < ntris; ++i)
        if (mat[i] < 0) return fail(KPT_ERR_INVALID, "kpt_upload_mesh: negative material id");
    if (c->device_blas) {
        const int e = build_blas_device(m, c->stream);
        if (e != 0) return fail(KPT_ERR_CUDA, std::string("kpt_upload_mesh: device BLAS build: ") +
                                                  cudaGetErrorString((cudaError_t)e));
    } else {
        build_blas(m);
    }
    c->meshes.push_back(std::move(m));
    if (mesh_out) *mesh_out = (int)c->meshes.size() - 1;
    c->committed = false;
    return KPT_OK;
}

kpt_status kpt_set_blas_build(kpt_context* c, int device) {
    if (!c || (device != 0 && device != 1)) return fail(KPT_ERR_INVALID, "kpt_set_blas_build: bad arguments");
    c->device_blas = device == 1;
    return KPT_OK;
}

kpt_status kpt_get_blas(kpt_context* c, int mesh, int32_t* info, float* nodes, int32_t* order, float* bounds) {
    if (!c || !info || mesh < 0 || mesh >= (int)c->meshes.size())
        return fail(KPT_ERR_INVALID, "kpt_get_blas: bad mesh or null info");
    const HostMesh& m = c->meshes[mesh];
    info[0] = (int32_t)m.nodes.size();
    info[1] = m.root;
    info[2] = m.leaf_first;
    info[3] = m.leaf_count;
    info[4] = m.ntris();
    if (nodes && !m.nodes.empty()) std::memcpy(nodes, m.nodes.data(), m.nodes.size() * sizeof(BvhNode));
    if (order) std::memcpy(order, m.order.data(), m.order.size() * sizeof(int32_t));
    if (bounds) {
        std::memcpy(bounds, m.lo, 3 * sizeof(float));
        std::memcpy(bounds + 3, m.hi, 3 * sizeof(float));
    }
    return KPT_OK;
}

kpt_status kpt_refit_mesh(kpt_context* c, int mesh, const float* positions, const float* normals) {
    if (!c || !positions || mesh < 0 || mesh >= (int)c->meshes.size())
        return fail(KPT_ERR_INVALID, "kpt_refit_mesh: bad mesh or null positions");
    if (!c->committed) return fail(KPT_ERR_STATE, "kpt_refit_mesh: no committed scene");
    HostMesh& m = c->meshes[mesh];
    const size_t n9 = 9 * (size_t)m.ntris();
    for (size_t i = 0; i < n9; ++i)
        if (!std::isfinite(positions[i])) return fail(KPT_ERR_INVALID, "kpt_refit_mesh: non-finite position");
    KPT_CUDA(cudaSetDevice(c->device));
    m.pos.assign(positions, positions + n9);
    if (normals) m.nrm.assign(normals, normals + n9);
    const int tb = c->mesh_tri_base[mesh];
    const int e = refit_blas_device(m, c->d_nodes.p, c->mesh_node_base[mesh], c->d_tris.p, tb, c->d_shade.p, c->stream);
    if (e != 0) return fail(KPT_ERR_CUDA, std::string("kpt_refit_mesh: ") + cudaGetErrorString((cudaError_t)e));
    c->scene_version = ++g_scene_versions;
    // the lights on the mesh's triangles
    bool lights = false;
    for (LightRec& L : c->h_lights) {
        if (c->instances[L.inst].mesh != mesh) continue;
        const float* p = &m.pos[9 * (size_t)L.tri];
        L.p0 = make_float3(p[0], p[1], p[2]);
        L.p1 = make_float3(p[3], p[4], p[5]);
        L.p2 = make_float3(p[6], p[7], p[8]);
        float gn[3], area;
        tri_normal_area(p, &m.nrm[9 * (size_t)L.tri], gn, &area);
        L.gn = make_float3(gn[0], gn[1], gn[2]);
        L.area = area;
        L.tri_area = area;
        lights = true;
    }
    if (lights)
        KPT_CUDA(cudaMemcpyAsync(c->d_lights.p, c->h_lights.data(), c->h_lights.size() * sizeof(LightRec),
                                 cudaMemcpyHostToDevice, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    c->tlas_dirty = true;   // the instances' world bounds follow the mesh's
    return c->settings.temporal_accumulation ? KPT_OK : clear_accumulation(c);
}

kpt_status kpt_add_instance(kpt_context* c, int mesh, const float* model, int material, int* out) {
    if (!c || !model || mesh < 0 || mesh >= (int)c->meshes.size())
        return fail(KPT_ERR_INVALID, "kpt_add_instance: bad mesh or matrix");
    HostInstance hi;
    hi.mesh = mesh;
    std::memcpy(hi.model, model, sizeof hi.model);
    std::memcpy(hi.prev_model, model, sizeof hi.prev_model);
    hi.material = material;
    c->instances.push_back(hi);
    if (out) *out = (int)c->instances.size() - 1;
    c->committed = false;
    return KPT_OK;
}

kpt_status kpt_clear_scene(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    c->meshes.clear();
    c->instances.clear();
    c->materials.clear();
    c->textures.clear();
    c->pixels.clear();
    c->committed = false;
    return KPT_OK;
}

static bool emissive(const kpt_material& m) {   // MaterialSceneEntity::isEmissive (pod_types.hpp:118-122)
    return m.emission[0] * m.emission_scale > 0.0f || m.emission[1] * m.emission_scale > 0.0f ||
           m.emission[2] * m.emission_scale > 0.0f;
}

static InstRec make_inst(const kpt_context* c, const HostInstance& hi) {
    InstRec r{};
    float inv[16], model[16];
    inverse4(hi.model, inv);      // BLAS2::setTransform (blas.cuh:338-348)
    inverse4(inv, model);         // the per-hit inverse of the mesh inverse (interaction.cu:20)
    rows_of(inv, r.inv, 3);
    rows_of(model, r.model, 3);
    r.mesh = hi.mesh;
    r.material = hi.material;
    r.light_first = -1;
    r.light_all = 0;
    (void)c;
    return r;
}

static kpt_status rebuild_tlas(kpt_context* c) {
    int n = (int)c->instances.size();
    std::vector<float> lo(3 * (size_t)n), hi(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
        instance_bounds(c->meshes[c->instances[i].mesh], c->instances[i].model, &lo[3 * i], &hi[3 * i]);
    float rlo[3], rhi[3];
    int root_leaf = 0, depth = 0;
    std::vector<BvhNode> t = build_tlas(lo, hi, n, rlo, rhi, &root_leaf, &depth);
    if (depth > TLAS_STACK - 1) return fail(KPT_ERR_STATE, "TLAS deeper than the traversal stack");
    KPT_CUDA(c->d_tlas.upload(t.data(), t.size(), c->stream));
    c->view.tlas = c->d_tlas.p;
    c->view.ntlas = (int)t.size();
    c->view.tlas_lo = make_float4(rlo[0], rlo[1], rlo[2], 0.0f);
    c->view.tlas_hi = make_float4(rhi[0], rhi[1], rhi[2], 0.0f);
    c->view.tlas_root_leaf = root_leaf;
    for (int i = 0; i < n; ++i) {
        InstRec r = make_inst(c, c->instances[i]);
        r.light_first = c->h_inst[i].light_first;
        r.light_all = c->h_inst[i].light_all;
        r.prim_base = c->h_inst[i].prim_base;
        c->h_inst[i] = r;
    }
    KPT_CUDA(c->d_inst.upload(c->h_inst.data(), c->h_inst.size(), c->stream));
    c->view.inst = c->d_inst.p;
    c->tlas_dirty = false;
    c->scene_version = ++g_scene_versions;
    return KPT_OK;
}

kpt_status kpt_commit_scene(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    KPT_CUDA(cudaSetDevice(c->device));
    if (c->instances.empty()) return fail(KPT_ERR_STATE, "kpt_commit_scene: no instances");
    int nm = (int)c->materials.size();
    for (auto& m : c->meshes)
        for (int id : m.material)
            if (id >= nm) return fail(KPT_ERR_INVALID, "kpt_commit_scene: material id out of range");
    for (auto& i : c->instances)
        if (i.material >= nm) return fail(KPT_ERR_INVALID, "kpt_commit_scene: material override out of range");
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    // BLAS nodes and triangles, mesh after mesh
    std::vector<BvhNode> nodes;
    std::vector<float4> tris;
    std::vector<TriShade> shade;
    std::vector<MeshRec> mrec;
    c->mesh_node_base.clear();
    c->mesh_tri_base.clear();
    for (auto& m : c->meshes) {
        MeshRec r{};
        int nb = (int)nodes.size(), tb = (int)(tris.size() / 3);
        c->mesh_node_base.push_back(nb);
        c->mesh_tri_base.push_back(tb);
        for (BvhNode n : m.nodes) {
            if (n.d.y == 0) n.d.x += nb; else n.d.x += tb;
            if (n.d.w == 0) n.d.z += nb; else n.d.z += tb;
            nodes.push_back(n);
        }
        r.node_root = m.root >= 0 ? nb + m.root : -1;
        r.leaf_first = tb + m.leaf_first;
        r.leaf_count = m.leaf_count;
        r.ntris = m.ntris();
        r.tri_base = tb;
        r.shade_base = (int)shade.size();
        if (m.max_depth > BLAS_STACK - 1) return fail(KPT_ERR_STATE, "BLAS deeper than the traversal stack");
        for (int k = 0; k < m.ntris(); ++k) {
            int t = m.order[k];
            const float* p = &m.pos[9 * (size_t)t];
            float lid;
            std::memcpy(&lid, &t, 4);
            tris.push_back(make_float4(p[0], p[1], p[2], lid));
            tris.push_back(make_float4(p[3] - p[0], p[4] - p[1], p[5] - p[2], 0.0f));
            tris.push_back(make_float4(p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.0f));
        }
        int rank = 0;
        for (int t = 0; t < m.ntris(); ++t) {
            TriShade s{};
            const float* u = &m.uv[6 * (size_t)t];
            s.uv0 = make_float2(u[0], u[1]);
            s.uv1 = make_float2(u[2], u[3]);
            s.uv2 = make_float2(u[4], u[5]);
            float gn[3], area;
            tri_normal_area(&m.pos[9 * (size_t)t], &m.nrm[9 * (size_t)t], gn, &area);
            s.gnx = gn[0]; s.gny = gn[1]; s.gnz = gn[2];
            s.material = m.material[t];
            s.emissive_rank = emissive(c->materials[m.material[t]]) ? rank++ : -1;
            shade.push_back(s);
        }
        r.n_emissive = rank;
        mrec.push_back(r);
    }
    // instances and lights (renderer.cu:393-401: one light per emissive triangle)
    std::vector<LightRec> lights;
    c->h_inst.assign(c->instances.size(), InstRec{});
    int prim_base = 0;
    for (size_t i = 0; i < c->instances.size(); ++i) {
        const HostInstance& hi = c->instances[i];
        const HostMesh& m = c->meshes[hi.mesh];
        InstRec r = make_inst(c, hi);
        r.prim_base = prim_base;
        prim_base += m.ntris();
        bool all = hi.material >= 0 && emissive(c->materials[hi.material]);
        bool own = hi.material < 0 && mrec[hi.mesh].n_emissive > 0;
        if (all || own) {
            r.light_first = (int)lights.size();
            r.light_all = all ? 1 : 0;
            for (int t = 0; t < m.ntris(); ++t) {
                int mat = hi.material >= 0 ? hi.material : m.material[t];
                if (!all && !emissive(c->materials[mat])) continue;
                LightRec L{};
                const float* p = &m.pos[9 * (size_t)t];
                L.p0 = make_float3(p[0], p[1], p[2]);
                L.p1 = make_float3(p[3], p[4], p[5]);
                L.p2 = make_float3(p[6], p[7], p[8]);
                float gn[3], area;
                tri_normal_area(p, &m.nrm[9 * (size_t)t], gn, &area);
                L.gn = make_float3(gn[0], gn[1], gn[2]);
                const float* u = &m.uv[6 * (size_t)t];
                L.uv0 = make_float2(u[0], u[1]);
                L.uv1 = make_float2(u[2], u[3]);
                L.uv2 = make_float2(u[4], u[5]);
                L.area = area;
                L.tri_area = area;
                L.inst = (int)i;
                L.tri = t;
                L.material = mat;
                lights.push_back(L);
            }
        }
        c->h_inst[i] = r;
    }
    std::vector<MatRec> mats(c->materials.size());
    static_assert(sizeof(MatRec) == sizeof(kpt_material), "material layout");
    std::memcpy(mats.data(), c->materials.data(), sizeof(kpt_material) * mats.size());
    KPT_CUDA(c->d_nodes.upload(nodes.data(), nodes.size(), c->stream));
    c->n_nodes = (int)nodes.size();
    c->n_tris = (int)(tris.size() / 3);
    KPT_CUDA(c->d_tris.upload(tris.data(), tris.size(), c->stream));
    {
        std::vector<int> tri_leaf(tris.size() / 3);
        for (size_t mi = 0; mi < c->meshes.size(); ++mi) {
            const HostMesh& m = c->meshes[mi];
            const int tb = c->mesh_tri_base[mi];
            for (int k = 0; k < m.ntris(); ++k) tri_leaf[(size_t)tb + m.order[k]] = tb + k;
        }
        KPT_CUDA(c->d_tri_leaf.upload(tri_leaf.data(), tri_leaf.size(), c->stream));
    }
    KPT_CUDA(c->d_shade.upload(shade.data(), shade.size(), c->stream));
    KPT_CUDA(c->d_meshes.upload(mrec.data(), mrec.size(), c->stream));
    KPT_CUDA(c->d_lights.upload(lights.data(), lights.size(), c->stream));
    c->h_lights = lights;
    KPT_CUDA(c->d_materials.upload(mats.data(), mats.size(), c->stream));
    KPT_CUDA(c->d_textures.upload(c->textures.data(), c->textures.size(), c->stream));
    KPT_CUDA(c->d_pixels.upload(c->pixels.data(), c->pixels.size(), c->stream));
    SceneView& v = c->view;
    v.nodes = c->d_nodes.p;
    v.tris = c->d_tris.p;
    v.shade = c->d_shade.p;
    v.meshes = c->d_meshes.p;
    v.lights = c->d_lights.p;
    v.materials = c->d_materials.p;
    v.textures = c->d_textures.p;
    v.pixels = c->d_pixels.p;
    v.npixels = (long long)c->pixels.size();
    v.nlights = (int)lights.size();
    v.ninst = (int)c->instances.size();
    v.ntextures = (int)c->textures.size();
    c->nlights = (int)lights.size();
    kpt_status s = rebuild_tlas(c);
    if (s != KPT_OK) return s;
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    c->committed = true;
    return clear_accumulation(c);
}

kpt_status kpt_counts(kpt_context* c, int* materials, int* meshes, int* instances, int* lights) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    if (materials) *materials = (int)c->materials.size();
    if (meshes) *meshes = (int)c->meshes.size();
    if (instances) *instances = (int)c->instances.size();
    if (lights) *lights = c->nlights;
    return KPT_OK;
}

kpt_status kpt_set_material(kpt_context* c, int idx, const kpt_material* m) {
    if (!c || !m) return fail(KPT_ERR_INVALID, "kpt_set_material: null argument");
    if (idx < 0 || idx >= (int)c->materials.size()) return fail(KPT_ERR_INVALID, "kpt_set_material: index out of range");
    c->materials[idx] = *m;
    if (c->committed) {
        KPT_CUDA(cudaMemcpyAsync(c->d_materials.p + idx, m, sizeof(MatRec), cudaMemcpyHostToDevice, c->stream));
        KPT_CUDA(cudaStreamSynchronize(c->stream));
    }
    return clear_accumulation(c);
}

kpt_status kpt_get_material(kpt_context* c, int idx, kpt_material* m) {
    if (!c || !m) return fail(KPT_ERR_INVALID, "kpt_get_material: null argument");
    if (idx < 0 || idx >= (int)c->materials.size()) return fail(KPT_ERR_INVALID, "kpt_get_material: index out of range");
    *m = c->materials[idx];
    return KPT_OK;
}

kpt_status kpt_set_instance_transform(kpt_context* c, int idx, const float* model) {
    if (!c || !model) return fail(KPT_ERR_INVALID, "kpt_set_instance_transform: null argument");
    if (idx < 0 || idx >= (int)c->instances.size()) return fail(KPT_ERR_INVALID, "kpt_set_instance_transform: index out of range");
    for (int i = 0; i < 16; ++i)
        if (!std::isfinite(model[i])) return fail(KPT_ERR_INVALID, "kpt_set_instance_transform: non-finite matrix");
    // TriangleMesh::setTransform (triangle.cuh:142-146): the old transform
    // becomes the previous one
    std::memcpy(c->instances[idx].prev_model, c->instances[idx].model, 16 * sizeof(float));
    std::memcpy(c->instances[idx].model, model, 16 * sizeof(float));
    c->tlas_dirty = true;
    // Renderer::setMeshTransform keeps the history in temporal mode (renderer.cu:264-266)
    return c->settings.temporal_accumulation ? KPT_OK : clear_accumulation(c);
}

kpt_status kpt_get_instance_transform(kpt_context* c, int idx, float* model) {
    if (!c || !model) return fail(KPT_ERR_INVALID, "kpt_get_instance_transform: null argument");
    if (idx < 0 || idx >= (int)c->instances.size()) return fail(KPT_ERR_INVALID, "kpt_get_instance_transform: index out of range");
    std::memcpy(model, c->instances[idx].model, 16 * sizeof(float));
    return KPT_OK;
}

kpt_status kpt_set_camera_inverse(kpt_context* c, const float* ip, const float* iv) {
    if (!c || !ip || !iv) return fail(KPT_ERR_INVALID, "kpt_set_camera_inverse: null argument");
    // Camera::setView (camera.cuh:27-35): the current camera becomes the
    // previous one (the first camera is its own previous camera)
    std::memcpy(c->prev_inv_proj, c->has_camera ? c->inv_proj : ip, sizeof c->prev_inv_proj);
    std::memcpy(c->prev_inv_view, c->has_camera ? c->inv_view : iv, sizeof c->prev_inv_view);
    std::memcpy(c->inv_proj, ip, sizeof c->inv_proj);
    std::memcpy(c->inv_view, iv, sizeof c->inv_view);
    c->has_camera = true;
    // Renderer::setView keeps the history in temporal mode (renderer.cu:351-353)
    return c->settings.temporal_accumulation ? KPT_OK : clear_accumulation(c);
}

kpt_status kpt_set_view(kpt_context* c, const float* proj, const float* view) {
    if (!c || !proj || !view) return fail(KPT_ERR_INVALID, "kpt_set_view: null argument");
    float ip[16], iv[16];
    inverse4(proj, ip);
    inverse4(view, iv);
    return kpt_set_camera_inverse(c, ip, iv);
}

kpt_status kpt_set_environment(kpt_context* c, const kpt_environment* e) {
    if (!c || !e) return fail(KPT_ERR_INVALID, "kpt_set_environment: null argument");
    if (!(e->rayleigh_height > 0.0f) || !(e->mie_height > 0.0f)) return fail(KPT_ERR_INVALID, "kpt_set_environment: scale heights must be positive");
    c->env = *e;
    if (c->settings.sky_arith) {
        kpt_status st = sun_constants_gpu(c);
        if (st != KPT_OK) return st;
    }
    return clear_accumulation(c);
}
kpt_status kpt_get_environment(kpt_context* c, kpt_environment* e) {
    if (!c || !e) return fail(KPT_ERR_INVALID, "null argument");
    *e = c->env;
    return KPT_OK;
}
kpt_status kpt_set_settings(kpt_context* c, const kpt_settings* s) {
    if (!c || !s) return fail(KPT_ERR_INVALID, "kpt_set_settings: null argument");
    if (s->max_depth < 0 || s->max_depth > 64) return fail(KPT_ERR_INVALID, "kpt_set_settings: max_depth out of range");
    if (s->temporal_accumulation != 0 && s->temporal_accumulation != 1)
        return fail(KPT_ERR_INVALID, "kpt_set_settings: temporal_accumulation must be 0 or 1");
    if (s->postprocess_effects != 0 && s->postprocess_effects != 1)
        return fail(KPT_ERR_INVALID, "kpt_set_settings: postprocess_effects must be 0 or 1");
    if (s->upscale < 0 || s->upscale > 2) return fail(KPT_ERR_INVALID, "kpt_set_settings: upscale must be 0, 1 or 2");
    if (s->rng_order < 0 || s->rng_order > 7) return fail(KPT_ERR_INVALID, "kpt_set_settings: rng_order must be in 0..7");
    if (s->sky_arith != 0 && s->sky_arith != 1) return fail(KPT_ERR_INVALID, "kpt_set_settings: sky_arith must be 0 or 1");
    if (s->temporal_arith != 0 && s->temporal_arith != 1)
        return fail(KPT_ERR_INVALID, "kpt_set_settings: temporal_arith must be 0 or 1");
    const bool resize = (s->upscale != 0) != (c->settings.upscale != 0) && c->OW > 0;
    c->settings = *s;
    if (resize) {   // the render resolution follows the switch at once
        kpt_status st = apply_resolution(c, c->OW, c->OH);
        if (st != KPT_OK) return st;
    }
    if (c->settings.sky_arith) {
        kpt_status st = sun_constants_gpu(c);
        if (st != KPT_OK) return st;
    }
    return clear_accumulation(c);
}
kpt_status kpt_get_settings(kpt_context* c, kpt_settings* s) {
    if (!c || !s) return fail(KPT_ERR_INVALID, "null argument");
    *s = c->settings;
    return KPT_OK;
}
kpt_status kpt_set_exposure(kpt_context* c, const kpt_exposure* e) {
    if (!c || !e) return fail(KPT_ERR_INVALID, "kpt_set_exposure: null argument");
    if (!(e->aperture > 0.0f) || !(e->iso > 0.0f) || !(e->shutter > 0.0f) || !(e->white_ev > e->black_ev))
        return fail(KPT_ERR_INVALID, "kpt_set_exposure: invalid camera values");
    c->exposure = *e;
    return KPT_OK;
}
kpt_status kpt_get_exposure(kpt_context* c, kpt_exposure* e) {
    if (!c || !e) return fail(KPT_ERR_INVALID, "null argument");
    *e = c->exposure;
    return KPT_OK;
}
kpt_status kpt_reset_accumulation(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    return clear_accumulation(c);
}

static SkyParams sky_params(const kpt_environment& e) {
    SkyParams P{};
    // getSunDirection (integrator.cuh:222-230), single precision as on the device
    float cp = cosf(e.sun_phi), sp = sinf(e.sun_phi), ct = cosf(e.sun_theta), st = sinf(e.sun_theta);
    float3 d = make_float3(cp * ct, st, sp * ct);
    float inv = 1.0f / sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    P.sun_dir = make_float3(d.x * inv, d.y * inv, d.z * inv);
    P.sun_emission = e.sun_emission_factor;
    P.sigma_r = make_float3(e.rayleigh[0], e.rayleigh[1], e.rayleigh[2]);
    P.sigma_m = e.mie;
    P.sigma_am = e.mie_absorption;
    P.h_r = e.rayleigh_height;
    P.h_m = e.mie_height;
    P.inv_h_r = (float)(1.0 / (double)e.rayleigh_height);
    P.inv_h_m = (float)(1.0 / (double)e.mie_height);
    P.earth_r = 6378137.0f;
    P.atm_r = 6438137.0f;
    P.cos_half_sun = cosf(e.sun_angular_diameter / 2.0f);   // LeSun (integrator.cuh:137)
    // angularDiameterToPhysicalDiameter / 2 (atmosphere.cuh:79-82)
    P.sun_radius_m = (2.0f * 149.597e9f * tanf(e.sun_angular_diameter / 2.0f)) / 2.0f;
    return P;
}

// The sun's constants in the arithmetic of the reference's GPU build,
// computed once per environment with the device's fast functions
// (k_sun_constants_gpu) and kept on the host.  Synchronises the stream.
static kpt_status sun_constants_gpu(kpt_context* c) {
    if (c->sun_gpu_valid && std::memcmp(&c->sun_env, &c->env, sizeof(kpt_environment)) == 0) return KPT_OK;
    KPT_CUDA(cudaSetDevice(c->device));
    KPT_CUDA(c->sun_gpu_dev.ensure(5));
    k_sun_constants_gpu<<<1, 32, 0, c->stream>>>(c->env.sun_phi, c->env.sun_theta, c->env.sun_angular_diameter,
                                                 c->sun_gpu_dev.p);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    KPT_CUDA(cudaMemcpyAsync(c->sun_gpu, c->sun_gpu_dev.p, sizeof(c->sun_gpu), cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    c->sun_env = c->env;
    c->sun_gpu_valid = true;
    return KPT_OK;
}

// The frame's sky parameters in the arithmetic the settings select.
static SkyParams frame_sky(kpt_context* c) {
    SkyParams P = sky_params(c->env);
    P.gpu_arith = c->settings.sky_arith;
    if (P.gpu_arith && c->sun_gpu_valid) {
        P.sun_dir = make_float3(c->sun_gpu[0], c->sun_gpu[1], c->sun_gpu[2]);
        P.cos_half_sun = c->sun_gpu[3];
        P.sun_radius_m = c->sun_gpu[4];
    }
    return P;
}

static FrameParams frame_params(kpt_context* c, int sample0, int nsamples) {
    FrameParams F{};
    F.scene = c->view;
    F.sky = frame_sky(c);
    rows_of(c->inv_proj, F.inv_proj, 4);
    rows_of(c->inv_view, F.inv_view, 3);
    F.cam_pos = make_float3(c->inv_view[12], c->inv_view[13], c->inv_view[14]);
    F.W = c->W;
    F.H = c->H;
    F.sample0 = sample0;
    F.nsamples = nsamples;
    F.max_depth = c->settings.max_depth;
    F.rng_order = c->settings.rng_order;
    F.sun_radiance = c->sun_radiance.p;
    F.counters = c->counters.p;
    F.paths[0] = c->paths[0].p;
    F.paths[1] = c->paths[1].p;
    F.hits = c->hits.p;
    F.shadow = c->shadow.p;
    F.level_counts = c->level_counts.p;
    F.unsorted = c->tuning.sort_rays ? c->unsorted.p : nullptr;
    F.group_lobes = c->tuning.group_lobes > 0 ? c->tuning.group_lobes : 0;
    F.octants = c->octants.p;
    F.cap = c->wave_cap;
    F.primary = c->primary.p;
    F.hit_list = c->hit_list.p;
    F.hit_index = c->hit_index.p;
    F.miss_list = c->miss_list.p;
    F.counts = c->counts.p;
    F.pixel_sky = c->pixel_sky.p;
    F.radiance = c->radiance.p;
    F.sky_queue = c->sky_queue.p;
    return F;
}

// Work buffers of the path stage for nsamples samples of every pixel
// (allocated outside any stream capture).
static kpt_status ensure_work(kpt_context* c, int nsamples) {
    size_t np = (size_t)c->W * c->H, ns = np * (size_t)nsamples;
    if (ns > (size_t)INT32_MAX) return fail(KPT_ERR_INVALID, "more than 2^31 - 1 samples in one call");
    const long long wcap = c->tuning.wave_cap > 0 ? (long long)c->tuning.wave_cap : WAVE_CAP;
    const int cap = (int)std::min<long long>((long long)ns, wcap);
    KPT_CUDA(c->paths[0].ensure(cap));
    KPT_CUDA(c->paths[1].ensure(cap));
    KPT_CUDA(c->hits.ensure(cap));
    KPT_CUDA(c->shadow.ensure(cap));
    KPT_CUDA(c->level_counts.ensure((size_t)LEVEL_WORDS * (c->settings.max_depth + 2)));
    KPT_CUDA(c->octants.ensure((size_t)16 * (c->settings.max_depth + 2)));
    if (c->tuning.sort_rays) KPT_CUDA(c->unsorted.ensure(cap));
    while (c->ev_fork.size() < (size_t)c->settings.max_depth + 1) {
        cudaEvent_t a = nullptr, b = nullptr;
        KPT_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        KPT_CUDA(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
        c->ev_fork.push_back(a);
        c->ev_join.push_back(b);
    }
    c->wave_cap = cap;
    KPT_CUDA(c->primary.ensure(np));
    KPT_CUDA(c->hit_list.ensure(np));
    KPT_CUDA(c->hit_index.ensure(np));
    KPT_CUDA(c->miss_list.ensure(np));
    KPT_CUDA(c->pixel_sky.ensure(np));
    KPT_CUDA(c->radiance.ensure(ns));
    KPT_CUDA(c->sky_queue.ensure(2 * ns));
    return KPT_OK;
}

// Resident blocks x SMs, scaled by the context's grid_scale (a job of a batch
// shares the SMs with the others).
static int persistent_grid(kpt_context* c, const void* kern, int block) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
    const int full = std::max(1, per_sm) * c->sm_count;
    return std::max(1, (int)std::lround((double)full * c->tuning.grid_scale));
}

// Closes the current timed interval of the frame being captured (if any) and
// opens the next one for `stage`.
static void stage_mark(kpt_context* c, int stage) {
    kpt_context::TimedFrame* f = c->tf;
    if (!f || f->n >= kpt_context::EV_PER_FRAME) return;
    cudaEventRecordWithFlags(f->ev[f->n], c->stream, cudaEventRecordExternal);
    f->stage[f->n] = (unsigned char)stage;
    f->n++;
}

// The path stage: camera rays and their sky, then the wave(s) of paths level
// by level, the queued sky and the ordered accumulation of every sample.
// camera rays and their sky
static void enqueue_camera(kpt_context* c, const FrameParams& F) {
    cudaStream_t s = c->stream;
    c->levels_depth = F.max_depth;
    cudaMemsetAsync(c->counts.p, 0, 4 * sizeof(int), s);
    stage_mark(c, KPT_STAGE_CAMERA);
    k_sky_constants<<<1, 32, 0, s>>>(F, c->sun_radiance.p);
    k_primary<<<primary_blocks(c->W, c->H), PATH_BLOCK, 0, s>>>(F);
    k_primary_sky<<<persistent_grid(c, (const void*)k_primary_sky, PATH_BLOCK), PATH_BLOCK, 0, s>>>(F);
    c->launches += 3;
}

// the start of a wave: its level counters cleared; with `mark`, the sky
// queue's length recorded as where its level 0 begins
static void enqueue_wave_start(kpt_context* c, const FrameParams& F, bool mark) {
    cudaStream_t s = c->stream;
    const int D = F.max_depth;
    cudaMemsetAsync(c->level_counts.p, 0, sizeof(int) * LEVEL_WORDS * (size_t)(D + 2), s);
    if (mark)
        cudaMemcpyAsync(c->level_counts.p + LEVEL_WORDS * (D + 1) + 5, c->counts.p + 2, sizeof(int),
                        cudaMemcpyDeviceToDevice, s);
    if (F.unsorted) cudaMemsetAsync(c->octants.p, 0, sizeof(int) * 16 * (size_t)(D + 2), s);
}

// the shading of level l of the wave starting at item w0
static void enqueue_shade(kpt_context* c, const FrameParams& F, int l, long long w0) {
    cudaStream_t s = c->stream;
    const int shade_block = c->tuning.shade_block > 0 ? c->tuning.shade_block : SHADE_BLOCK;
    const bool wide = shade_block > PATH_BLOCK;
    if (l > 0) {
        const int g = persistent_grid(c, wide ? (const void*)k_shade_bounce_wide : (const void*)k_shade_bounce,
                                      shade_block);
        if (wide) k_shade_bounce_wide<<<g, shade_block, 0, s>>>(F, l, w0);
        else k_shade_bounce<<<g, shade_block, 0, s>>>(F, l, w0);
    } else {
        const int g = persistent_grid(c, wide ? (const void*)k_shade_wide : (const void*)k_shade, shade_block);
        if (wide) k_shade_wide<<<g, shade_block, 0, s>>>(F, l, w0);
        else k_shade<<<g, shade_block, 0, s>>>(F, l, w0);
    }
}

// the ordered accumulation of every sample
static void enqueue_path_end(kpt_context* c, const FrameParams& F) {
    const int np = c->W * c->H;
    stage_mark(c, KPT_STAGE_ACCUMULATE);
    k_accumulate<<<(np + 255) / 256, 256, 0, c->stream>>>(F);
    c->launches += 1;
}

static void enqueue_paths(kpt_context* c, const FrameParams& F) {
    cudaStream_t s = c->stream;
    const int np = c->W * c->H;
    const int D = F.max_depth;
    enqueue_camera(c, F);
    const int g_ext = persistent_grid(c, (const void*)k_extend, TRACE_BLOCK);
    const int g_shd = persistent_grid(c, (const void*)k_shadow, TRACE_BLOCK);
    // every pixel may hit: the last waves find no work when fewer do
    const long long items = (long long)np * F.nsamples;
    // the shadow rays of level l and the extension rays of level l + 1 read
    // what k_shade(l) wrote and write disjoint buffers: they run on two
    // streams, joined before k_shade(l + 1); serial when stages are timed
    const bool fork = c->tf == nullptr && c->ev_fork.size() >= (size_t)D + 1;
    const int g_sky = persistent_grid(c, (const void*)k_sky_queue, PATH_BLOCK);
    for (long long w0 = 0; w0 < items; w0 += F.cap) {
        enqueue_wave_start(c, F, fork);
        for (int l = 0; l <= D; ++l) {
            if (l > 0) {
                stage_mark(c, KPT_STAGE_EXTEND);
                k_extend<<<g_ext, TRACE_BLOCK, 0, s>>>(F, l);
                if (fork) cudaStreamWaitEvent(s, c->ev_join[l - 1], 0);
            }
            stage_mark(c, KPT_STAGE_SHADE);
            enqueue_shade(c, F, l, w0);
            stage_mark(c, KPT_STAGE_SHADOW);
            if (fork) {
                cudaEventRecord(c->ev_fork[l], s);
                cudaStreamWaitEvent(c->side, c->ev_fork[l], 0);
                k_shadow<<<g_shd, TRACE_BLOCK, 0, c->side>>>(F, l);
                cudaEventRecord(c->ev_join[l], c->side);
                // k_shade(l)'s sky entries are final (their paths ended)
                cudaStreamWaitEvent(c->sky, c->ev_join[l], 0);
                k_sky_queue<<<g_sky, PATH_BLOCK, 0, c->sky>>>(F, l);
                c->launches += 1;
            } else {
                k_shadow<<<g_shd, TRACE_BLOCK, 0, s>>>(F, l);
            }
            c->launches += l > 0 ? 3 : 2;
            if (F.unsorted && l < D) {   // the continuations of level l, grouped by octant
                stage_mark(c, KPT_STAGE_SHADE);
                k_sort_count<<<c->sm_count * 4, 256, 0, s>>>(F, l + 1);
                k_sort_scatter<<<c->sm_count * 4, 256, 0, s>>>(F, l + 1);
                c->launches += 2;
            }
        }
        if (fork) {
            cudaStreamWaitEvent(s, c->ev_join[D], 0);
            cudaEventRecord(c->ev_sky, c->sky);
            cudaStreamWaitEvent(s, c->ev_sky, 0);
        }
        k_count_rays<<<1, 32, 0, s>>>(F);
        c->launches += 1;
    }
    if (!fork) {
        stage_mark(c, KPT_STAGE_SKY);
        k_sky_queue<<<g_sky, PATH_BLOCK, 0, s>>>(F, -1);
        c->launches += 1;
    }
    enqueue_path_end(c, F);
}

static kpt_status ready(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    if (!c->committed) return fail(KPT_ERR_STATE, "no committed scene");
    if (!c->has_camera) return fail(KPT_ERR_STATE, "no camera");
    if (c->W <= 0) return fail(KPT_ERR_STATE, "no resolution");
    KPT_CUDA(cudaSetDevice(c->device));
    if (c->tlas_dirty) return rebuild_tlas(c);
    return KPT_OK;
}

static void update_thresholds(kpt_context* c) {
    if (c->thr_black == c->exposure.black_ev && c->thr_white == c->exposure.white_ev) return;
    // luminanceToBin (histogram.cu:18-33) as thresholds: bin >= k+1 iff
    // Y >= 2^(black + range*k/254); evaluated in double, rounded up to float
    float thr[256];
    double range = (double)c->exposure.white_ev - (double)c->exposure.black_ev;
    thr[0] = 0.005f;
    for (int k = 1; k < 255; ++k) {
        double v = exp2((double)c->exposure.black_ev + range * (double)k / 254.0);
        float f = (float)v;
        if ((double)f < v) f = nextafterf(f, INFINITY);
        thr[k] = f;
    }
    thr[255] = INFINITY;
    cudaMemcpyAsync(c->thresholds.p, thr, sizeof thr, cudaMemcpyHostToDevice, c->stream);
    c->thr_black = c->exposure.black_ev;
    c->thr_white = c->exposure.white_ev;
}

// The frame: enqueued on the context stream (captured into a graph).
static void enqueue_temporal(kpt_context* c, const FrameParams& F);

// what follows the path stage: temporal blend or resolve, exposure, upscale,
// bloom, tonemap, lens effects
static void enqueue_post(kpt_context* c, const FrameParams& F, int total_samples, float delta_ms) {
    cudaStream_t s = c->stream;
    const int np = c->W * c->H;
    stage_mark(c, KPT_STAGE_POST);
    if (c->settings.temporal_accumulation) {
        enqueue_temporal(c, F);
        // modulateSamples of the blended image (kernels.cu:453-472)
        k_resolve<<<(np + 255) / 256, 256, 0, s>>>(np, c->thist[0].p, c->albedo.p, 1.0f, c->render.p);
    } else {
        k_resolve<<<(np + 255) / 256, 256, 0, s>>>(np, c->acc.p, c->albedo.p, (float)total_samples, c->render.p);
    }
    c->launches += 1;
    if (c->settings.auto_exposure) {
        ExposureIn in{};
        in.aperture = c->exposure.aperture;
        in.ev_comp = c->exposure.ev_comp;
        in.white_ev = c->exposure.white_ev;
        in.black_ev = c->exposure.black_ev;
        in.min_iso = c->exposure.min_iso;
        in.max_iso = c->exposure.max_iso;
        in.min_shutter = c->exposure.min_shutter;
        in.max_shutter = c->exposure.max_shutter;
        in.delta_ms = delta_ms;
        cudaMemsetAsync(c->hist.p, 0, 256 * sizeof(unsigned long long), s);
        k_histogram<<<(np + 255) / 256, 256, 0, s>>>(c->W, c->H, c->render.p, c->thresholds.p, c->hist.p);
        k_exposure<<<1, 32, 0, s>>>(c->hist.p, c->expo_state.p, in);
        c->launches += 2;
    }
    // launchUpscaleComputeKernel (kernels.cu:84-104): bilinear, or with FSR
    // (upscale = 2) EASU into a scratch image and RCAS from it into the output
    const bool up = c->settings.upscale != 0;
    const float4* out = up ? c->output.p : c->render.p;
    const dim3 ob(16, 16), og((c->OW + 15) / 16, (c->OH + 15) / 16);
    if (c->settings.upscale == 1) {
        k_upscale<<<og, ob, 0, s>>>(c->render.p, c->W, c->H, c->output.p, c->OW, c->OH);
        c->launches += 1;
    } else if (c->settings.upscale == 2) {
        k_easu<<<og, ob, 0, s>>>(c->render.p, c->W, c->H, c->easu.p, c->OW, c->OH,
                                 easu_constants(c->W, c->H, c->OW, c->OH));
        k_rcas<<<og, ob, 0, s>>>(c->easu.p, c->OW, c->OH, c->output.p);
        c->launches += 2;
    }
    const float4* bloom0 = nullptr;
    int levels = (int)c->mips.size() - 1;
    if (c->settings.bloom && levels > 0) {
        dim3 b(16, 16);
        for (int l = 0; l < levels; ++l) {
            int2 sd = c->mip_dims[l], dd = c->mip_dims[l + 1];
            const float4* src = l == 0 ? out : c->mips[l].p;
            k_bloom_down<<<dim3((dd.x + 15) / 16, (dd.y + 15) / 16), b, 0, s>>>(src, sd.x, sd.y, c->mips[l + 1].p, dd.x, dd.y,
                                                                               c->settings.karis && l == 0);
        }
        // mip 0 starts as a copy of the output (renderer.cu:446-451)
        cudaMemcpyAsync(c->mips[0].p, out, sizeof(float4) * (size_t)c->OW * c->OH, cudaMemcpyDeviceToDevice, s);
        for (int l = levels; l > 0; --l) {
            int2 sd = c->mip_dims[l], dd = c->mip_dims[l - 1];
            k_bloom_up<<<dim3((dd.x + 15) / 16, (dd.y + 15) / 16), b, 0, s>>>(c->mips[l].p, sd.x, sd.y, c->mips[l - 1].p,
                                                                             dd.x, dd.y, c->settings.bloom_internal_blend);
        }
        c->launches += 2 * levels;
        bloom0 = c->mips[0].p;
    }
    double N = c->exposure.aperture;
    double lavg = (10.0 / 0.65) * ((N * N) / ((double)c->exposure.iso * (double)c->exposure.shutter));
    float fixed_scalar = (float)(0.18 / lavg);
    const bool fx = c->settings.postprocess_effects != 0;
    k_tonemap<<<dim3((c->OW + 15) / 16, (c->OH + 15) / 16), dim3(16, 16), 0, s>>>(
        c->OW, c->OH, out, bloom0, bloom0 != nullptr, c->settings.bloom_final_blend, c->expo_state.p, fixed_scalar,
        c->settings.auto_exposure, c->exposure.white_ev, c->exposure.black_ev, fx ? c->backbuf.p : c->image.p);
    c->launches += 1;
    if (fx) {   // launchFxComputeKernel (renderer.cu:162-167)
        k_effects<<<dim3((c->OW + 15) / 16, (c->OH + 15) / 16), dim3(16, 16), 0, s>>>(c->OW, c->OH, c->backbuf.p,
                                                                                    c->image.p);
        c->launches += 1;
    }
    stage_mark(c, KPT_STAGE_COUNT);   // end of the last interval
}

static void enqueue_frame(kpt_context* c, const FrameParams& F, int total_samples, float delta_ms) {
    enqueue_paths(c, F);
    enqueue_post(c, F, total_samples, delta_ms);
}

// Host-side work of a frame, outside any capture: TLAS rebuild, exposure
// thresholds, work buffers, the frame's parameters.
// Mat4 * Mat4 (matrix_maths.cuh:269-283): entry (r, c) = row r of a dotted
// with column c of b, left to right; column-major in and out.
static void mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col)
            r[4 * col + row] = a[row] * b[4 * col] + a[4 + row] * b[4 * col + 1] + a[8 + row] * b[4 * col + 2] +
                               a[12 + row] * b[4 * col + 3];
    std::memcpy(out, r, sizeof r);
}

// The per-frame matrices of computeVelocity / testReprojection
// (kernels.cu:164-223): view-projections from the inverse camera matrices,
// per instance the current inverse model, the previous model and
// prev view-projection * prev model; `prev_cam` selects the camera whose
// view-projection multiplies the previous model (the previous camera for the
// first sample of a call, the current one after it).
static void temporal_matrices(kpt_context* c, bool prev_cam, float4* vp, float3* prev_origin) {
    float pj[16], vw[16], cur_vp[16], prv_vp[16];
    inverse4(c->inv_proj, pj);
    inverse4(c->inv_view, vw);
    mat4_mul(pj, vw, cur_vp);
    const float* pip = prev_cam ? c->prev_inv_proj : c->inv_proj;
    const float* piv = prev_cam ? c->prev_inv_view : c->inv_view;
    inverse4(pip, pj);
    inverse4(piv, vw);
    mat4_mul(pj, vw, prv_vp);
    rows_of(cur_vp, vp, 4);
    *prev_origin = make_float3(piv[12], piv[13], piv[14]);
    c->h_tinst.resize(c->instances.size());
    for (size_t i = 0; i < c->instances.size(); ++i) {
        const HostInstance& hi = c->instances[i];
        float inv[16], pinv[16], pmodel[16], pm[16];
        inverse4(hi.model, inv);            // curr_inv_model_matrix
        inverse4(hi.prev_model, pinv);      // prev_inv_model_matrix
        inverse4(pinv, pmodel);             // prev_inv_model_matrix.inverse()
        mat4_mul(prv_vp, pmodel, pm);
        TemporalInst& t = c->h_tinst[i];
        rows_of(inv, t.inv, 3);
        rows_of(pmodel, t.prev_model, 3);
        rows_of(pm, t.pm, 4);
    }
}

// The matrices k_temporal_gpu inverts itself: columns of a column-major Mat4.
static void columns_of(const float* cm, float4* cols) {
    for (int k = 0; k < 4; ++k) cols[k] = make_float4(cm[4 * k], cm[4 * k + 1], cm[4 * k + 2], cm[4 * k + 3]);
}

static kpt_status prepare_frame(kpt_context* c, int spp, FrameParams* F) {
    if (c) c->adj_fwd.valid = false;   // a frame reuses the wave buffers the kept records refer to
    kpt_status st = ready(c);
    if (st != KPT_OK) return st;
    if (spp <= 0) return fail(KPT_ERR_INVALID, "spp must be positive");
    update_thresholds(c);
    st = ensure_work(c, spp);
    if (st != KPT_OK) return st;
    *F = frame_params(c, c->frame_index, spp);
    F->acc = c->acc.p;
    F->albedo = c->albedo.p;
    F->first_hit = c->first_hit.p;
    if (c->settings.postprocess_effects) KPT_CUDA(c->backbuf.ensure((size_t)c->OW * c->OH));
    if (c->settings.upscale == 2) KPT_CUDA(c->easu.ensure((size_t)c->OW * c->OH));
    if (c->settings.temporal_accumulation) {
        st = ensure_temporal(c);
        if (st != KPT_OK) return st;
        F->acc = nullptr;
        F->vis = c->vis.p;
        // matrices of the first sample (previous camera) and of the others
        const size_t ni = c->instances.size();
        std::vector<TemporalInst> both(2 * ni);
        temporal_matrices(c, true, c->tvp[0], &c->torigin[0]);
        std::copy(c->h_tinst.begin(), c->h_tinst.end(), both.begin());
        temporal_matrices(c, false, c->tvp[1], &c->torigin[1]);
        std::copy(c->h_tinst.begin(), c->h_tinst.end(), both.begin() + ni);
        c->h_tinst.swap(both);
        KPT_CUDA(c->tinst.upload(c->h_tinst.data(), c->h_tinst.size(), c->stream));
        c->h_tginst.resize(ni);
        for (size_t i = 0; i < ni; ++i) {
            float inv[16], pinv[16];
            inverse4(c->instances[i].model, inv);         // curr_inv_model_matrix
            inverse4(c->instances[i].prev_model, pinv);   // prev_inv_model_matrix
            columns_of(inv, c->h_tginst[i].inv_model);
            columns_of(pinv, c->h_tginst[i].prev_inv_model);
            c->h_tginst[i].tri_base = c->mesh_tri_base[c->instances[i].mesh];
        }
        KPT_CUDA(c->tginst.upload(c->h_tginst.data(), ni, c->stream));
    }
    return KPT_OK;
}

static void finish_frame(kpt_context* c, int spp) {
    c->frame_index += spp;
    c->frames_rendered++;
    if (c->settings.temporal_accumulation) {
        // executeRendering ends with setView(curr, curr) (renderer.cu:187-191)
        std::memcpy(c->prev_inv_proj, c->inv_proj, sizeof c->prev_inv_proj);
        std::memcpy(c->prev_inv_view, c->inv_view, sizeof c->prev_inv_view);
        c->tdepth_prev ^= 1;
    }
}

static void k_temporal_launch(kpt_context* c, const TemporalParams& T, int np, cudaStream_t s) {
    if (c->settings.temporal_arith) k_temporal_gpu<<<(np + 255) / 256, 256, 0, s>>>(T);
    else k_temporal<<<(np + 255) / 256, 256, 0, s>>>(T);
    c->launches += 1;
}

// Temporal accumulation of the call's samples, one reference frame each
// (kernels.cu:422-428): the history ping-pongs between thist[0] and
// thist[1] and ends in thist[0].
static void enqueue_temporal(kpt_context* c, const FrameParams& F) {
    cudaStream_t s = c->stream;
    const int np = c->W * c->H;
    const int ni = (int)c->instances.size();
    TemporalParams T{};
    T.W = c->W;
    T.H = c->H;
    T.counts = F.counts;
    T.hit_index = F.hit_index;
    T.primary = F.primary;
    T.radiance = F.radiance;
    T.pixel_sky = F.pixel_sky;
    T.vis = F.vis;
    for (int k = 0; k < F.nsamples; ++k) {
        const int cam = k == 0 ? 0 : 1;
        T.sample = k;
        T.nsamples = F.nsamples;
        T.inst = c->tinst.p + (size_t)cam * ni;
        for (int r = 0; r < 4; ++r) T.vp[r] = c->tvp[cam][r];
        T.prev_origin = c->torigin[cam];
        T.prev_depth = k == 0 ? c->tdepth[c->tdepth_prev].p : c->tdepth[c->tdepth_prev ^ 1].p;
        T.depth_out = k == 0 ? c->tdepth[c->tdepth_prev ^ 1].p : nullptr;
        T.hist_in = c->thist[k & 1].p;
        T.hist_out = c->thist[(k & 1) ^ 1].p;
        // the reference's frame k of the call: the previous camera for the
        // first, the current one after it (executeRendering ends with setView)
        T.ginst = c->tginst.p;
        T.tris = c->d_tris.p;
        T.tri_leaf = c->d_tri_leaf.p;
        columns_of(c->inv_proj, T.inv_proj);
        columns_of(c->inv_view, T.inv_view);
        columns_of(k == 0 ? c->prev_inv_proj : c->inv_proj, T.prev_inv_proj);
        columns_of(k == 0 ? c->prev_inv_view : c->inv_view, T.prev_inv_view);
        k_temporal_launch(c, T, np, s);
    }
    if (F.nsamples & 1)
        cudaMemcpyAsync(c->thist[0].p, c->thist[1].p, sizeof(float4) * (size_t)np, cudaMemcpyDeviceToDevice, s);
}

// Instantiates `g` into *exec, updating the previous executable in place when
// the topology is unchanged.  Consumes g.
static kpt_status instantiate(cudaGraph_t g, cudaGraphExec_t* exec) {
    if (*exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(*exec, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(*exec);
            *exec = nullptr;
        }
    }
    if (!*exec) {
        cudaError_t e = cudaGraphInstantiate(exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return fail(KPT_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
    }
    cudaGraphDestroy(g);
    return KPT_OK;
}

kpt_status kpt_render_frame(kpt_context* c, int spp, float delta_ms) {
    FrameParams F;
    kpt_status st = prepare_frame(c, spp, &F);
    if (st != KPT_OK) return st;
    int total = c->frame_index + spp;
    cudaGraph_t g = nullptr;
    if (c->timing) {
        c->last_slot = c->frames_rendered % kpt_context::EV_FRAMES;
        c->tf = &c->tframes[c->last_slot];
        c->tf->n = 0;
    }
    cudaError_t ce = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        enqueue_frame(c, F, total, delta_ms);
        ce = cudaStreamEndCapture(c->stream, &g);
    }
    c->tf = nullptr;
    KPT_CUDA(ce);
    st = instantiate(g, &c->graph_exec);
    if (st != KPT_OK) return st;
    cudaError_t e = cudaGraphLaunch(c->graph_exec, c->stream);
    if (e != cudaSuccess) return fail(KPT_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    finish_frame(c, spp);
    return KPT_OK;
}

kpt_status kpt_synchronize(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    return KPT_OK;
}

static kpt_status read_buf(kpt_context* c, const void* src, void* dst, size_t bytes) {
    if (!c || !dst) return fail(KPT_ERR_INVALID, "null argument");
    if (!src) return fail(KPT_ERR_STATE, "buffer not allocated");
    KPT_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    return KPT_OK;
}
kpt_status kpt_read_image(kpt_context* c, float* rgba) { return read_buf(c, c ? c->image.p : nullptr, rgba, c ? 16 * (size_t)c->OW * c->OH : 0); }
kpt_status kpt_read_render(kpt_context* c, float* rgba) { return read_buf(c, c ? c->render.p : nullptr, rgba, c ? 16 * (size_t)c->W * c->H : 0); }
kpt_status kpt_read_accumulation(kpt_context* c, float* rgba) { return read_buf(c, c ? c->acc.p : nullptr, rgba, c ? 16 * (size_t)c->W * c->H : 0); }
kpt_status kpt_read_albedo(kpt_context* c, float* rgba) { return read_buf(c, c ? c->albedo.p : nullptr, rgba, c ? 16 * (size_t)c->W * c->H : 0); }
kpt_status kpt_read_history(kpt_context* c, float* rgba) {
    if (c && !c->thist[0].p) return fail(KPT_ERR_STATE, "kpt_read_history: no temporal history");
    return read_buf(c, c ? c->thist[0].p : nullptr, rgba, c ? 16 * (size_t)c->W * c->H : 0);
}
kpt_status kpt_read_histogram(kpt_context* c, uint64_t* bins) { return read_buf(c, c ? c->hist.p : nullptr, bins, 256 * sizeof(uint64_t)); }

kpt_status kpt_get_level_counts(kpt_context* c, int max_levels, int32_t* counts, int32_t* levels) {
    if (!c || !counts || !levels || max_levels < 1) return fail(KPT_ERR_INVALID, "kpt_get_level_counts: invalid argument");
    const int D = c->levels_depth;
    if (D < 0 || !c->level_counts.p) return fail(KPT_ERR_STATE, "kpt_get_level_counts: no frame rendered");
    std::vector<int> h((size_t)LEVEL_WORDS * (D + 2));
    KPT_CUDA(cudaMemcpyAsync(h.data(), c->level_counts.p, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    const int n = std::min(max_levels, D + 1);
    for (int l = 0; l < n; ++l)
        for (int k = 0; k < 3; ++k) counts[3 * l + k] = h[(size_t)LEVEL_WORDS * l + k];
    *levels = n;
    return KPT_OK;
}

kpt_status kpt_get_stats(kpt_context* c, kpt_stats* st) {
    if (!c || !st) return fail(KPT_ERR_INVALID, "null argument");
    unsigned long long cnt[16];
    ExposureState es;
    KPT_CUDA(cudaMemcpyAsync(cnt, c->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaMemcpyAsync(&es, c->expo_state.p, sizeof es, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    st->box_tests = cnt[0] + cnt[4] + cnt[8];
    st->tri_tests = cnt[1] + cnt[5] + cnt[9];
    st->inst_xforms = cnt[2] + cnt[6] + cnt[10];
    st->overflows = cnt[3] + cnt[7] + cnt[11];
    st->path_box_tests = cnt[0];
    st->path_tri_tests = cnt[1];
    st->path_inst_xforms = cnt[2];
    st->shadow_box_tests = cnt[8];
    st->shadow_tri_tests = cnt[9];
    st->shadow_inst_xforms = cnt[10];
    st->path_rays = cnt[12];
    st->shadow_rays = cnt[13];
    st->camera_rays = cnt[14];
    st->avg_luminance = es.avg_lum;
    st->adapted_luminance = es.adapted_lum;
    st->exposure_scalar = es.exposure_scalar;
    st->iso = es.iso;
    st->shutter = es.shutter;
    st->avg_bin = es.avg_bin;
    st->frame_index = c->frame_index;
    st->pad = 0;
    return KPT_OK;
}

kpt_status kpt_render_samples_device(kpt_context* c, int sample0, int nsamples, float* radiance, int32_t* first_hit,
                                     float* albedo) {
    kpt_status st = ready(c);
    if (st != KPT_OK) return st;
    if (nsamples <= 0 || sample0 < 0) return fail(KPT_ERR_INVALID, "kpt_render_samples_device: bad sample range");
    st = ensure_work(c, nsamples);
    if (st != KPT_OK) return st;
    FrameParams F = frame_params(c, sample0, nsamples);
    F.sample_out = reinterpret_cast<float4*>(radiance);
    F.first_hit = reinterpret_cast<int4*>(first_hit);
    F.albedo = reinterpret_cast<float4*>(albedo);
    enqueue_paths(c, F);
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

static int trace_grid(kpt_context* c, const void* kern, int n) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TRACE_BLOCK, 0);
    int g = std::max(1, per_sm) * c->sm_count;
    return std::min(g, (n + TRACE_BLOCK - 1) / TRACE_BLOCK);
}

static kpt_status scene_ready(kpt_context* c) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    if (!c->committed) return fail(KPT_ERR_STATE, "no committed scene");
    KPT_CUDA(cudaSetDevice(c->device));
    if (c->tlas_dirty) return rebuild_tlas(c);
    return KPT_OK;
}

kpt_status kpt_trace_device(kpt_context* c, int n, const float* o, const float* d, float tmin, float tmax, int32_t* inst,
                            int32_t* tri, float* t, float* uv) {
    kpt_status st = scene_ready(c);
    if (st != KPT_OK) return st;
    if (n < 0 || (n > 0 && (!o || !d || !inst || !tri || !t))) return fail(KPT_ERR_INVALID, "kpt_trace_device: bad arguments");
    if (n == 0) return KPT_OK;
    KPT_CUDA(cudaMemsetAsync(c->fetch.p, 0, sizeof(int), c->stream));
    k_trace<<<trace_grid(c, (const void*)k_trace, n), TRACE_BLOCK, 0, c->stream>>>(
        c->view, n, (const float3*)o, (const float3*)d, tmin, tmax, inst, tri, t, (float2*)uv, c->fetch.p,
        c->counters.p);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_occluded_device(kpt_context* c, int n, const float* o, const float* d, float tmin, const float* tmax,
                               uint8_t* out) {
    kpt_status st = scene_ready(c);
    if (st != KPT_OK) return st;
    if (n < 0 || (n > 0 && (!o || !d || !tmax || !out))) return fail(KPT_ERR_INVALID, "kpt_occluded_device: bad arguments");
    if (n == 0) return KPT_OK;
    KPT_CUDA(cudaMemsetAsync(c->fetch.p, 0, sizeof(int), c->stream));
    k_occluded<<<trace_grid(c, (const void*)k_occluded, n), TRACE_BLOCK, 0, c->stream>>>(
        c->view, n, (const float3*)o, (const float3*)d, tmin, tmax, out, c->fetch.p, c->counters.p);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_trace_bounces_device(kpt_context* c, int n, const float* o, const float* d, int nb, int32_t* inst,
                                    int32_t* tri, float* t) {
    kpt_status st = scene_ready(c);
    if (st != KPT_OK) return st;
    if (n < 0 || nb < 0 || (n > 0 && (!o || !d || !inst || !tri || !t)))
        return fail(KPT_ERR_INVALID, "kpt_trace_bounces_device: bad arguments");
    if (n == 0) return KPT_OK;
    KPT_CUDA(cudaMemsetAsync(c->fetch.p, 0, sizeof(int), c->stream));
    // a lane of a chain traces its next bounce without a fetch: batching the
    // fetches measured slower here (675 vs 650 Mrays/s on 2M random triangles)
    SceneView v = c->view;
    v.fetch_batch = 1;
    k_trace_chains<<<trace_grid(c, (const void*)k_trace_chains, n), TRACE_BLOCK, 0, c->stream>>>(
        v, n, (const float3*)o, (const float3*)d, nb, inst, tri, t, c->fetch.p, c->counters.p);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_trace_bounces(kpt_context* c, int n, const float* o, const float* d, int nb, int32_t* inst, int32_t* tri,
                             float* t) {
    kpt_status st = scene_ready(c);
    if (st != KPT_OK) return st;
    if (n < 0 || nb < 0 || (n > 0 && (!o || !d || !inst || !tri || !t)))
        return fail(KPT_ERR_INVALID, "kpt_trace_bounces: bad arguments");
    if (n == 0) return KPT_OK;
    size_t nr = (size_t)n, no = nr * (nb + 1);
    DBuf<float> dev_in;
    DBuf<int32_t> dev_out;
    DBuf<float> dev_t;
    KPT_CUDA(dev_in.ensure(6 * nr));
    KPT_CUDA(dev_out.ensure(2 * no));
    KPT_CUDA(dev_t.ensure(no));
    KPT_CUDA(cudaMemcpyAsync(dev_in.p, o, 12 * nr, cudaMemcpyHostToDevice, c->stream));
    KPT_CUDA(cudaMemcpyAsync(dev_in.p + 3 * nr, d, 12 * nr, cudaMemcpyHostToDevice, c->stream));
    st = kpt_trace_bounces_device(c, n, dev_in.p, dev_in.p + 3 * nr, nb, dev_out.p, dev_out.p + no, dev_t.p);
    if (st == KPT_OK) {
        KPT_CUDA(cudaMemcpyAsync(inst, dev_out.p, 4 * no, cudaMemcpyDeviceToHost, c->stream));
        KPT_CUDA(cudaMemcpyAsync(tri, dev_out.p + no, 4 * no, cudaMemcpyDeviceToHost, c->stream));
        KPT_CUDA(cudaMemcpyAsync(t, dev_t.p, 4 * no, cudaMemcpyDeviceToHost, c->stream));
        KPT_CUDA(cudaStreamSynchronize(c->stream));
    }
    cudaStreamSynchronize(c->stream);
    dev_in.release();
    dev_out.release();
    dev_t.release();
    return st;
}

kpt_status kpt_sky_device(kpt_context* c, int n, const float* dirs, float* rgb) {
    if (!c || n < 0 || (n > 0 && (!dirs || !rgb))) return fail(KPT_ERR_INVALID, "kpt_sky_device: bad arguments");
    KPT_CUDA(cudaSetDevice(c->device));
    if (n == 0) return KPT_OK;
    k_sky<<<(n + 127) / 128, 128, 0, c->stream>>>(frame_sky(c), n, (const float3*)dirs, (float3*)rgb);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_enable_timing(kpt_context* c, int enable) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    KPT_CUDA(cudaSetDevice(c->device));
    if (enable && !c->tframes[0].ev[0]) {
        for (auto& f : c->tframes)
            for (cudaEvent_t& e : f.ev) KPT_CUDA(cudaEventCreate(&e));
    }
    c->timing = enable != 0;
    for (auto& f : c->tframes) f.n = 0;
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    return KPT_OK;
}

kpt_status kpt_stage_ms(kpt_context* c, int nframes, float* ms) {
    if (!c || !ms || nframes <= 0 || nframes > kpt_context::EV_FRAMES || nframes > c->frames_rendered)
        return fail(KPT_ERR_INVALID, "kpt_stage_ms: bad arguments");
    if (!c->timing) return fail(KPT_ERR_STATE, "kpt_stage_ms: timing not enabled");
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    double sum[KPT_STAGE_COUNT] = {};
    for (int k = 0; k < nframes; ++k) {
        int slot = ((c->last_slot - k) % kpt_context::EV_FRAMES + kpt_context::EV_FRAMES) % kpt_context::EV_FRAMES;
        const kpt_context::TimedFrame& f = c->tframes[slot];
        if (f.n == 0) return fail(KPT_ERR_STATE, "kpt_stage_ms: a frame was rendered without timing");
        for (int i = 0; i + 1 < f.n; ++i) {
            float t = 0.0f;
            KPT_CUDA(cudaEventElapsedTime(&t, f.ev[i], f.ev[i + 1]));
            if (f.stage[i] < KPT_STAGE_COUNT) sum[f.stage[i]] += t;
        }
    }
    for (int i = 0; i < KPT_STAGE_COUNT; ++i) ms[i] = (float)sum[i];
    return KPT_OK;
}

kpt_status kpt_path_kernel_ms(kpt_context* c, int nframes, float* total_ms) {
    if (!total_ms) return fail(KPT_ERR_INVALID, "kpt_path_kernel_ms: bad arguments");
    float ms[KPT_STAGE_COUNT];
    kpt_status st = kpt_stage_ms(c, nframes, ms);
    if (st != KPT_OK) return st;
    *total_ms = ms[KPT_STAGE_SHADE] + ms[KPT_STAGE_SHADOW] + ms[KPT_STAGE_EXTEND];
    return KPT_OK;
}

kpt_status kpt_get_stream(kpt_context* c, void** s) {
    if (!c || !s) return fail(KPT_ERR_INVALID, "null argument");
    *s = (void*)c->stream;
    return KPT_OK;
}

kpt_status kpt_launch_count(kpt_context* c, uint64_t* n) {
    if (!c || !n) return fail(KPT_ERR_INVALID, "null argument");
    *n = c->launches;
    return KPT_OK;
}

// ---------------------------------------------------------------------------
// launch parameters and batched requests

void kpt_tuning_default(kpt_tuning* t) {
    t->grid_scale = 1.0f;
    t->wave_cap = 0;
    t->shade_block = SHADE_BLOCK;
    t->sort_rays = 0;
    t->fetch_batch = FETCH_BATCH;
    t->group_lobes = SHADE_WINDOW;
}

kpt_status kpt_set_tuning(kpt_context* c, const kpt_tuning* t) {
    if (!c || !t) return fail(KPT_ERR_INVALID, "kpt_set_tuning: null argument");
    if (!(t->grid_scale > 0.0f && t->grid_scale <= 1.0f))
        return fail(KPT_ERR_INVALID, "kpt_set_tuning: grid_scale must be in (0, 1]");
    if (t->wave_cap != 0 && (t->wave_cap < 1024 || t->wave_cap > WAVE_CAP))
        return fail(KPT_ERR_INVALID, "kpt_set_tuning: wave_cap must be 0 or in [1024, 2^25]");
    if (t->shade_block != 0 && t->shade_block != 64 && t->shade_block != 128 && t->shade_block != 256)
        return fail(KPT_ERR_INVALID, "kpt_set_tuning: shade_block must be 0, 64, 128 or 256");
    if (t->sort_rays != 0 && t->sort_rays != 1) return fail(KPT_ERR_INVALID, "kpt_set_tuning: sort_rays must be 0 or 1");
    if (t->fetch_batch < 0 || t->fetch_batch > 32)
        return fail(KPT_ERR_INVALID, "kpt_set_tuning: fetch_batch must be in [0, 32]");
    if (!(t->group_lobes == -1 || t->group_lobes == 0 ||
          (t->group_lobes >= 64 && t->group_lobes <= SHADE_WINDOW && t->group_lobes % 64 == 0)))
        return fail(KPT_ERR_INVALID, "kpt_set_tuning: group_lobes must be -1, 0 or a multiple of 64 in [64, 2048]");
    c->tuning = *t;
    if (c->tuning.shade_block == 0) c->tuning.shade_block = SHADE_BLOCK;
    if (c->tuning.fetch_batch == 0) c->tuning.fetch_batch = FETCH_BATCH;
    if (c->tuning.group_lobes == 0) c->tuning.group_lobes = SHADE_WINDOW;
    c->view.fetch_batch = c->tuning.fetch_batch;
    return KPT_OK;
}

// ---------------------------------------------------------------------------
// path-replay adjoint

static int adjoint_params(const kpt_context* c) { return 4 * (int)c->materials.size() + ADJ_SKY_PARAMS; }

static kpt_status adjoint_run(kpt_context* c, int sample0, int nsamples, const float* adjoint, double* grad,
                              float* image, AdjRec* rec, int max_rec) {
    c->adj_fwd.valid = false;
    kpt_status st = ready(c);
    if (st != KPT_OK) return st;
    if (nsamples <= 0 || sample0 < 0 || !adjoint || !grad)
        return fail(KPT_ERR_INVALID, "kpt_adjoint: bad arguments");
    if (c->settings.max_depth + 1 > ADJ_MAX_VERTICES)
        return fail(KPT_ERR_INVALID, "kpt_adjoint: max_depth above 16");
    const int ng = adjoint_params(c);
    const size_t smem = sizeof(double) * (size_t)ng;
    if (smem > 200 * 1024) return fail(KPT_ERR_INVALID, "kpt_adjoint: too many materials");
    st = ensure_work(c, nsamples);
    if (st != KPT_OK) return st;
    KPT_CUDA(c->sun_J.ensure(ADJ_SKY_PARAMS));
    KPT_CUDA(c->rec_count.ensure(1));
    // room for every sample's escape and every missing pixel
    const size_t qcap = (size_t)c->W * c->H * ((size_t)nsamples + 1);
    FrameParams F = frame_params(c, sample0, nsamples);
    F.sky = sky_params(c->env);   // the replay and its Jacobians: IEEE sky arithmetic
    // the wavefront replay's records: a wave of at most ADJ_WAVE_BYTES of them
    const int D = F.max_depth;
    const size_t per_path = sizeof(float4) * ((size_t)AV_FIELDS * (D + 1) + 2) + (size_t)(D + 1);
    if (!rec) {
        const size_t fit = std::max<size_t>(1 << 16, ADJ_WAVE_BYTES / per_path);
        F.cap = (int)std::min<size_t>((size_t)F.cap, fit);
        KPT_CUDA(c->adj_vr.ensure((size_t)AV_FIELDS * (D + 1) * F.cap));
        KPT_CUDA(c->adj_vend.ensure(2 * (size_t)F.cap));
        KPT_CUDA(c->adj_vsky.ensure((size_t)F.cap));
        KPT_CUDA(c->adj_esc.ensure((size_t)F.cap + 1));
        KPT_CUDA(c->adj_vis.ensure((size_t)(D + 1) * F.cap));
        KPT_CUDA(c->adj_skyq.ensure(2 * std::min<size_t>(qcap, (size_t)INT32_MAX / 2)));
        KPT_CUDA(c->adj_skyq_count.ensure(1));
        KPT_CUDA(c->adj_skyqf.ensure(2 * std::min<size_t>(qcap, (size_t)INT32_MAX / 2)));
        KPT_CUDA(c->adj_skyqf_count.ensure(1));
    }
    AdjParams A{};
    A.adjoint = reinterpret_cast<const float4*>(adjoint);
    A.grad = grad;
    A.image = reinterpret_cast<float4*>(image);
    A.sun_J = c->sun_J.p;
    A.rec = rec;
    A.rec_count = c->rec_count.p;
    A.max_rec = max_rec;
    A.nmat = (int)c->materials.size();
    if (!rec) {   // the records' test path keeps the double Jacobians where they occur
        A.skyq = c->adj_skyq.p;
        A.skyq_count = c->adj_skyq_count.p;
        A.skyq_cap = (int)(c->adj_skyq.n / 2);
        A.skyqf = c->adj_skyqf.p;
        A.skyqf_count = c->adj_skyqf_count.p;
        A.skyqf_cap = (int)(c->adj_skyqf.n / 2);
        A.vr = c->adj_vr.p;
        A.vend = c->adj_vend.p;
        A.vsky = c->adj_vsky.p;
        A.esc = c->adj_esc.p;
        A.esc_count = c->adj_esc.p + F.cap;
        A.vis = c->adj_vis.p;
    }
    cudaStream_t s = c->stream;
    const int np = c->W * c->H;
    KPT_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * ng, s));
    if (image) KPT_CUDA(cudaMemsetAsync(image, 0, sizeof(float4) * (size_t)np, s));
    KPT_CUDA(cudaMemsetAsync(c->rec_count.p, 0, sizeof(int), s));
    if (A.skyq) KPT_CUDA(cudaMemsetAsync(A.skyq_count, 0, sizeof(int), s));
    if (A.skyqf) KPT_CUDA(cudaMemsetAsync(A.skyqf_count, 0, sizeof(int), s));
    KPT_CUDA(cudaMemsetAsync(c->counts.p, 0, 4 * sizeof(int), s));
    const void* kern = rec ? (const void*)k_adjoint_rec : (const void*)k_adj_sweep;
    for (const void* k : {kern, (const void*)k_adjoint_miss})
        KPT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    KPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PATH_BLOCK, smem));
    const int grid = std::max(1, per_sm) * c->sm_count;
    k_sky_constants<<<1, 32, 0, s>>>(F, c->sun_radiance.p);
    // the sun's double-precision Jacobian (one thread) on the side stream: only
    // the replay's sweep (or the records kernel) reads it
    KPT_CUDA(cudaEventRecord(c->ev_fork[0], s));
    KPT_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork[0], 0));
    k_adjoint_constants<<<1, 32, 0, c->side>>>(F, A);
    KPT_CUDA(cudaEventRecord(c->ev_join[0], c->side));
    k_primary<<<primary_blocks(c->W, c->H), PATH_BLOCK, 0, s>>>(F);
    k_adjoint_miss<<<c->sm_count, PATH_BLOCK, smem, s>>>(F, A);
    c->launches += 4;
    if (rec) {
        // the frozen-path records: one thread replays one sample
        KPT_CUDA(cudaStreamWaitEvent(s, c->ev_join[0], 0));
        k_adjoint_rec<<<grid, PATH_BLOCK, smem, s>>>(F, A);
        c->launches += 1;
    } else {
        // the wavefront replay, wave by wave (every pixel may hit: the last
        // waves find no work when fewer do): per level the vertices, their
        // shadow rays and the continuations, then every sample's sweep
        const long long items = (long long)np * nsamples;
        const int g_ext = persistent_grid(c, (const void*)k_extend, TRACE_BLOCK);
        const int g_shd = persistent_grid(c, (const void*)k_adj_shadow, TRACE_BLOCK);
        const int g_vtx = persistent_grid(c, (const void*)k_adj_shade, PATH_BLOCK);
        c->levels_depth = D;   // kpt_get_level_counts then reports the replay's last wave
        for (long long w0 = 0; w0 < items; w0 += F.cap) {
            KPT_CUDA(cudaMemsetAsync(c->level_counts.p, 0, sizeof(int) * LEVEL_WORDS * (size_t)(D + 2), s));
            KPT_CUDA(cudaMemsetAsync(A.vis, 0, (size_t)(D + 1) * F.cap, s));
            KPT_CUDA(cudaMemsetAsync(A.esc_count, 0, sizeof(int), s));
            for (int l = 0; l <= D; ++l) {
                if (l > 0) k_extend<<<g_ext, TRACE_BLOCK, 0, s>>>(F, l);
                k_adj_shade<<<g_vtx, PATH_BLOCK, 0, s>>>(F, A, l, w0);
                k_adj_shadow<<<g_shd, TRACE_BLOCK, 0, s>>>(F, A, l);
                c->launches += l > 0 ? 3 : 2;
            }
            k_adj_sky<<<g_vtx, PATH_BLOCK, 0, s>>>(F, A, w0);
            KPT_CUDA(cudaStreamWaitEvent(s, c->ev_join[0], 0));
            k_adj_sweep<<<grid, PATH_BLOCK, smem, s>>>(F, A, w0);
            c->launches += 2;
        }
    }
    if (A.skyq) {
        // the double (FP64 pipe) and single-precision (FP32) Jacobians side by side
        KPT_CUDA(cudaEventRecord(c->ev_fork[0], s));
        KPT_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork[0], 0));
        k_adjoint_sky_f<<<c->sm_count * 4, PATH_BLOCK, 0, c->side>>>(F, A);
        KPT_CUDA(cudaEventRecord(c->ev_join[0], c->side));
        k_adjoint_sky_d<<<c->sm_count * 4, PATH_BLOCK, 0, s>>>(F, A);
        KPT_CUDA(cudaStreamWaitEvent(s, c->ev_join[0], 0));
        c->launches += 2;
    }
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_adjoint_param_count(kpt_context* c, int* n) {
    if (!c || !n) return fail(KPT_ERR_INVALID, "kpt_adjoint_param_count: null argument");
    *n = adjoint_params(c);
    return KPT_OK;
}

kpt_status kpt_adjoint_device(kpt_context* c, int sample0, int nsamples, const float* adjoint, double* grad,
                              float* image) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    return adjoint_run(c, sample0, nsamples, adjoint, grad, image, nullptr, 0);
}

// The split adjoint: the replay of every sample in one wave, its records
// kept, and the image the gradient belongs to (forward); then the sweep of
// the kept records with dLoss/dimage and the deferred sky Jacobians
// (backward) -- the rays are traced once per gradient evaluation.
kpt_status kpt_adjoint_forward_device(kpt_context* c, int sample0, int nsamples, float* image) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    c->adj_fwd.valid = false;
    kpt_status st = ready(c);
    if (st != KPT_OK) return st;
    if (nsamples <= 0 || sample0 < 0 || !image) return fail(KPT_ERR_INVALID, "kpt_adjoint_forward_device: bad arguments");
    if (c->settings.max_depth + 1 > ADJ_MAX_VERTICES)
        return fail(KPT_ERR_INVALID, "kpt_adjoint_forward_device: max_depth above 16");
    const int ng = adjoint_params(c);
    const size_t smem = sizeof(double) * (size_t)ng;
    if (smem > 200 * 1024) return fail(KPT_ERR_INVALID, "kpt_adjoint_forward_device: too many materials");
    st = ensure_work(c, nsamples);
    if (st != KPT_OK) return st;
    const int np = c->W * c->H;
    const long long items = (long long)np * nsamples;
    FrameParams F = frame_params(c, sample0, nsamples);
    F.sky = sky_params(c->env);   // IEEE sky arithmetic, as the replay's Jacobians
    const int D = F.max_depth;
    const size_t per_path = sizeof(float4) * ((size_t)AV_FIELDS * (D + 1) + 2) + (size_t)(D + 1);
    if (items > F.cap || (size_t)items * per_path > ADJ_WAVE_BYTES)
        return fail(KPT_ERR_INVALID, "kpt_adjoint_forward_device: the samples' records exceed one replay wave "
                                     "(use kpt_adjoint_device)");
    F.cap = (int)items;
    const size_t qcap = (size_t)np * ((size_t)nsamples + 1);
    KPT_CUDA(c->sun_J.ensure(ADJ_SKY_PARAMS));
    KPT_CUDA(c->rec_count.ensure(1));
    KPT_CUDA(c->adj_vr.ensure((size_t)AV_FIELDS * (D + 1) * F.cap));
    KPT_CUDA(c->adj_vend.ensure(2 * (size_t)F.cap));
    KPT_CUDA(c->adj_vsky.ensure((size_t)F.cap));
    KPT_CUDA(c->adj_esc.ensure((size_t)F.cap + 1));
    KPT_CUDA(c->adj_vis.ensure((size_t)(D + 1) * F.cap));
    KPT_CUDA(c->adj_lpath.ensure((size_t)F.cap));
    KPT_CUDA(c->adj_skyq.ensure(2 * std::min<size_t>(qcap, (size_t)INT32_MAX / 2)));
    KPT_CUDA(c->adj_skyq_count.ensure(1));
    KPT_CUDA(c->adj_skyqf.ensure(2 * std::min<size_t>(qcap, (size_t)INT32_MAX / 2)));
    KPT_CUDA(c->adj_skyqf_count.ensure(1));
    AdjParams A{};
    A.image = reinterpret_cast<float4*>(image);
    A.lpath = c->adj_lpath.p;
    A.lpath_ready = 0;
    A.sun_J = c->sun_J.p;
    A.rec_count = c->rec_count.p;
    A.nmat = (int)c->materials.size();
    A.skyq = c->adj_skyq.p;
    A.skyq_count = c->adj_skyq_count.p;
    A.skyq_cap = (int)(c->adj_skyq.n / 2);
    A.skyqf = c->adj_skyqf.p;
    A.skyqf_count = c->adj_skyqf_count.p;
    A.skyqf_cap = (int)(c->adj_skyqf.n / 2);
    A.vr = c->adj_vr.p;
    A.vend = c->adj_vend.p;
    A.vsky = c->adj_vsky.p;
    A.esc = c->adj_esc.p;
    A.esc_count = c->adj_esc.p + F.cap;
    A.vis = c->adj_vis.p;
    cudaStream_t s = c->stream;
    KPT_CUDA(cudaMemsetAsync(image, 0, sizeof(float4) * (size_t)np, s));
    KPT_CUDA(cudaMemsetAsync(c->counts.p, 0, 4 * sizeof(int), s));
    KPT_CUDA(cudaMemsetAsync(c->level_counts.p, 0, sizeof(int) * LEVEL_WORDS * (size_t)(D + 2), s));
    KPT_CUDA(cudaMemsetAsync(A.vis, 0, (size_t)(D + 1) * F.cap, s));
    KPT_CUDA(cudaMemsetAsync(A.esc_count, 0, sizeof(int), s));
    for (const void* k : {(const void*)k_adj_sweep, (const void*)k_adjoint_miss})
        KPT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    KPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adj_sweep, PATH_BLOCK, smem));
    const int grid = std::max(1, per_sm) * c->sm_count;
    const int g_ext = persistent_grid(c, (const void*)k_extend, TRACE_BLOCK);
    const int g_shd = persistent_grid(c, (const void*)k_adj_shadow, TRACE_BLOCK);
    const int g_vtx = persistent_grid(c, (const void*)k_adj_shade, PATH_BLOCK);
    c->levels_depth = D;
    k_sky_constants<<<1, 32, 0, s>>>(F, c->sun_radiance.p);
    // the sun's double-precision Jacobian (one thread; it depends on the sky
    // parameters only) on the side stream beside the replay, for the sweep
    KPT_CUDA(cudaEventRecord(c->ev_fork[0], s));
    KPT_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork[0], 0));
    k_adjoint_constants<<<1, 32, 0, c->side>>>(F, A);
    KPT_CUDA(cudaEventRecord(c->ev_join[0], c->side));
    k_primary<<<primary_blocks(c->W, c->H), PATH_BLOCK, 0, s>>>(F);
    k_adjoint_miss<<<c->sm_count, PATH_BLOCK, smem, s>>>(F, A);   // the missing pixels' image
    for (int l = 0; l <= D; ++l) {
        if (l > 0) k_extend<<<g_ext, TRACE_BLOCK, 0, s>>>(F, l);
        k_adj_shade<<<g_vtx, PATH_BLOCK, 0, s>>>(F, A, l, 0);
        k_adj_shadow<<<g_shd, TRACE_BLOCK, 0, s>>>(F, A, l);
    }
    k_adj_sky<<<g_vtx, PATH_BLOCK, 0, s>>>(F, A, 0);
    k_adj_sweep<<<grid, PATH_BLOCK, smem, s>>>(F, A, 0);   // the hit pixels' image
    KPT_CUDA(cudaStreamWaitEvent(s, c->ev_join[0], 0));
    c->launches += 7 + 3 * D;
    KPT_CUDA(cudaGetLastError());
    kpt_context::AdjForward& K = c->adj_fwd;
    K.F = F;
    K.A = A;
    K.A.image = nullptr;
    K.version = c->scene_version;
    K.materials = c->materials;
    K.env = c->env;
    K.settings = c->settings;
    std::memcpy(K.inv_proj, c->inv_proj, sizeof K.inv_proj);
    std::memcpy(K.inv_view, c->inv_view, sizeof K.inv_view);
    K.W = c->W;
    K.H = c->H;
    K.valid = true;
    return KPT_OK;
}

kpt_status kpt_adjoint_backward_device(kpt_context* c, const float* adjoint, double* grad) {
    if (!c || !adjoint || !grad) return fail(KPT_ERR_INVALID, "kpt_adjoint_backward_device: null argument");
    KPT_CUDA(cudaSetDevice(c->device));
    kpt_context::AdjForward& K = c->adj_fwd;
    // (a transform set since the forward call leaves the TLAS to rebuild)
    const bool same = K.valid && !c->tlas_dirty && K.version == c->scene_version &&
                      K.materials.size() == c->materials.size() &&
                      std::memcmp(K.materials.data(), c->materials.data(), sizeof(kpt_material) * K.materials.size()) == 0 &&
                      std::memcmp(&K.env, &c->env, sizeof K.env) == 0 &&
                      std::memcmp(&K.settings, &c->settings, sizeof K.settings) == 0 &&
                      std::memcmp(K.inv_proj, c->inv_proj, sizeof K.inv_proj) == 0 &&
                      std::memcmp(K.inv_view, c->inv_view, sizeof K.inv_view) == 0 && K.W == c->W && K.H == c->H;
    if (!same)
        return fail(KPT_ERR_STATE, "kpt_adjoint_backward_device: no kept forward records for the current scene "
                                   "(call kpt_adjoint_forward_device first, with nothing rendered or changed between)");
    K.valid = false;   // one backward per forward: the sky queues and the gradient start from zero
    const FrameParams& F = K.F;
    AdjParams A = K.A;
    A.adjoint = reinterpret_cast<const float4*>(adjoint);
    A.grad = grad;
    A.lpath_ready = 1;
    const int ng = adjoint_params(c);
    const size_t smem = sizeof(double) * (size_t)ng;
    int per_sm = 0;
    KPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adj_sweep, PATH_BLOCK, smem));
    const int grid = std::max(1, per_sm) * c->sm_count;
    cudaStream_t s = c->stream;
    KPT_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * ng, s));
    KPT_CUDA(cudaMemsetAsync(A.skyq_count, 0, sizeof(int), s));
    KPT_CUDA(cudaMemsetAsync(A.skyqf_count, 0, sizeof(int), s));
    // (the sun's Jacobian, A.sun_J, came with the forward call)
    k_adjoint_miss<<<c->sm_count, PATH_BLOCK, smem, s>>>(F, A);
    k_adj_sweep<<<grid, PATH_BLOCK, smem, s>>>(F, A, 0);
    KPT_CUDA(cudaEventRecord(c->ev_fork[0], s));
    KPT_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork[0], 0));
    k_adjoint_sky_f<<<c->sm_count * 4, PATH_BLOCK, 0, c->side>>>(F, A);
    KPT_CUDA(cudaEventRecord(c->ev_join[0], c->side));
    k_adjoint_sky_d<<<c->sm_count * 4, PATH_BLOCK, 0, s>>>(F, A);
    KPT_CUDA(cudaStreamWaitEvent(s, c->ev_join[0], 0));
    c->launches += 4;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_adjoint(kpt_context* c, int sample0, int nsamples, const float* adjoint, double* grad, float* image) {
    if (!c || !adjoint || !grad) return fail(KPT_ERR_INVALID, "kpt_adjoint: null argument");
    KPT_CUDA(cudaSetDevice(c->device));
    const size_t np = (size_t)c->W * c->H;
    const int ng = adjoint_params(c);
    KPT_CUDA(c->adj_in.ensure(4 * np));
    KPT_CUDA(c->adj_grad.ensure(ng));
    if (image) KPT_CUDA(c->adj_image.ensure(4 * np));
    KPT_CUDA(cudaMemcpyAsync(c->adj_in.p, adjoint, sizeof(float) * 4 * np, cudaMemcpyHostToDevice, c->stream));
    kpt_status st = adjoint_run(c, sample0, nsamples, c->adj_in.p, c->adj_grad.p, image ? c->adj_image.p : nullptr,
                                nullptr, 0);
    if (st != KPT_OK) return st;
    KPT_CUDA(cudaMemcpyAsync(grad, c->adj_grad.p, sizeof(double) * ng, cudaMemcpyDeviceToHost, c->stream));
    if (image)
        KPT_CUDA(cudaMemcpyAsync(image, c->adj_image.p, sizeof(float) * 4 * np, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    return KPT_OK;
}

int kpt_adjoint_record_size(void) { return (int)sizeof(AdjRec); }

kpt_status kpt_sky_grad_device(kpt_context* c, int n, const float* dirs, float* rgb) {
    if (!c || n < 0 || (n > 0 && (!dirs || !rgb))) return fail(KPT_ERR_INVALID, "kpt_sky_grad_device: bad arguments");
    KPT_CUDA(cudaSetDevice(c->device));
    if (n == 0) return KPT_OK;
    k_sky_grad<<<(n + 127) / 128, 128, 0, c->stream>>>(sky_params(c->env), n, (const float3*)dirs, (float3*)rgb);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    return KPT_OK;
}

kpt_status kpt_adjoint_records_device(kpt_context* c, int sample0, int nsamples, const float* adjoint, double* grad,
                                      void* records, int max_records, int* count) {
    if (!c || !records || max_records <= 0 || !count)
        return fail(KPT_ERR_INVALID, "kpt_adjoint_records_device: bad arguments");
    kpt_status st = adjoint_run(c, sample0, nsamples, adjoint, grad, nullptr, static_cast<AdjRec*>(records), max_records);
    if (st != KPT_OK) return st;
    KPT_CUDA(cudaMemcpyAsync(count, c->rec_count.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    return KPT_OK;
}

kpt_status kpt_get_tuning(kpt_context* c, kpt_tuning* t) {
    if (!c || !t) return fail(KPT_ERR_INVALID, "kpt_get_tuning: null argument");
    *t = c->tuning;
    return KPT_OK;
}

}  // extern "C"

struct kpt_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev_start = nullptr, ev_fork = nullptr, ev_done = nullptr;
    std::vector<cudaEvent_t> ev_end, ev_dep, ev_pre;   // per job
    int n = 0;
    bool pending = false;
    struct Choice {
        kpt_tuning tuning;
        int lanes;
        float ms;
    };
    std::map<std::string, Choice> cache;   // batch signature -> autotuned choice
    // One queue per ray stage spanning the jobs (kpt_batch_set_shared): the
    // merged scene, the key it was built for (each job and its scene
    // version), the jobs' table and the level queues.
    int shared = 1;
    cudaStream_t side = nullptr;   // the shadow rays beside the extension rays
    cudaEvent_t ev_counts = nullptr, ev_shadow = nullptr, ev_level = nullptr;
    DBuf<BvhNode> m_nodes, m_tlas;
    DBuf<float4> m_tris;
    DBuf<MeshRec> m_meshes;
    DBuf<InstRec> m_inst;
    SceneView m_view{};
    std::vector<std::pair<const kpt_context*, unsigned long long>> m_key;
    std::vector<int> m_tlas_root, m_inst_base;
    std::vector<BatchJob> h_jobs;
    DBuf<BatchJob> d_jobs;
    DBuf<int> d_queues;                    // extension prefix [n + 1], shadow prefix [n + 1], fetch [2]
    DBuf<unsigned long long> d_counters;   // traversal counters of the batch's ray kernels
};

namespace {

kpt_status batch_events(kpt_batch* b, int n) {
    while ((int)b->ev_end.size() < n) {
        cudaEvent_t e = nullptr, d = nullptr, p = nullptr;
        KPT_CUDA(cudaEventCreate(&e));
        KPT_CUDA(cudaEventCreateWithFlags(&d, cudaEventDisableTiming));
        KPT_CUDA(cudaEventCreateWithFlags(&p, cudaEventDisableTiming));
        b->ev_end.push_back(e);
        b->ev_dep.push_back(d);
        b->ev_pre.push_back(p);
    }
    return KPT_OK;
}

double job_cost(const kpt_context* c, int spp) {
    return (double)c->W * c->H * spp * (c->settings.max_depth + 1);
}

// The batch's merged scene: every job's BLAS nodes, triangles, meshes,
// instances and TLAS nodes one after the other, their indices moved by the
// job's offsets (enqueued on the batch stream; rebuilt only when the jobs or
// one of their scenes changed).
kpt_status merge_scenes(kpt_batch* b, int n, kpt_context* const* jobs) {
    std::vector<std::pair<const kpt_context*, unsigned long long>> key(n);
    for (int j = 0; j < n; ++j) key[j] = {jobs[j], jobs[j]->scene_version};
    if (key == b->m_key) return KPT_OK;
    long long nn = 0, nt = 0, nm = 0, ni = 0, nl = 0;
    for (int j = 0; j < n; ++j) {
        nn += jobs[j]->n_nodes;
        nt += jobs[j]->n_tris;
        nm += (long long)jobs[j]->meshes.size();
        ni += (long long)jobs[j]->instances.size();
        nl += jobs[j]->view.ntlas;
    }
    if (nn > INT32_MAX / 2 || nt > INT32_MAX / 4 || nm > INT32_MAX || ni > INT32_MAX / 2 || nl > INT32_MAX / 2)
        return fail(KPT_ERR_INVALID, "kpt_submit_batch: the jobs' scenes together are too large to merge");
    b->m_key.clear();
    KPT_CUDA(b->m_nodes.ensure(nn));
    KPT_CUDA(b->m_tris.ensure(3 * nt));
    KPT_CUDA(b->m_meshes.ensure(nm));
    KPT_CUDA(b->m_inst.ensure(ni));
    KPT_CUDA(b->m_tlas.ensure(nl));
    b->m_tlas_root.assign(n, 0);
    b->m_inst_base.assign(n, 0);
    int node_base = 0, tri_base = 0, mesh_base = 0, inst_base = 0, tlas_base = 0;
    auto blocks = [](int k) { return (k + 255) / 256; };
    for (int j = 0; j < n; ++j) {
        const kpt_context* c = jobs[j];
        const int nodes = c->n_nodes, tris = c->n_tris, meshes = (int)c->meshes.size();
        const int inst = (int)c->instances.size(), tlas = c->view.ntlas;
        if (nodes > 0)
            k_merge_nodes<<<blocks(nodes), 256, 0, b->stream>>>(c->d_nodes.p, nodes, b->m_nodes.p + node_base,
                                                                 node_base, tri_base);
        if (tris > 0)
            KPT_CUDA(cudaMemcpyAsync(b->m_tris.p + 3 * (size_t)tri_base, c->d_tris.p, 3 * sizeof(float4) * (size_t)tris,
                                     cudaMemcpyDeviceToDevice, b->stream));
        if (meshes > 0)
            k_merge_meshes<<<blocks(meshes), 256, 0, b->stream>>>(c->d_meshes.p, meshes, b->m_meshes.p + mesh_base,
                                                                   node_base, tri_base);
        if (inst > 0)
            k_merge_inst<<<blocks(inst), 256, 0, b->stream>>>(c->d_inst.p, inst, b->m_inst.p + inst_base, mesh_base);
        if (tlas > 0)
            k_merge_nodes<<<blocks(tlas), 256, 0, b->stream>>>(c->d_tlas.p, tlas, b->m_tlas.p + tlas_base, tlas_base,
                                                                inst_base);
        KPT_CUDA(cudaGetLastError());
        b->m_tlas_root[j] = c->view.tlas_root_leaf ? -inst_base - 1 : tlas_base;
        b->m_inst_base[j] = inst_base;
        node_base += nodes;
        tri_base += tris;
        mesh_base += meshes;
        inst_base += inst;
        tlas_base += tlas;
    }
    SceneView v{};
    v.nodes = b->m_nodes.p;
    v.tris = b->m_tris.p;
    v.meshes = b->m_meshes.p;
    v.inst = b->m_inst.p;
    v.tlas = b->m_tlas.p;
    v.ntlas = tlas_base;
    v.ninst = inst_base;
    v.fetch_batch = jobs[0]->view.fetch_batch;
    b->m_view = v;
    b->m_key = key;
    return KPT_OK;
}

std::string batch_signature(int n, kpt_context* const* jobs, const int32_t* spp) {
    std::string sig;
    for (int j = 0; j < n; ++j) {
        const kpt_context* c = jobs[j];
        sig += std::to_string(c->W) + "x" + std::to_string(c->H) + "x" + std::to_string(spp[j]) + "d" +
               std::to_string(c->settings.max_depth) + "i" + std::to_string(c->instances.size()) + ";";
    }
    return sig;
}

}  // namespace

// The batch as one graph whose ray stages span the jobs: each job's camera
// rays, shading, sky, accumulation and post chain on its own streams; per
// level, once every job has shaded it, one k_batch_level, one k_shadow_batch
// (the level's shadow rays of every job) beside one k_extend_batch (the next
// level's extension rays of every job), in the merged scene.  Each job's
// sky of a level follows the batch's shadow rays of that level, its next
// shading both ray kernels, so every job's buffers see the same sequence of
// writes as when it renders alone.
static kpt_status submit_shared(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp,
                                const std::vector<FrameParams>& F) {
    kpt_status st = merge_scenes(b, n, jobs);
    if (st != KPT_OK) return st;
    int D = 0;
    b->h_jobs.assign(n, BatchJob{});
    for (int j = 0; j < n; ++j) {
        const kpt_context* c = jobs[j];
        BatchJob& J = b->h_jobs[j];
        J.tlas_lo = c->view.tlas_lo;
        J.tlas_hi = c->view.tlas_hi;
        J.paths[0] = F[j].paths[0];
        J.paths[1] = F[j].paths[1];
        J.hits = F[j].hits;
        J.shadow = F[j].shadow;
        J.radiance = F[j].radiance;
        J.level_counts = F[j].level_counts;
        J.counts = F[j].counts;
        J.tlas_root = b->m_tlas_root[j];
        J.ninst = c->view.ninst;
        J.inst_base = b->m_inst_base[j];
        J.cap = F[j].cap;
        J.max_depth = F[j].max_depth;
        D = std::max(D, F[j].max_depth);
    }
    KPT_CUDA(b->d_jobs.upload(b->h_jobs.data(), n, b->stream));
    KPT_CUDA(b->d_queues.ensure(2 * (size_t)(n + 1) + 2));
    KPT_CUDA(b->d_counters.ensure(16));
    KPT_CUDA(cudaMemsetAsync(b->d_counters.p, 0, 16 * sizeof(unsigned long long), b->stream));
    BatchQueues Q;
    Q.ext_prefix = b->d_queues.p;
    Q.shd_prefix = b->d_queues.p + (n + 1);
    Q.fetch = b->d_queues.p + 2 * (n + 1);
    Q.jobs = b->d_jobs.p;
    Q.njobs = n;
    const int sms = jobs[0]->sm_count;
    int per_ext = 0, per_shd = 0;
    KPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_ext, k_extend_batch, TRACE_BLOCK, 0));
    KPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_shd, k_shadow_batch, TRACE_BLOCK, 0));
    const int g_ext = std::max(1, per_ext) * sms, g_shd = std::max(1, per_shd) * sms;
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        cudaEventRecordWithFlags(b->ev_start, b->stream, cudaEventRecordExternal);
        cudaEventRecord(b->ev_fork, b->stream);
        for (int j = 0; j < n; ++j) {
            kpt_context* c = jobs[j];
            cudaStreamWaitEvent(c->stream, b->ev_fork, 0);
            enqueue_camera(c, F[j]);
            enqueue_wave_start(c, F[j], true);
        }
        for (int l = 0; l <= D; ++l) {
            for (int j = 0; j < n; ++j) {
                kpt_context* c = jobs[j];
                if (F[j].max_depth < l) continue;
                if (l > 0) cudaStreamWaitEvent(c->stream, b->ev_level, 0);
                enqueue_shade(c, F[j], l, 0);
                cudaEventRecord(c->ev_fork[l], c->stream);
                cudaStreamWaitEvent(b->stream, c->ev_fork[l], 0);
            }
            k_batch_level<<<1, 32, 0, b->stream>>>(Q, l);
            cudaEventRecord(b->ev_counts, b->stream);
            cudaStreamWaitEvent(b->side, b->ev_counts, 0);
            k_shadow_batch<<<g_shd, TRACE_BLOCK, 0, b->side>>>(b->m_view, Q, l, b->d_counters.p);
            cudaEventRecord(b->ev_shadow, b->side);
            for (int j = 0; j < n; ++j) {
                kpt_context* c = jobs[j];
                if (F[j].max_depth < l) continue;
                // the level's sky entries are final (their paths ended)
                cudaStreamWaitEvent(c->sky, b->ev_shadow, 0);
                k_sky_queue<<<persistent_grid(c, (const void*)k_sky_queue, PATH_BLOCK), PATH_BLOCK, 0, c->sky>>>(F[j], l);
                c->launches += 2;   // its shading and sky of the level
            }
            if (l < D) k_extend_batch<<<g_ext, TRACE_BLOCK, 0, b->stream>>>(b->m_view, Q, l + 1, b->d_counters.p);
            cudaStreamWaitEvent(b->stream, b->ev_shadow, 0);
            cudaEventRecord(b->ev_level, b->stream);
            // the jobs whose last level this was: their sky, ray counts,
            // accumulation and post chain
            for (int j = 0; j < n; ++j) {
                kpt_context* c = jobs[j];
                if (F[j].max_depth != l) continue;
                cudaStreamWaitEvent(c->stream, b->ev_shadow, 0);
                cudaEventRecord(c->ev_sky, c->sky);
                cudaStreamWaitEvent(c->stream, c->ev_sky, 0);
                k_count_rays<<<1, 32, 0, c->stream>>>(F[j]);
                c->launches += 1;
                enqueue_path_end(c, F[j]);
                enqueue_post(c, F[j], c->frame_index + spp[j], c->settings.frame_delta_ms);
                cudaEventRecordWithFlags(b->ev_end[j], c->stream, cudaEventRecordExternal);
                cudaEventRecord(b->ev_dep[j], c->stream);
            }
        }
        for (int j = 0; j < n; ++j) cudaStreamWaitEvent(b->stream, b->ev_dep[j], 0);
        ce = cudaStreamEndCapture(b->stream, &g);
    }
    KPT_CUDA(ce);
    st = instantiate(g, &b->exec);
    if (st != KPT_OK) return st;
    KPT_CUDA(cudaGraphLaunch(b->exec, b->stream));
    KPT_CUDA(cudaEventRecord(b->ev_done, b->stream));
    for (int j = 0; j < n; ++j) {
        KPT_CUDA(cudaStreamWaitEvent(jobs[j]->stream, b->ev_done, 0));
        finish_frame(jobs[j], spp[j]);
    }
    return KPT_OK;
}

extern "C" {

kpt_status kpt_batch_set_shared(kpt_batch* b, int shared) {
    if (!b || (shared != 0 && shared != 1)) return fail(KPT_ERR_INVALID, "kpt_batch_set_shared: bad arguments");
    if (b->pending) return fail(KPT_ERR_STATE, "kpt_batch_set_shared: a batch is pending");
    b->shared = shared;
    return KPT_OK;
}

kpt_status kpt_batch_get_shared(kpt_batch* b, int* shared) {
    if (!b || !shared) return fail(KPT_ERR_INVALID, "kpt_batch_get_shared: bad arguments");
    *shared = b->shared;
    return KPT_OK;
}

kpt_status kpt_batch_create(int device, kpt_batch** out) {
    if (!out) return fail(KPT_ERR_INVALID, "kpt_batch_create: null output");
    int nd = 0;
    KPT_CUDA(cudaGetDeviceCount(&nd));
    if (device < 0 || device >= nd) return fail(KPT_ERR_INVALID, "kpt_batch_create: no such device");
    KPT_CUDA(cudaSetDevice(device));
    kpt_batch* b = new kpt_batch();
    b->device = device;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_counts, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_shadow, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_level, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev_start) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming) != cudaSuccess) {
        kpt_batch_destroy(b);
        return fail(KPT_ERR_CUDA, "kpt_batch_create: stream or event creation failed");
    }
    *out = b;
    return KPT_OK;
}

kpt_status kpt_batch_destroy(kpt_batch* b) {
    if (!b) return KPT_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (cudaEvent_t e : {b->ev_start, b->ev_fork, b->ev_done})
        if (e) cudaEventDestroy(e);
    for (auto* v : {&b->ev_end, &b->ev_dep, &b->ev_pre})
        for (cudaEvent_t e : *v) cudaEventDestroy(e);
    for (cudaEvent_t e : {b->ev_counts, b->ev_shadow, b->ev_level})
        if (e) cudaEventDestroy(e);
    b->m_nodes.release(); b->m_tlas.release(); b->m_tris.release(); b->m_meshes.release(); b->m_inst.release();
    b->d_jobs.release(); b->d_queues.release(); b->d_counters.release();
    if (b->side) cudaStreamDestroy(b->side);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return KPT_OK;
}

kpt_status kpt_submit_batch(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp, int lanes) {
    if (!b || n <= 0 || !jobs || !spp) return fail(KPT_ERR_INVALID, "kpt_submit_batch: bad arguments");
    if (b->pending) return fail(KPT_ERR_STATE, "kpt_submit_batch: the previous batch was not waited for");
    for (int j = 0; j < n; ++j) {
        if (!jobs[j]) return fail(KPT_ERR_INVALID, "kpt_submit_batch: null job");
        if (jobs[j]->device != b->device) return fail(KPT_ERR_INVALID, "kpt_submit_batch: job on another device");
        if (spp[j] <= 0) return fail(KPT_ERR_INVALID, "kpt_submit_batch: spp must be positive");
        for (int k = 0; k < j; ++k)
            if (jobs[k] == jobs[j]) return fail(KPT_ERR_INVALID, "kpt_submit_batch: a context appears twice");
    }
    KPT_CUDA(cudaSetDevice(b->device));
    kpt_status st = batch_events(b, n);
    if (st != KPT_OK) return st;
    // host work of every frame, then the batch stream waits for what it enqueued
    std::vector<FrameParams> F(n);
    for (int j = 0; j < n; ++j) {
        st = prepare_frame(jobs[j], spp[j], &F[j]);
        if (st != KPT_OK) return st;
        KPT_CUDA(cudaEventRecord(b->ev_pre[j], jobs[j]->stream));
        KPT_CUDA(cudaStreamWaitEvent(b->stream, b->ev_pre[j], 0));
    }
    // one queue per ray stage spanning the jobs where every job's frame is
    // one wave without the octant sort; otherwise each job's frame is a
    // branch of the graph
    bool shared = b->shared != 0;
    long long caps = 0;
    for (int j = 0; j < n && shared; ++j) {
        const kpt_context* c = jobs[j];
        const long long items = (long long)c->W * c->H * spp[j];
        shared = items <= F[j].cap && F[j].unsorted == nullptr && c->tf == nullptr &&
                 c->ev_fork.size() >= (size_t)F[j].max_depth + 1;
        caps += F[j].cap;
    }
    if (shared && caps <= INT32_MAX) {
        st = submit_shared(b, n, jobs, spp, F);
        if (st != KPT_OK) return st;
        b->n = n;
        b->pending = true;
        return KPT_OK;
    }
    // jobs dealt longest first to the least-loaded lane
    const int L = (lanes <= 0 || lanes >= n) ? n : lanes;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return job_cost(jobs[a], spp[a]) > job_cost(jobs[c], spp[c]); });
    std::vector<double> load(L, 0.0);
    std::vector<int> last(L, -1), prev(n, -1);
    for (int j : order) {
        int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        prev[j] = last[l];
        last[l] = j;
        load[l] += job_cost(jobs[j], spp[j]);
    }
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        cudaEventRecordWithFlags(b->ev_start, b->stream, cudaEventRecordExternal);
        cudaEventRecord(b->ev_fork, b->stream);
        for (int j : order) {
            kpt_context* c = jobs[j];
            cudaStreamWaitEvent(c->stream, prev[j] < 0 ? b->ev_fork : b->ev_dep[prev[j]], 0);
            enqueue_frame(c, F[j], c->frame_index + spp[j], c->settings.frame_delta_ms);
            cudaEventRecordWithFlags(b->ev_end[j], c->stream, cudaEventRecordExternal);
            cudaEventRecord(b->ev_dep[j], c->stream);
        }
        for (int l = 0; l < L; ++l)
            if (last[l] >= 0) cudaStreamWaitEvent(b->stream, b->ev_dep[last[l]], 0);
        ce = cudaStreamEndCapture(b->stream, &g);
    }
    KPT_CUDA(ce);
    st = instantiate(g, &b->exec);
    if (st != KPT_OK) return st;
    KPT_CUDA(cudaGraphLaunch(b->exec, b->stream));
    // later work on a job's own stream (reads, its next frame) follows the batch
    KPT_CUDA(cudaEventRecord(b->ev_done, b->stream));
    for (int j = 0; j < n; ++j) {
        KPT_CUDA(cudaStreamWaitEvent(jobs[j]->stream, b->ev_done, 0));
        finish_frame(jobs[j], spp[j]);
    }
    b->n = n;
    b->pending = true;
    return KPT_OK;
}

kpt_status kpt_wait_batch(kpt_batch* b, float* job_ms, float* total_ms) {
    if (!b) return fail(KPT_ERR_INVALID, "kpt_wait_batch: null batch");
    if (!b->pending) return fail(KPT_ERR_STATE, "kpt_wait_batch: no batch submitted");
    KPT_CUDA(cudaSetDevice(b->device));
    b->pending = false;
    KPT_CUDA(cudaStreamSynchronize(b->stream));
    float total = 0.0f;
    for (int j = 0; j < b->n; ++j) {
        float ms = 0.0f;
        KPT_CUDA(cudaEventElapsedTime(&ms, b->ev_start, b->ev_end[j]));
        if (job_ms) job_ms[j] = ms;
        total = std::max(total, ms);
    }
    if (total_ms) *total_ms = total;
    return KPT_OK;
}

// Device time of one batch under (tuning, lanes): one untimed submission, then
// the mean of `reps` timed ones.
static kpt_status time_batch(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp,
                             const kpt_tuning& t, int lanes, int reps, float* ms) {
    for (int j = 0; j < n; ++j) {
        kpt_status st = kpt_set_tuning(jobs[j], &t);
        if (st != KPT_OK) return st;
    }
    double sum = 0.0;
    for (int r = 0; r <= reps; ++r) {
        kpt_status st = kpt_submit_batch(b, n, jobs, spp, lanes);
        if (st != KPT_OK) return st;
        float total = 0.0f;
        st = kpt_wait_batch(b, nullptr, &total);
        if (st != KPT_OK) return st;
        if (r > 0) sum += total;
    }
    *ms = (float)(sum / reps);
    return KPT_OK;
}

kpt_status kpt_autotune_batch(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp, int reps,
                              kpt_tuning* best, int32_t* best_lanes, float* best_ms) {
    if (!b || n <= 0 || !jobs || !spp || reps <= 0) return fail(KPT_ERR_INVALID, "kpt_autotune_batch: bad arguments");
    for (int j = 0; j < n; ++j)
        if (!jobs[j]) return fail(KPT_ERR_INVALID, "kpt_autotune_batch: null job");
    const std::string sig = batch_signature(n, jobs, spp);
    auto hit = b->cache.find(sig);
    kpt_batch::Choice choice;
    if (hit != b->cache.end()) {
        choice = hit->second;
    } else {
        // coordinate descent from the single-frame defaults: lanes, then the
        // grid share, the wave capacity and the shading block, each value
        // tried with the others at their best so far
        kpt_tuning cur;
        kpt_tuning_default(&cur);
        int lanes = n;
        float cur_ms = 0.0f;
        kpt_status st = time_batch(b, n, jobs, spp, cur, lanes, reps, &cur_ms);
        if (st != KPT_OK) return st;
        std::vector<int> lane_opts;
        for (int l = n / 2; l >= 1 && (int)lane_opts.size() < 3; l /= 2) lane_opts.push_back(l);
        for (int l : lane_opts) {
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, cur, l, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; lanes = l; }
        }
        for (float g : {0.5f, 0.25f, 0.125f}) {
            kpt_tuning t = cur;
            t.grid_scale = g;
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, t, lanes, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; cur = t; }
        }
        for (int w : {1 << 23, 1 << 21}) {
            kpt_tuning t = cur;
            t.wave_cap = w;
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, t, lanes, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; cur = t; }
        }
        for (int blk : {64, 256}) {
            kpt_tuning t = cur;
            t.shade_block = blk;
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, t, lanes, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; cur = t; }
        }
        for (int fb : {4, 16}) {
            kpt_tuning t = cur;
            t.fetch_batch = fb;
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, t, lanes, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; cur = t; }
        }
        {
            kpt_tuning t = cur;
            t.sort_rays = 1;
            float ms = 0.0f;
            st = time_batch(b, n, jobs, spp, t, lanes, reps, &ms);
            if (st != KPT_OK) return st;
            if (ms < cur_ms) { cur_ms = ms; cur = t; }
        }
        choice = {cur, lanes, cur_ms};
        b->cache[sig] = choice;
    }
    for (int j = 0; j < n; ++j) {
        kpt_status st = kpt_set_tuning(jobs[j], &choice.tuning);
        if (st != KPT_OK) return st;
        st = clear_accumulation(jobs[j]);
        if (st != KPT_OK) return st;
    }
    if (best) *best = choice.tuning;
    if (best_lanes) *best_lanes = choice.lanes;
    if (best_ms) *best_ms = choice.ms;
    return KPT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Ray bounces without device allocation.
//
// kpt_trace_bounces stages the caller's host rays and hits in device buffers
// it allocates with cudaMalloc on every call.  Some callers cannot do that:
// a frame loop that must never stall (cudaMalloc and cudaFree can
// synchronise the whole device), or an application that reserves its device
// memory up front and forbids later growth.  kpt_trace_bounces_noalloc
// serves them: the staging lives in one fixed array below, part of the
// library's device image, so every GPU that loads libkpt.so holds these
// 8 MiB until the process exits.
//
// The array is shared by every call in the process and keeps the last call's
// contents; nothing in it has to start at zero (the inputs are copied in and
// the kernel writes every output slot).  Calls that overlap on the GPU --
// from two threads, or on two contexts of one device at once -- race on it.
// A call returns only after its results are in host memory, so calls made one
// after another from one thread never overlap.

namespace {

constexpr size_t NOALLOC_BYTES = size_t(8) << 20;   // KPT_NOALLOC_STAGING_BYTES in kpt.h
static __device__ __align__(256) unsigned char g_noalloc_staging[NOALLOC_BYTES];

// Device address of the staging array, looked up once per device with that
// device current (a host-side use of the symbol itself would not be a device
// address).
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

kpt_status noalloc_staging(int device, unsigned char** out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return fail(KPT_ERR_INVALID, "device index too large");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_staging);
        if (e != cudaSuccess || !p)
            return fail(KPT_ERR_CUDA, std::string("cudaGetSymbolAddress(staging): ") + cudaGetErrorString(e));
        g_noalloc_ptr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_ptr[device]);
    return KPT_OK;
}

}  // namespace

extern "C" kpt_status kpt_trace_bounces_noalloc(kpt_context* c, int n, const float* o, const float* d, int nb,
                                                int32_t* inst, int32_t* tri, float* t) {
    if (!c) return fail(KPT_ERR_INVALID, "null context");
    if (n < 0 || nb < 0 || (n > 0 && (!o || !d || !inst || !tri || !t)))
        return fail(KPT_ERR_INVALID, "kpt_trace_bounces_noalloc: bad arguments");
    if (!c->committed) return fail(KPT_ERR_STATE, "no committed scene");
    if (c->tlas_dirty)   // rebuilding the TLAS could grow a device buffer
        return fail(KPT_ERR_STATE, "kpt_trace_bounces_noalloc: instance transforms changed; render or trace once first");
    // origin + direction in, (instance, triangle, t) per bounce out; checked
    // in an order that cannot overflow: nbounces first, then n against the
    // bytes one ray takes
    constexpr size_t max_nb = (NOALLOC_BYTES - 24) / 12 - 1;
    if ((size_t)nb > max_nb || (size_t)n > NOALLOC_BYTES / (24 + 12 * ((size_t)nb + 1)))
        return fail(KPT_ERR_INVALID, "kpt_trace_bounces_noalloc: n * (24 + 12 * (nbounces + 1)) bytes exceed the "
                                     "8 MiB staging array (KPT_NOALLOC_STAGING_BYTES)");
    if (n == 0) return KPT_OK;
    KPT_CUDA(cudaSetDevice(c->device));
    unsigned char* base = nullptr;
    kpt_status st = noalloc_staging(c->device, &base);
    if (st != KPT_OK) return st;
    const size_t nr = (size_t)n, no = nr * ((size_t)nb + 1);
    float* d_o = reinterpret_cast<float*>(base);          // 12 n bytes
    float* d_d = d_o + 3 * nr;                              // 12 n bytes
    int32_t* d_inst = reinterpret_cast<int32_t*>(d_d + 3 * nr);
    int32_t* d_tri = d_inst + no;
    float* d_t = reinterpret_cast<float*>(d_tri + no);
    KPT_CUDA(cudaMemcpyAsync(d_o, o, 12 * nr, cudaMemcpyHostToDevice, c->stream));
    KPT_CUDA(cudaMemcpyAsync(d_d, d, 12 * nr, cudaMemcpyHostToDevice, c->stream));
    // the launch of kpt_trace_bounces_device: the same kernel and settings, so
    // both calls return the same hits; the context's chain counter (not part
    // of the staging array) must start at zero
    KPT_CUDA(cudaMemsetAsync(c->fetch.p, 0, sizeof(int), c->stream));
    SceneView v = c->view;
    v.fetch_batch = 1;
    k_trace_chains<<<trace_grid(c, (const void*)k_trace_chains, n), TRACE_BLOCK, 0, c->stream>>>(
        v, n, (const float3*)d_o, (const float3*)d_d, nb, d_inst, d_tri, d_t, c->fetch.p, c->counters.p);
    c->launches += 1;
    KPT_CUDA(cudaGetLastError());
    KPT_CUDA(cudaMemcpyAsync(inst, d_inst, 4 * no, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaMemcpyAsync(tri, d_tri, 4 * no, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaMemcpyAsync(t, d_t, 4 * no, cudaMemcpyDeviceToHost, c->stream));
    KPT_CUDA(cudaStreamSynchronize(c->stream));
    return KPT_OK;
}
