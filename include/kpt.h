/* kpt.h -- C ABI of the GB300 path tracer (libkpt.so).
 *
 * The reference exposes its path-tracing hot path through the C++ class
 * KittlesPT::Renderer (KittlesPT/src/renderer.hpp:13-58) and the POD scene
 * types of KittlesPT/src/pod_types.hpp.  This header is the plain-C boundary
 * a host binding (ctypes, cgo, JNI, N-API) calls; include/kittlespt_gb300/
 * renderer.hpp puts the reference's C++ method set back on top of it.
 *
 * Conventions: every function returns a kpt_status (0 = KPT_OK); on error
 * kpt_last_error() returns a message for the calling thread.  Matrices are
 * 16 floats, column-major (the reference's Mat4 / glm layout).  Host arrays
 * passed in are copied; the library owns all device memory of a context.
 * Functions whose name ends in _device take device pointers and enqueue work
 * on the context's stream without synchronising.  A context belongs to one
 * host thread at a time.
 */
#ifndef KPT_H
#define KPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int kpt_status;
enum {
    KPT_OK = 0,
    KPT_ERR_INVALID = -1,     /* bad argument or index out of range */
    KPT_ERR_CUDA = -2,        /* a CUDA call failed; see kpt_last_error() */
    KPT_ERR_STATE = -3,       /* call not valid in the current state (e.g. no scene) */
    KPT_ERR_NOMEM = -4,       /* device allocation failed */
    KPT_ERR_TRAVERSAL = -5    /* a ray exceeded the traversal stack (result incomplete) */
};

typedef struct kpt_context kpt_context;

/* MaterialSceneEntity (pod_types.hpp:60-123) / Material (shaders/material.cuh:91-145). */
typedef struct kpt_material {
    float albedo[3];
    float metallic, roughness, transmission, ior;
    float emission[3];
    float emission_scale;      /* nits */
    float normal_scale;
    int32_t albedo_tex, orm_tex, transmission_tex, emission_tex, normal_tex;  /* -1: none */
    int32_t pad;
} kpt_material;

/* ProceduralEnvironmentSettings (pod_types.hpp:37-44) plus the Nishita
 * coefficients that the reference hard-codes (shaders/atmosphere.cuh:292-310);
 * kpt_environment_default() fills the reference values. */
typedef struct kpt_environment {
    float sun_angular_diameter, sun_phi, sun_theta, sun_emission_factor;
    float rayleigh[3];         /* sea-level Rayleigh scattering, 1/m */
    float mie;                 /* sea-level Mie scattering, 1/m */
    float mie_absorption;      /* sea-level Mie absorption, 1/m */
    float rayleigh_height, mie_height;   /* scale heights, m */
    float pad;
} kpt_environment;

/* RendererSettings (pod_types.hpp:46-57).
 * temporal_accumulation: the reference's integrator_use_temporal_accumulation
 * (kernels.cu:164-327, :422-428): every sample is one reference frame; its
 * radiance is blended into the previous frame's image reprojected along the
 * visible surface's motion (camera and instance transforms), with depth
 * rejection and a history of at most 16 frames, instead of the running mean.
 * In this mode setting the view or an instance transform keeps the history
 * (other setters clear it, as in the reference).  The first camera a context
 * receives is its own previous camera.
 * postprocess_effects: the reference's lens effects on the display image
 * (computeEffects, kernels.cu:340-374, 506-527): fisheye (power 1.65) and
 * chromatic aberration.
 * upscale: the reference's upscale_enable.  0 off; 1 and 2: the paths,
 * accumulation, modulation and histogram run at the output resolution / 2.5
 * (truncated), the render is upscaled to the output resolution, and bloom,
 * tonemapping and effects run there.  1 upscales bilinearly as the reference
 * builds it (upscale.cuh:260-291); 2 runs the FSR 1.0 path the reference
 * compiles with USE_FSR (kernels.cuh:3, kernels.cu:84-104): EASU
 * (upscale.cuh:13-258) then RCAS sharpening (upscale.cuh:300-433).  The render resolution follows the switch at once (the
 * reference waits for its next resizeResolution); kpt_get_render_size
 * gives it. */
typedef struct kpt_settings {
    int32_t max_depth;
    int32_t bloom, karis, auto_exposure;
    float bloom_final_blend, bloom_internal_blend;
    float frame_delta_ms;
    int32_t rng_order;         /* argument evaluation order of the reference's three calls that draw
                                  two random values in one expression, a set bit meaning right to
                                  left: 1 = make_float2(get1D(), get1D()) (samplers.cuh:37-40),
                                  2 = the sun-disc offset (integrator.cuh:155), 4 = the BSDF
                                  sample's two pairs (integrator.cuh:382); the reference's GPU
                                  build: 0 (the default), its host build: 7 */
    int32_t temporal_accumulation;
    int32_t postprocess_effects;
    int32_t upscale;
    int32_t sky_arith;         /* arithmetic of the Nishita sky and the sun's constants: 1 (the
                                  default) that of the reference's GPU build -- fast square root,
                                  division and exponentials, contracted products, fast sine, cosine
                                  and tangent for the sun -- so that sky values agree with its
                                  megakernel's; 0 IEEE single precision, as its host build computes
                                  them.  The sky's altitudes are lengths of ~6.4e6 m vectors (0.5 m
                                  per ulp against a 1200 m Mie scale height), so the two differ by
                                  up to ~1e-2 relative in places.  The path-replay adjoint always
                                  uses IEEE. */
    int32_t temporal_arith;    /* arithmetic of the temporal reprojection (temporal_accumulation =
                                  1): 1 (the default) that of the reference's GPU build, which
                                  inverts the camera and previous model matrices for every pixel
                                  with contracted products and an approximate reciprocal, and
                                  whose visible-surface position and depth come from its
                                  fast-maths camera ray and triangle test (a still camera then
                                  has a velocity of a few ulps, and the truncated previous pixel
                                  and the bilinear weights follow them); 0 IEEE single precision
                                  with the matrices inverted once on the host. */
} kpt_settings;

/* ExposureValues (pod_types.hpp:9-33) with the compensation and white/black
 * points passed to Renderer::setExposure (renderer.cu:312-329). */
typedef struct kpt_exposure {
    float aperture, iso, shutter, ev_comp, white_ev, black_ev;
    float max_iso, min_iso, max_shutter, min_shutter;
    float pad0, pad1;
} kpt_exposure;

/* Traversal counters (cumulative since kpt_create, counted in-kernel): every
 * query, then the path stage's extension rays (closest hit) and shadow rays
 * (any hit); and the state of the last exposure update. */
typedef struct kpt_stats {
    uint64_t box_tests, tri_tests, inst_xforms, overflows;
    uint64_t path_box_tests, path_tri_tests, path_inst_xforms;
    uint64_t shadow_box_tests, shadow_tri_tests, shadow_inst_xforms;
    uint64_t path_rays, shadow_rays, camera_rays;   /* rays traced by the path stage */
    float avg_luminance, adapted_luminance, exposure_scalar, iso, shutter, avg_bin;
    int32_t frame_index, pad;
} kpt_stats;

const char* kpt_last_error(void);
void kpt_environment_default(kpt_environment* env);
void kpt_settings_default(kpt_settings* s);
void kpt_exposure_default(kpt_exposure* e);

/* Renderer::initialize / shutdown (renderer.cu:22-53). */
kpt_status kpt_create(int device, kpt_context** out);
kpt_status kpt_destroy(kpt_context* ctx);

/* Renderer::resizeResolution (renderer.cu:55-101): render size; clears the accumulation. */
kpt_status kpt_resize(kpt_context* ctx, int width, int height);
/* The render resolution (the output's unless upscaling); kpt_read_render,
 * kpt_read_accumulation and kpt_read_albedo have this size, kpt_read_image
 * the output's. */
kpt_status kpt_get_render_size(kpt_context* ctx, int* width, int* height);

/* Scene upload, Renderer::loadScene (renderer.cu:356-436).  A mesh is a
 * triangle list (positions and normals 9 floats per triangle, uvs 6, one
 * material id per triangle); its BLAS is built on upload.  An instance places
 * a mesh with a model matrix and an optional material override (-1: the
 * mesh's ids); the reference has no instancing and copies one mesh per
 * instance, which gives the same images.  kpt_commit_scene builds the TLAS
 * and the light list and uploads everything. */
kpt_status kpt_set_materials(kpt_context* ctx, int n, const kpt_material* materials);
kpt_status kpt_set_textures(kpt_context* ctx, int n, const int32_t* desc /* n x (w, h, channels, byte offset) */,
                            size_t nbytes, const uint8_t* pixels);
kpt_status kpt_upload_mesh(kpt_context* ctx, int ntris, const float* positions, const float* normals,
                           const float* uvs, const int32_t* material_ids, int* mesh_out);
kpt_status kpt_add_instance(kpt_context* ctx, int mesh, const float* model, int material_override, int* instance_out);
kpt_status kpt_commit_scene(kpt_context* ctx);
kpt_status kpt_clear_scene(kpt_context* ctx);

/* New vertex positions (and optionally normals, 9 floats per triangle each,
 * the mesh's triangle order) for a mesh of the committed scene, keeping its
 * tree: the BLAS child boxes are refit on the GPU bottom up (each box the
 * bounds of the triangles under it, as a build of the same tree would give),
 * the triangle, shading and light records updated and the TLAS rebuilt on
 * the next frame.  The reference's refitBLAS (as_builder.cuh:263-286) is
 * not used by its renderer; a tree refit over large deformations traverses
 * slower than a rebuild but returns the same hits.  Clears the accumulation
 * (keeps the history in temporal mode, like a transform change). */
kpt_status kpt_refit_mesh(kpt_context* ctx, int mesh, const float* positions, const float* normals);

/* Where kpt_upload_mesh builds a BLAS.  No counterpart in the reference,
 * which builds every BLAS on the host (BLASBuilder, as_builder.cuh:181-261).
 * device = 1: on the GPU, on the context's stream -- the reference's tree
 * exactly (the same splits, child boxes and triangle order in every leaf);
 * 0 (the default): on the host. */
kpt_status kpt_set_blas_build(kpt_context* ctx, int device);

/* The BLAS of an uploaded mesh in the device format.  info[5] = interior
 * nodes, root node (-1: the root is a leaf), the root leaf's first triangle
 * and count, the mesh's triangles; nodes[16 per interior node] = both children's boxes (lo xyz, hi
 * xyz, 12 floats) then four int32 bit patterns (child 1 reference, child 1
 * triangle count, child 2 reference, count; a count of 0 marks an interior
 * child, whose reference is its node index, else the reference is the first
 * triangle in leaf order), depth-first with the left child first;
 * order[ntris] = the mesh triangle at each leaf-order position; bounds[6] =
 * the mesh's box.  Any output but info may be null. */
kpt_status kpt_get_blas(kpt_context* ctx, int mesh, int32_t* info, float* nodes, int32_t* order, float* bounds);

/* getMaterialsCount / getMeshCount (renderer.cu:280-288); the reference's
 * meshes are this library's instances. */
kpt_status kpt_counts(kpt_context* ctx, int* materials, int* meshes, int* instances, int* lights);

/* Renderer::setMaterial / getMaterial (renderer.cu:207-248): KPT_ERR_INVALID
 * for an index out of range (the reference returns false / asserts). */
kpt_status kpt_set_material(kpt_context* ctx, int index, const kpt_material* m);
kpt_status kpt_get_material(kpt_context* ctx, int index, kpt_material* m);

/* Renderer::setMeshTransform / getMeshTransform (renderer.cu:250-278): the
 * TLAS is rebuilt before the next frame. */
kpt_status kpt_set_instance_transform(kpt_context* ctx, int index, const float* model);
kpt_status kpt_get_instance_transform(kpt_context* ctx, int index, float* model);

/* Renderer::setView (renderer.cu:342-354) takes projection and view and
 * inverts them; kpt_set_camera_inverse takes the inverses directly
 * (Camera::setView, shaders/camera.cuh:28-36). */
kpt_status kpt_set_view(kpt_context* ctx, const float* projection, const float* view);
kpt_status kpt_set_camera_inverse(kpt_context* ctx, const float* inv_projection, const float* inv_view);

/* setProceduralEnvironmentData / setRendererSettings / setExposure and their
 * getters (renderer.cu:290-334). */
kpt_status kpt_set_environment(kpt_context* ctx, const kpt_environment* env);
kpt_status kpt_get_environment(kpt_context* ctx, kpt_environment* env);
kpt_status kpt_set_settings(kpt_context* ctx, const kpt_settings* s);
kpt_status kpt_get_settings(kpt_context* ctx, kpt_settings* s);
kpt_status kpt_set_exposure(kpt_context* ctx, const kpt_exposure* e);
kpt_status kpt_get_exposure(kpt_context* ctx, kpt_exposure* e);

/* Renderer::resetAccumulation (renderer.cu:336-340). */
kpt_status kpt_reset_accumulation(kpt_context* ctx);

/* Renderer::executeRendering (renderer.cu:103-195) for `spp` samples per
 * pixel in one frame: the samples use the reference's frame indices
 * frame_index .. frame_index+spp-1 and are added to the accumulation in that
 * order; then the post chain (modulate, histogram + exposure, bloom, AgX)
 * runs on the device, all captured in one CUDA graph.  Asynchronous. */
kpt_status kpt_render_frame(kpt_context* ctx, int spp, float delta_ms);
kpt_status kpt_synchronize(kpt_context* ctx);

/* Headless replacements for getRenderTargetTexture (renderer.cu:197-200):
 * the display image (AgX, [H][W] RGBA float), the modulated render, the
 * accumulation sum and the visible-surface albedo.  Synchronous copies to
 * host memory. */
kpt_status kpt_read_image(kpt_context* ctx, float* rgba);
kpt_status kpt_read_render(kpt_context* ctx, float* rgba);
kpt_status kpt_read_accumulation(kpt_context* ctx, float* rgba);
kpt_status kpt_read_albedo(kpt_context* ctx, float* rgba);
/* With temporal accumulation: the blended history the reference keeps in its
 * accumulation texture (rgb, and the history length in alpha), [H][W]; no
 * frame rendered with temporal accumulation: KPT_ERR_STATE. */
kpt_status kpt_read_history(kpt_context* ctx, float* rgba);
kpt_status kpt_read_histogram(kpt_context* ctx, uint64_t* bins256);
kpt_status kpt_get_stats(kpt_context* ctx, kpt_stats* st);
/* Diagnostics, no reference counterpart: for each level 0 .. min(max_levels,
 * max_depth + 1) - 1 of the last wave of the last frame rendered (or adjoint
 * replayed) on this context, counts[3 l] = paths shaded at level l (level
 * >= 1: extension rays
 * traced into it), counts[3 l + 1] = sun shadow rays and counts[3 l + 2] =
 * area-light shadow rays it sent; *levels = the number of levels written.  A
 * frame has one wave unless width x height x spp exceeds the wave capacity
 * (kpt_tuning.wave_cap).  After kpt_submit_batch, call kpt_wait_batch first. */
kpt_status kpt_get_level_counts(kpt_context* ctx, int max_levels, int32_t* counts, int32_t* levels);

/* Per-sample radiance of the plain method (the megakernel body,
 * shaders/kernels.cu:385-413), for parity checks: samples sample0 ..
 * sample0+n-1 of every pixel, [n][H][W] float4 (rgb, 0) into device memory,
 * plus (instance, triangle, t bits, 0) of the first hit per pixel.  Does not
 * touch the accumulation. */
kpt_status kpt_render_samples_device(kpt_context* ctx, int sample0, int nsamples, float* radiance,
                                     int32_t* first_hit, float* albedo);

/* Closest hit (TLAS::intersect, shaders/tlas.cu:60-125) and any hit
 * (TLAS::intersectP, tlas.cu:8-58) for n rays; origins and directions are
 * 3 floats per ray.  Device pointers. */
kpt_status kpt_trace_device(kpt_context* ctx, int n, const float* origins, const float* dirs, float tmin,
                            float tmax, int32_t* instance, int32_t* triangle, float* t, float* uv);
kpt_status kpt_occluded_device(kpt_context* ctx, int n, const float* origins, const float* dirs, float tmin,
                               const float* tmax, uint8_t* occluded);
/* Closest hit plus nbounces diffuse bounces per ray (the traversal
 * workload); outputs are (nbounces+1) x n. */
kpt_status kpt_trace_bounces_device(kpt_context* ctx, int n, const float* origins, const float* dirs, int nbounces,
                                    int32_t* instance, int32_t* triangle, float* t);
/* Host-memory variant of kpt_trace_bounces_device (copies in and out). */
kpt_status kpt_trace_bounces(kpt_context* ctx, int n, const float* origins, const float* dirs, int nbounces,
                             int32_t* instance, int32_t* triangle, float* t);

/* kpt_trace_bounces for callers that must not allocate device memory.  No
 * counterpart in the reference.  Some callers cannot call cudaMalloc: a frame
 * loop that must never stall (cudaMalloc and cudaFree can synchronise the
 * whole device), or an application that reserves a fixed device-memory budget
 * up front and forbids later growth.  This call allocates nothing: rays and
 * hits are staged through one fixed array of KPT_NOALLOC_STAGING_BYTES inside
 * the library, which every GPU that loads libkpt.so holds until the process
 * exits; n * (24 + 12 * (nbounces + 1)) must fit in it, larger requests fail
 * with KPT_ERR_INVALID.  The first call on a device looks the array up on
 * that device, so make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU (two threads, or two contexts of one
 * device at once) race; a call returns once its hits are in host memory.
 * Needs a committed scene with no pending transform change (KPT_ERR_STATE
 * otherwise).  Returns what kpt_trace_bounces returns. */
#define KPT_NOALLOC_STAGING_BYTES (8u << 20)
kpt_status kpt_trace_bounces_noalloc(kpt_context* ctx, int n, const float* origins, const float* dirs, int nbounces,
                                     int32_t* instance, int32_t* triangle, float* t);

/* Nishita sky radiance seen from 1 m above the ground for n directions
 * (NishitaAtmosphereModel::sampleLi, shaders/atmosphere.cuh:132-223). */
kpt_status kpt_sky_device(kpt_context* ctx, int n, const float* dirs, float* rgb);

/* Device timing of the frame's stages inside the frame graph (event-record
 * nodes between its launches).  kpt_stage_ms sums, per stage, the time of
 * the last n frames rendered with timing on (n <= 32) into
 * ms[KPT_STAGE_COUNT]; kpt_path_kernel_ms sums the path wave (shade, shadow
 * and extension kernels).  Both synchronise the stream. */
enum {
    KPT_STAGE_CAMERA = 0,     /* sky constants, camera rays, their sky */
    KPT_STAGE_SHADE = 1,      /* path vertices: emission, light sample, BSDF sample */
    KPT_STAGE_SHADOW = 2,     /* shadow rays (any hit) */
    KPT_STAGE_EXTEND = 3,     /* extension rays (closest hit) */
    KPT_STAGE_SKY = 4,        /* sky of the paths that left the scene */
    KPT_STAGE_ACCUMULATE = 5, /* clamped samples added in sample order */
    KPT_STAGE_POST = 6,       /* resolve, histogram, exposure, bloom, tonemap */
    KPT_STAGE_COUNT = 7
};
kpt_status kpt_enable_timing(kpt_context* ctx, int enable);
kpt_status kpt_stage_ms(kpt_context* ctx, int nframes, float* ms);
kpt_status kpt_path_kernel_ms(kpt_context* ctx, int nframes, float* total_ms);

/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order work around the library's launches. */
kpt_status kpt_get_stream(kpt_context* ctx, void** stream);

/* Kernel-launch counter of the context (every kernel the library enqueues). */
kpt_status kpt_launch_count(kpt_context* ctx, uint64_t* launches);

/* ---- Batched requests.  No counterpart in the reference, which renders one
 * frame of one scene per Renderer::executeRendering call (renderer.cu:103-195)
 * and synchronises after every launch. ---- */

/* Launch parameters of a context's path stage.  grid_scale: fraction of the
 * persistent grid (resident blocks x SMs) its wave kernels launch with, so
 * that jobs of one batch share the SMs; wave_cap: paths advanced together per
 * wave (queue capacity), 0 = 2^25; shade_block: threads per block of the
 * shading kernel (64, 128 or 256, 0 = 256); sort_rays: 1 groups each level's
 * extension rays by direction octant before they are traced, 0 keeps them in
 * pixel order (results are the same either way); fetch_batch: in the ray
 * kernels, the lanes of a warp whose rays are done wait until this many are
 * (or the whole warp is) and then store their results and fetch their next
 * rays together (1 .. 32, 0 = 7; results are the same for every value);
 * group_lobes: the shading kernel regroups windows of this many of a
 * level's paths by the lobe family of their hit (opaque, conductor,
 * transparent, mixed, none) before shading them, levels >= 1 (a multiple of
 * 64 in [64, 2048], rounded down to a multiple of the shading block and at
 * least one block; -1 off; 0 = 2048; results are the same either way). */
typedef struct kpt_tuning {
    float grid_scale;
    int32_t wave_cap;
    int32_t shade_block;
    int32_t sort_rays;
    int32_t fetch_batch;
    int32_t group_lobes;
} kpt_tuning;
void kpt_tuning_default(kpt_tuning* t);
kpt_status kpt_set_tuning(kpt_context* ctx, const kpt_tuning* t);
kpt_status kpt_get_tuning(kpt_context* ctx, kpt_tuning* t);

/* A batch renders one frame (spp samples, then the post chain) of each of n
 * jobs -- contexts of the batch's device, each with its own scene, camera,
 * resolution and settings, none twice -- as one CUDA graph on the batch's
 * stream.  Shared queues (the default, kpt_batch_set_shared(b, 1)): when
 * every job's frame is one wave (W*H*spp <= its wave_cap) without the octant
 * sort, each level's extension rays and shadow rays of all jobs are traced by
 * one persistent launch each, from one queue spanning the jobs, in a merged
 * copy of the jobs' scenes (rebuilt only when a job or its scene changes);
 * the jobs' camera rays, shading, sky and post chains run concurrently on
 * their own streams and `lanes` is not used.  Otherwise (or with
 * kpt_batch_set_shared(b, 0)) each job's frame is a branch of the graph:
 * `lanes` chains of jobs run concurrently (jobs are dealt to the lanes
 * longest first by W*H*spp*max_depth; lanes <= 0 or >= n: one lane per
 * job).  Either way every job's frame is the one it renders alone, bit for
 * bit.  kpt_submit_batch returns after the launch; kpt_wait_batch waits and
 * returns each job's device latency from the start of the batch to the end
 * of its frame (job_ms[n], may be null) and the batch's device time. */
typedef struct kpt_batch kpt_batch;
kpt_status kpt_batch_create(int device, kpt_batch** out);
kpt_status kpt_batch_destroy(kpt_batch* b);
kpt_status kpt_batch_set_shared(kpt_batch* b, int shared);   /* 1 (default) or 0; not while a batch is pending */
kpt_status kpt_batch_get_shared(kpt_batch* b, int* shared);
kpt_status kpt_submit_batch(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp, int lanes);
kpt_status kpt_wait_batch(kpt_batch* b, float* job_ms, float* total_ms);

/* The batch autotuner: renders the batch under each candidate (grid_scale,
 * wave_cap, shade_block, lanes) -- one untimed and `reps` timed submissions
 * each -- keeps the fastest total device time, applies its tuning to every
 * job and returns it with its lane count and time.  The result is cached per
 * batch signature (the jobs' sizes, spp and depths): a second call with the
 * same signature applies the cached choice without rendering.  Frames
 * rendered while tuning are discarded: every job's accumulation is reset. */
kpt_status kpt_autotune_batch(kpt_batch* b, int n, kpt_context* const* jobs, const int32_t* spp, int reps,
                              kpt_tuning* best, int32_t* best_lanes, float* best_ms);

/* ---- Path-replay adjoint.  No counterpart in the reference. ----
 *
 * The differentiated image is, per pixel, the mean over the samples sample0 ..
 * sample0+nsamples-1 of the clamped path radiance (the quantity the
 * accumulation receives per frame, before modulation and the post chain).
 * Given adjoint = dLoss/dimage ([H][W] RGBA float, alpha ignored), the adjoint
 * replays every sample's path from its random-number stream and returns
 * dLoss/dtheta for theta = per material m (albedo r, g, b, roughness) in
 * material order, then the sky (Rayleigh r, g, b, Mie, Rayleigh scale height,
 * Mie scale height): kpt_adjoint_param_count() values.  Sampled directions,
 * lobe, light and sun choices, Russian roulette, pdfs and MIS weights are held
 * fixed (detached sampling): the gradient is that of the estimator with
 * respect to the BSDF values and the sky radiance.  image (may be null)
 * receives the image itself.  Requires max_depth <= 16.
 * kpt_adjoint_device takes device pointers (grad: doubles) and does not
 * synchronise; kpt_adjoint takes host arrays.  The replay runs in waves whose
 * per-vertex records take at most 12 GiB of device memory, plus two sky
 * queues of 32 B per pixel and sample; the context keeps these buffers for
 * the next call until kpt_destroy. */
kpt_status kpt_adjoint_param_count(kpt_context* ctx, int* n);
kpt_status kpt_adjoint_device(kpt_context* ctx, int sample0, int nsamples, const float* adjoint, double* grad,
                              float* image);
kpt_status kpt_adjoint(kpt_context* ctx, int sample0, int nsamples, const float* adjoint, double* grad, float* image);
/* The same adjoint in two calls, for a caller whose loss needs the image
 * first (an optimisation step): kpt_adjoint_forward_device replays the
 * samples once, keeps every path's records and writes the image the
 * gradient belongs to (image, device, [H][W] RGBA float); after the caller
 * has formed dLoss/dimage, kpt_adjoint_backward_device sweeps the kept
 * records -- no ray is traced twice -- and writes the gradient (device
 * doubles).  Both enqueue on the context's stream and do not synchronise.
 * The records of all W*H*nsamples samples must fit one replay wave (12 GiB,
 * and at most 2^25 samples): otherwise KPT_ERR_INVALID (kpt_adjoint_device
 * has no such limit).  The backward call needs the forward call's records
 * and state: after any frame, adjoint call, scene, material, environment,
 * settings, camera or resolution change in between it returns
 * KPT_ERR_STATE; each forward call allows one backward call. */
kpt_status kpt_adjoint_forward_device(kpt_context* ctx, int sample0, int nsamples, float* image);
kpt_status kpt_adjoint_backward_device(kpt_context* ctx, const float* adjoint, double* grad);

/* Test support for the adjoint's FP64 oracle: as kpt_adjoint_device, and
 * also writes every path vertex the replay visited -- all its fixed quantities
 * (local directions, pdfs, roulette factors, light-sample factors, emission,
 * the sample's adjoint weight, the escape direction) -- as 192-byte records
 * (kpt_adjoint_record_size) to records (device), at most max_records; *count
 * (host) receives the number of vertices visited.  Synchronises. */
int kpt_adjoint_record_size(void);
/* The sky radiance (as kpt_sky_device) and its derivatives with respect to
 * the six sky parameters above, for n directions (device): rgb[7 i] is the
 * radiance, rgb[7 i + 1 + k] its derivative for parameter k (3 floats each). */
kpt_status kpt_sky_grad_device(kpt_context* ctx, int n, const float* dirs, float* rgb);
kpt_status kpt_adjoint_records_device(kpt_context* ctx, int sample0, int nsamples, const float* adjoint, double* grad,
                                      void* records, int max_records, int* count);

#ifdef __cplusplus
}
#endif
#endif /* KPT_H */
