// ref_harness.cpp -- drives the reference's own path-tracing code on the
// host CPU, to pin the oracle (oracle/kpt_oracle.cpp) against it.
//
// TEST INFRASTRUCTURE ONLY.  This is our driver; the code it runs is the
// reference's, compiled unmodified from its source tree by
// oracle/build_ref.sh into oracle/_ref/ (never committed).  Each entry point
// mirrors a reference host routine or kernel body and says which; the C ABI
// matches the oracle's so that tests/golden/make_golden.py can call both the
// same way.  The reference has no tests and no golden vectors of its own, so
// the fixtures under tests/golden/ are generated from this harness compiled
// with the reference's sources.
//
// The scene set-up replays Renderer::loadScene (renderer.cu:356-436) followed
// by Renderer::setMeshTransform (renderer.cu:250-269) for every mesh, with one
// difference: the mesh inverse is the reference's own Mat4::inverse of the
// model matrix rather than glm::inverse, so that the oracle and this harness
// share one inverse routine.

#include "shaders/tlas.cu"
#include "shaders/interaction.cu"
#include "shaders/light.cu"
#include "shaders/material.cu"
#include "shaders/texture.cu"
#include "shaders/histogram.cu"
#include "shaders/bloom.cu"
#include "shaders/upscale.cuh"
#include "shaders/integrator.cuh"
#include "shaders/film.cuh"
#include "shaders/filter.cuh"
#include "shaders/packing.cuh"
#include "as_builder.cuh"
#include "autoexposure_program.hpp"
#include "pod_types.hpp"
#include "ref_records.h"
#include "ref_scene.h"

#include <algorithm>
#include <cstdio>
#include <thread>
#include <atomic>

using namespace KittlesPT;

namespace {

void bind_views(RefScene& r) {  // RendererResource::updateResource (renderer_resource.cuh:28-40)
    ShaderData& sd = r.sd;
    sd.tlas_nodes_buffer = Buffer<TLASNode>(thrust::raw_pointer_cast(r.tlasnodes.data()), r.tlasnodes.size());
    sd.blas_buffer = Buffer<BLAS2>(thrust::raw_pointer_cast(r.blas.data()), r.blas.size());
    sd.bvh_nodes_buffer = Buffer<BVH2Node>(thrust::raw_pointer_cast(r.nodes.data()), r.nodes.size());
    sd.triangle_index_buffer = Buffer<int32_t>(thrust::raw_pointer_cast(r.tri_index.data()), r.tri_index.size());
    sd.meshes_buffer = Buffer<TriangleMesh>(thrust::raw_pointer_cast(r.meshes.data()), r.meshes.size());
    sd.lights_buffer = Buffer<Light>(thrust::raw_pointer_cast(r.lights.data()), r.lights.size());
    sd.triangles_buffer = Buffer<Triangle>(thrust::raw_pointer_cast(r.tris.data()), r.tris.size());
    sd.materials_buffer = Buffer<Material>(thrust::raw_pointer_cast(r.materials.data()), r.materials.size());
    sd.texture_buffer = Buffer<Texture>(thrust::raw_pointer_cast(r.textures.data()), r.textures.size());
    sd.pixel_buffer = Buffer<uint8_t>(thrust::raw_pointer_cast(r.pixels.data()), r.pixels.size());
}

template <class Fn>
void parallel_rows(int n, int nthreads, Fn fn) {
    if (nthreads <= 1 || n < 2) { for (int i = 0; i < n; ++i) fn(i); return; }
    nthreads = std::min(nthreads, n);
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&] { for (int i; (i = next.fetch_add(1)) < n;) fn(i); });
    for (auto& t : th) t.join();
}

}  // namespace

extern "C" {

void* ref_scene_create(int ntris, const float* pos, const float* nrm, const float* uv, const int* mat,
                       int nmeshes, const int* mesh_off, const int* mesh_cnt, const float* models,
                       int nmaterials, const void* materials,
                       int ntextures, const int* tex_desc, long long npixels, const unsigned char* pixels) {
    RefScene* r = new RefScene();
    ref_replay_load_scene(r, ntris, pos, nrm, uv, mat, nmeshes, mesh_off, mesh_cnt, models, nmaterials, materials,
                          ntextures, tex_desc, npixels, pixels);
    bind_views(*r);
    return r;
}

void ref_scene_destroy(void* h) { delete (RefScene*)h; }

void ref_scene_counts(void* hp, long long* out) {
    RefScene& r = *(RefScene*)hp;
    out[0] = (long long)r.nodes.size();
    out[1] = (long long)r.tri_index.size();
    out[2] = (long long)r.tlasnodes.size();
    out[3] = (long long)r.lights.size();
    out[4] = (long long)r.meshes.size();
}

void ref_scene_bvh(void* hp, int* left_first, unsigned* count, float* bounds, int* tri_index,
                   long long* blas_root, float* blas_bounds, float* blas_inv) {
    RefScene& r = *(RefScene*)hp;
    for (size_t i = 0; i < r.nodes.size(); ++i) {
        const BVH2Node& n = r.nodes[i];
        left_first[i] = n.left_child_node_index_or_tris_index_start_index;
        count[i] = n.node_tris_index_count;
        float v[6] = {n.bounds.pmin.x, n.bounds.pmin.y, n.bounds.pmin.z, n.bounds.pmax.x, n.bounds.pmax.y, n.bounds.pmax.z};
        std::memcpy(bounds + 6 * i, v, sizeof v);
    }
    for (size_t i = 0; i < r.tri_index.size(); ++i) tri_index[i] = r.tri_index[i];
    for (size_t i = 0; i < r.blas.size(); ++i) {
        const BLAS2& b = r.blas[i];
        blas_root[i] = b.bvhnode_root_index;
        float v[6] = {b.bounds.pmin.x, b.bounds.pmin.y, b.bounds.pmin.z, b.bounds.pmax.x, b.bounds.pmax.y, b.bounds.pmax.z};
        std::memcpy(blas_bounds + 6 * i, v, sizeof v);
        std::memcpy(blas_inv + 16 * i, &b.inv_model_matrix, 64);
    }
}

void ref_scene_tlas(void* hp, unsigned* lr, int* blas, float* bounds) {
    RefScene& r = *(RefScene*)hp;
    for (size_t i = 0; i < r.tlasnodes.size(); ++i) {
        const TLASNode& n = r.tlasnodes[i];
        lr[i] = n.left_right_index;
        blas[i] = n.blas_index;
        float v[6] = {n.bounds.pmin.x, n.bounds.pmin.y, n.bounds.pmin.z, n.bounds.pmax.x, n.bounds.pmax.y, n.bounds.pmax.z};
        std::memcpy(bounds + 6 * i, v, sizeof v);
    }
}

// TLAS::intersect (tlas.cu:60-125); counters are not collected here.
void ref_trace(void* hp, int n, const float* o, const float* d, float tmin, float tmax,
               int* prim, int* inst, float* t, float* bary, int brute, long long* counters, int nthreads) {
    RefScene& r = *(RefScene*)hp;
    const int CH = 256;
    parallel_rows((n + CH - 1) / CH, nthreads, [&](int blk) {
        for (int i = blk * CH; i < std::min(n, (blk + 1) * CH); ++i) {
            Ray ray(make_float3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), make_float3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            DebugData dbg;
            Intersection h;
            if (!brute) {
                h = r.sd.top_level_acceleration_structure.intersect(r.sd, ray, tmin, tmax, dbg);
            } else {
                // the INTERSECT_DEBUG loop of Integrator::intersect (integrator.cuh:72-93)
                Intersection intr;
                for (int32_t mi = 0; mi < (int32_t)r.meshes.size(); ++mi) {
                    const TriangleMesh& mesh = r.meshes[mi];
                    Ray orr = ray.transform(r.blas[mesh.blas_index].inv_model_matrix);
                    for (int32_t p = mesh.prim_offset; p < mesh.prim_offset + (int32_t)mesh.prim_count; ++p) {
                        r.tris[p].intersect(orr, tmin, tmax, &intr);
                        if (intr.distance < INFINITY && intr.distance < tmax && intr.distance > tmin && intr.distance < h.distance) {
                            h = intr; h.primitive_id = p; h.instance_id = mi;
                        }
                    }
                }
            }
            prim[i] = h.primitive_id; inst[i] = h.instance_id; t[i] = h.distance;
            if (bary) { bary[3 * i] = h.bary_coords.x; bary[3 * i + 1] = h.bary_coords.y; bary[3 * i + 2] = h.bary_coords.z; }
        }
    });
    if (counters) for (int k = 0; k < 8; ++k) counters[k] = 0;
}

// Diffuse bounce chain of the traversal workload (the same rule as the
// oracle's orc_trace_bounces: Malley's method with a rejection-sampled disk
// point), built from the reference's own sampler, basis and traversal.
void ref_trace_bounces(void* hp, int n, const float* o, const float* d, int nbounces,
                       int* prim, float* t, long long* counters, int nthreads) {
    RefScene& r = *(RefScene*)hp;
    const int CH = 256;
    parallel_rows((n + CH - 1) / CH, nthreads, [&](int blk) {
        for (int i = blk * CH; i < std::min(n, (blk + 1) * CH); ++i) {
            Ray ray(make_float3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), make_float3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            for (int b = 0; b <= nbounces; ++b) {
                size_t k = (size_t)b * n + i;
                DebugData dbg;
                Intersection h = r.sd.top_level_acceleration_structure.intersect(r.sd, ray, 0.0f, INFINITY, dbg);
                prim[k] = h.primitive_id; t[k] = h.distance;
                if (h.primitive_id < 0) {
                    for (int bb = b + 1; bb <= nbounces; ++bb) { prim[(size_t)bb * n + i] = -1; t[(size_t)bb * n + i] = INFINITY; }
                    break;
                }
                if (b == nbounces) break;
                const Triangle& tr = r.tris[h.primitive_id];
                Mat4 model = r.meshes[h.instance_id].curr_inv_model_matrix.inverse();
                float3 nn = normalize(make_float3(model * make_float4(tr.local_geometric_normal, 0)));
                if (dot(nn, ray.getDirection()) > 0.0f) nn = -nn;
                float3 p = ray.getPointAt(h.distance);
                IndependentSampler S;
                S.setSeed((uint32_t)i * 4u + (uint32_t)b);
                float x = 0.0f, y = 0.0f, r2 = 0.0f;
                for (int q = 0; q < 64; ++q) {
                    float u0 = S.get1D();
                    float u1 = S.get1D();
                    float a = 2.0f * u0 - 1.0f, c = 2.0f * u1 - 1.0f;
                    float m = a * a + c * c;
                    if (m < 1.0f) { x = a; y = c; r2 = m; break; }
                }
                float3 l = make_float3(x, y, sqrtf(1.0f - r2));
                float3 w = generateONBFrisvad(nn) * l;
                ray = Ray(p + nn * Constants::HIT_EPSILON, w);
            }
        }
    });
    if (counters) for (int k = 0; k < 8; ++k) counters[k] = 0;
}

// The megakernel body (kernels.cu:385-413) for sample k = frame index
// sample0 + k; same outputs as orc_render_samples.  The reference fixes the
// Nishita coefficients, so only the sun parameters of `env` are used.
void ref_render_samples(void* hp, const float* inv_proj, const float* inv_view, const void* env,
                        const void* settings, int W, int H, int sample0, int nsamples, int rng_order,
                        int row0, int nrows, float* radiance, float* albedo, int* first_hit, float* first_t,
                        long long* counters, int nthreads) {
    RefScene& r = *(RefScene*)hp;
    const EnvRecord& e = *(const EnvRecord*)env;
    const SettingsRecord& st = *(const SettingsRecord*)settings;
    ShaderData sd = r.sd;
    sd.render_resolution = make_int2(W, H);
    sd.output_resolution = make_int2(W, H);
    sd.procedural_environment_data.sun_angular_diameter_rad = e.sun_angular_diameter;
    sd.procedural_environment_data.sun_phi_rad = e.sun_phi;
    sd.procedural_environment_data.sun_theta_rad = e.sun_theta;
    sd.procedural_environment_data.sun_emission_factor = e.sun_emission_factor;
    sd.renderer_settings.integrator_max_ray_depth = st.max_depth;
    Camera cam;
    cam.setView(mat_from(inv_proj), mat_from(inv_view));
    sd.scene_camera = cam;
    if (nrows <= 0) nrows = H - row0;
    parallel_rows(nrows, nthreads, [&](int ry) {
        int y = row0 + ry;
        for (int x = 0; x < W; ++x) {
            for (int k = 0; k < nsamples; ++k) {
                int2 pixel = make_int2(x, y);
                IndependentSampler sampler;
                sampler.initPixelSeed(pixel, W, sample0 + k);
                BoxFilter filter({1.0f, 1.0f});
                FilterSample fs = filter.sample(sampler.get2D());
                float2 uv = (make_float2(pixel) + 0.5f) / make_int2(W, H);
                float2 ndc = 2.0f * uv - 1.0f;
                DebugData dbg;
                VisibleSurface vs;
                Ray primary = sd.scene_camera.generateRay(ndc);
                RGBSpectrum L = RGBSpectrum(fs.weight) * 1.0f * Integrator::Li(sd, primary, sampler, &vs, &dbg);
                L = L.clampOutput();
                if (radiance) {
                    size_t o = (((size_t)k * nrows + ry) * W + x) * 3;
                    radiance[o] = L.r; radiance[o + 1] = L.g; radiance[o + 2] = L.b;
                }
                if (k == nsamples - 1) {
                    size_t p = (size_t)ry * W + x;
                    if (albedo) { albedo[3 * p] = vs.albedo.x; albedo[3 * p + 1] = vs.albedo.y; albedo[3 * p + 2] = vs.albedo.z; }
                    if (first_hit) { first_hit[2 * p] = vs.primitive_id; first_hit[2 * p + 1] = vs.instance_id; }
                    if (first_t) first_t[p] = vs.depth;
                }
            }
        }
    });
    if (counters) for (int k = 0; k < 8; ++k) counters[k] = 0;
    (void)rng_order;
}

// NishitaAtmosphereModel::sampleLi from 1 m above the ground.
void ref_sky(const void* env, int n, const float* dirs, float* out) {
    const EnvRecord& e = *(const EnvRecord*)env;
    ShaderData sd;
    sd.procedural_environment_data.sun_phi_rad = e.sun_phi;
    sd.procedural_environment_data.sun_theta_rad = e.sun_theta;
    float3 sun = Integrator::getSunDirection(sd);
    Atmosphere::NishitaAtmosphereModel atm(sun, e.sun_emission_factor);
    float3 obs = make_float3(0, atm.getEarthRadiusMeters() + 1, 0);
    for (int i = 0; i < n; ++i) {
        RGBSpectrum L = atm.sampleLi(Ray(obs, make_float3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2])));
        out[3 * i] = L.r; out[3 * i + 1] = L.g; out[3 * i + 2] = L.b;
    }
}

// UnifiedBSDF f / pdf / sampleF (bsdf.cuh:166-268), same layout as orc_bsdf_eval.
void ref_bsdf_eval(int n, const float* params, const float* dirs, const float* u, float* out) {
    for (int i = 0; i < n; ++i) {
        const float* p = params + 12 * i;
        UnifiedBSDF b(generateONBFrisvad(make_float3(p[0], p[1], p[2])), RGBSpectrum(p[3], p[4], p[5]),
                      p[6], p[7], p[8], p[9], p[10] != 0.0f);
        if (p[11] != 0.0f) b.regularize();
        float3 wo = make_float3(dirs[6 * i], dirs[6 * i + 1], dirs[6 * i + 2]);
        float3 wi = make_float3(dirs[6 * i + 3], dirs[6 * i + 4], dirs[6 * i + 5]);
        RGBSpectrum fv = b.f(wo, wi);
        float pd = b.pdf(wo, wi);
        BSDFSample bs = b.sampleF(wo, make_float2(u[4 * i], u[4 * i + 1]), make_float2(u[4 * i + 2], u[4 * i + 3]));
        float* o = out + 12 * i;
        o[0] = fv.r; o[1] = fv.g; o[2] = fv.b; o[3] = pd;
        o[4] = bs.f.r; o[5] = bs.f.g; o[6] = bs.f.b;
        o[7] = bs.wi.x; o[8] = bs.wi.y; o[9] = bs.wi.z; o[10] = bs.pdf; o[11] = (float)bs.scatter;
    }
}

// luminanceToBin (histogram.cu:18-33) for a list of luminances.
void ref_lum_bins(int n, const float* Y, float black_ev, float white_ev, int* bins) {
    for (int i = 0; i < n; ++i) bins[i] = (int)luminanceToBin(Y[i], black_ev, 1.0f / (white_ev - black_ev));
}

// addSample + modulateSamples (integrator.cuh:406-415, kernels.cu:453-472):
// render = (sum / n) * 8-bit G-buffer albedo, alpha 1.
void ref_modulate(int W, int H, const float* acc_sum, int nsamples, const float* albedo, float* render_out) {
    for (size_t p = 0; p < (size_t)W * H; ++p) {
        RGBSpectrum est = RGBSpectrum(acc_sum[3 * p], acc_sum[3 * p + 1], acc_sum[3 * p + 2]) / float(nsamples);
        VisibleSurface vs;
        vs.albedo = make_float3(albedo[3 * p], albedo[3 * p + 1], albedo[3 * p + 2]);
        vs.normal = make_float3(0, 0, 1);
        vs.depth = 1.0f;
        GBuffer gb(vs);
        GBuffer un = GBuffer::unpackGBuffer(gb.packGBuffer());
        est *= RGBSpectrum(un.albedo);
        float4 f = make_float4(est.toFloat3(), 1);
        std::memcpy(render_out + 4 * p, &f, 16);
    }
}

// histogramComputeKernel (histogram.cu:55-90) run block by block, thread by
// thread, with float sums in that order; bins whose owning thread lies
// outside the image are not flushed, as in the kernel.
void ref_histogram(int W, int H, const float* render, float black_ev, float white_ev, float* hist) {
    for (int b = 0; b < 256; ++b) hist[b] = 0.0f;
    int gx = W / 16 + 1, gy = H / 16 + 1;
    std::vector<float> shared(256);
    for (int by = 0; by < gy; ++by)
        for (int bx = 0; bx < gx; ++bx) {
            std::fill(shared.begin(), shared.end(), 0.0f);
            for (int li = 0; li < 256; ++li) {
                int x = bx * 16 + (li & 15), y = by * 16 + (li >> 4);
                if (x >= W || y >= H) continue;
                const float* c = render + 4 * ((size_t)y * W + x);
                RGBSpectrum lin(c[0], c[1], c[2]);
                float dr = white_ev - black_ev;
                uint bin = luminanceToBin(lin.getLuminance(), black_ev, (1.0f / dr));
                float w = centerMeteringWeight(make_int2(W, H), make_int2(x, y), 0.4f);
                w = (bin > 0) ? w : 1;
                shared[bin] += w;
            }
            for (int li = 0; li < 256; ++li) {
                int x = bx * 16 + (li & 15), y = by * 16 + (li >> 4);
                if (x >= W || y >= H) continue;
                hist[li] += shared[li];
            }
        }
}

// histogramAverageLuminanceComputeKernel's float maths (histogram.cu:93-154)
// in tree-reduction order, then AutoExposureProgram::computeExposure
// (autoexposure_program.hpp:18-24) and the exposure scalar of
// Renderer::setExposure (renderer.cu:312-329).  out: avg bin, avg lum,
// adapted lum, exposure scalar, iso, shutter.
void ref_exposure(const float* hist, float aperture, float iso, float shutter, float ev_comp,
                  float white_ev, float black_ev, float min_iso, float max_iso, float min_shutter,
                  float max_shutter, float last_lum, float delta_ms, float* out) {
    float nw[256], nb[256];
    for (int i = 0; i < 256; ++i) { nw[i] = hist[i]; nb[i] = hist[i] * i; }
    for (unsigned cutoff = 128; cutoff > 0; cutoff >>= 1)
        for (unsigned i = 0; i < cutoff; ++i) { nb[i] += nb[i + cutoff]; nw[i] += nw[i + cutoff]; }
    float non_black = max(nw[0] - hist[0], 0.001);
    float avg_bin = nb[0] / non_black;
    float dr = white_ev - black_ev;
    float avg_lum = powf(2, (clamp((avg_bin - 1.0f) / float(Constants::HISTOGRAM_SIZE - 2), 0.0f, 1.0f) * dr) + black_ev);
    float adapted = lerp(last_lum, avg_lum, 1.0f - expf(-delta_ms * 0.5f));
    ExposureValues ev(aperture, (int32_t)iso, shutter, (int32_t)max_iso, (int32_t)min_iso, max_shutter, min_shutter);
    AutoExposureProgram ae;
    ae.recordValues(ev, ev_comp, white_ev, black_ev);
    ae.computeExposure(adapted);
    ExposureValues o = ae.getExposureValues();
    float scalar = AutoExposureProgram::getStandardOutputBasedExposure(o.aperture_f_num, o.shutter_speed_secs, o.ISO);
    float v[6] = {avg_bin, avg_lum, adapted, scalar, o.ISO, o.shutter_speed_secs};
    std::memcpy(out, v, sizeof v);
}

// Bloom: executeBloomGeneration (renderer.cu:438-475) over the mip chain of
// mipchain.cuh:17-36 (levels = min(log2 W, log2 H, 6)), running the
// downSample / upSampleCombine kernels of shaders/bloom.cu one thread at a
// time.  render/bloom_out: [H][W][4].
void ref_bloom(int W, int H, const float* render, int karis, float internal_blend, float* bloom_out) {
    int levels = std::min((int)std::log2(W), (int)std::log2(H));
    levels = std::min(levels, 6);
    std::vector<std::vector<float4>> mips(levels + 1);
    std::vector<DeviceTextureBuffer> dt(levels + 1);
    auto& surfs = host_surfaces();
    surfs.resize(1);
    for (int l = 0; l <= levels; ++l) {
        int w = W >> l, h = H >> l;
        mips[l].assign((size_t)w * h, make_float4(0, 0, 0, 0));
        if (l == 0) std::memcpy(mips[0].data(), render, sizeof(float4) * (size_t)w * h);
    }
    for (int l = 0; l <= levels; ++l) {
        surfs.push_back({mips[l].data(), W >> l, H >> l});
        dt[l].dimensions = make_int2(W >> l, H >> l);
        dt[l].m_surface_object = (cudaSurfaceObject_t)(surfs.size() - 1);
    }
    ShaderData sd;
    sd.renderer_settings.bloom_internal_blend = internal_blend;
    auto run = [&](int w, int h, auto kern) {
        blockDim = dim3(8, 8, 1);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                blockIdx = make_uint3(x / 8, y / 8, 0);
                threadIdx = make_uint3(x % 8, y % 8, 0);
                kern();
            }
    };
    for (int l = 0; l < levels; ++l)
        run(W >> (l + 1), H >> (l + 1), [&] { downSample(sd, dt[l], dt[l + 1], karis != 0 && l == 0); });
    for (int l = levels; l > 0; --l)
        run(W >> (l - 1), H >> (l - 1), [&] { upSampleCombine(sd, dt[l], dt[l - 1]); });
    std::memcpy(bloom_out, mips[0].data(), sizeof(float4) * (size_t)W * H);
    surfs.resize(1);
}

// computePostProcess body (kernels.cu:475-504) with the reference's Film.
void ref_post_image(int W, int H, const float* render, const float* bloom, int use_bloom, float final_blend,
                    float expo, float white_ev, float black_ev, float* image_out) {
    auto& surfs = host_surfaces();
    surfs.resize(1);
    std::vector<float4> r((size_t)W * H), b((size_t)W * H);
    std::memcpy(r.data(), render, sizeof(float4) * r.size());
    if (bloom) std::memcpy(b.data(), bloom, sizeof(float4) * b.size());
    surfs.push_back({r.data(), W, H});
    surfs.push_back({b.data(), W, H});
    ShaderData sd;
    sd.output_resolution = make_int2(W, H);
    sd.output_texture.dimensions = make_int2(W, H);
    sd.output_texture.m_surface_object = 1;
    sd.bloom_texture.dimensions = make_int2(W, H);
    sd.bloom_texture.m_surface_object = 2;
    sd.renderer_settings.bloom_generate_bloom = use_bloom != 0;
    sd.renderer_settings.bloom_final_blend = final_blend;
    sd.scene_camera.setExposure(expo, white_ev, black_ev);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float2 uv = (make_float2(make_int2(x, y)) + 0.5f) / make_int2(W, H);
            RGBSpectrum s = RGBSpectrum(sd.output_texture.textureReadNearestUV(uv));
            if (sd.renderer_settings.bloom_generate_bloom) {
                RGBSpectrum v = RGBSpectrum(sd.bloom_texture.textureReadNearestUV(uv));
                s = lerp(s, v, sd.renderer_settings.bloom_final_blend);
            }
            {
                float3 Yxy = s.toYxy();
                Yxy.x *= sd.scene_camera.getFilm().luminance_exposure_scalar;
                s = RGBSpectrum::fromYxy(Yxy);
            }
            float3 frag = sd.scene_camera.getFilm().computeNormalizedNonLinearSRGB(s);
            float4 f = make_float4(frag, 1.0f);
            std::memcpy(image_out + 4 * ((size_t)y * W + x), &f, 16);
        }
    surfs.resize(1);
}

// The upscale kernel (upscale.cuh:260-291) as the reference builds it
// (USE_FSR undefined, kernels.cuh:3): every output pixel reads the render
// bilinearly.  src: [sh][sw][4], dst: [dh][dw][4].
void ref_upscale(int sw, int sh, const float* src, int dw, int dh, float* dst) {
    auto& surfs = host_surfaces();
    surfs.resize(1);
    std::vector<float4> s((size_t)sw * sh), d((size_t)dw * dh, make_float4(0, 0, 0, 0));
    std::memcpy(s.data(), src, sizeof(float4) * s.size());
    surfs.push_back({s.data(), sw, sh});
    surfs.push_back({d.data(), dw, dh});
    DeviceTextureBuffer ts, td;
    ts.dimensions = make_int2(sw, sh);
    ts.m_surface_object = 1;
    td.dimensions = make_int2(dw, dh);
    td.m_surface_object = 2;
    blockDim = dim3(8, 8, 1);
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            blockIdx = make_uint3(x / 8, y / 8, 0);
            threadIdx = make_uint3(x % 8, y % 8, 0);
            upscale(ts, td);
        }
    std::memcpy(dst, d.data(), sizeof(float4) * d.size());
    surfs.resize(1);
}

// The reference's FSR 1.0 path, compiled out of its build by default
// (USE_FSR, kernels.cuh:3): launchUpscaleComputeKernel (kernels.cu:84-104)
// runs the upscale kernel's USE_FSR branch (upscale.cuh:271-283: FsrEasuCon +
// FsrEasuF of the render into the output) and then the sharpen kernel
// (upscale.cuh:415-433, RCAS of the output); renderer.cu:142-147 copies the
// sharpened image back into the output.  This driver runs that branch's body
// per output pixel with the reference's own FsrEasuCon/FsrEasuF, then the
// unmodified sharpen kernel one thread at a time.
void ref_fsr(int sw, int sh, const float* src, int dw, int dh, float* easu_out, float* dst) {
    auto& surfs = host_surfaces();
    surfs.resize(1);
    std::vector<float4> s((size_t)sw * sh), e((size_t)dw * dh, make_float4(0, 0, 0, 0)), d(e);
    std::memcpy(s.data(), src, sizeof(float4) * s.size());
    surfs.push_back({s.data(), sw, sh});
    surfs.push_back({e.data(), dw, dh});
    surfs.push_back({d.data(), dw, dh});
    DeviceTextureBuffer ts, te, td;
    ts.dimensions = make_int2(sw, sh);
    ts.m_surface_object = 1;
    te.dimensions = make_int2(dw, dh);
    te.m_surface_object = 2;
    td.dimensions = make_int2(dw, dh);
    td.m_surface_object = 3;
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            float3 c;
            float4 con0, con1, con2, con3;
            float2 rendersize = make_float2(ts.dimensions);
            FsrEasuCon(con0, con1, con2, con3, rendersize, rendersize, make_float2(te.dimensions));
            FsrEasuF(c, make_float2(make_int2(x, y)), con0, con1, con2, con3, ts);
            te.textureWrite(make_float4(c, 1), make_int2(x, y));
        }
    blockDim = dim3(8, 8, 1);
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            blockIdx = make_uint3(x / 8, y / 8, 0);
            threadIdx = make_uint3(x % 8, y % 8, 0);
            sharpen(te, td);
        }
    std::memcpy(easu_out, e.data(), sizeof(float4) * e.size());
    std::memcpy(dst, d.data(), sizeof(float4) * d.size());
    surfs.resize(1);
}

// centerMeteringWeight (histogram.cu:35-48) for every pixel.
void ref_metering_weights(int W, int H, float* out) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            out[(size_t)y * W + x] = centerMeteringWeight(make_int2(W, H), make_int2(x, y), 0.4f);
}

}  // extern "C"
