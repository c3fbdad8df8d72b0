// renderer.hpp -- C++ facade with the reference's KittlesPT::Renderer method
// set (KittlesPT/src/renderer.hpp:13-58) and scene types
// (KittlesPT/src/pod_types.hpp:7-212) over the C ABI of include/kpt.h, so
// that host code written against the reference's Renderer compiles against
// libkpt.so.  Header-only; link with -lkpt.
//
// Differences from the reference, all at the edges of the path:
//   * frame images are device buffers: getRenderTargetTexture(GLuint) becomes
//     getRenderTarget(float* rgba) (headless; no graphics API is involved);
//   * executeRendering(delta_ms) renders one sample per pixel as the
//     reference does; executeRendering(delta_ms, spp) renders spp in one frame;
//   * CUDA failures throw KittlesPT::Error instead of exit(99)
//     (error_check.cu:4-13); setters on a bad index return false as in the
//     reference, getters on a bad index throw instead of asserting;
//   * vector and matrix fields are glm types when <glm/glm.hpp> is available,
//     otherwise minimal structs with glm's memory layout (column-major
//     matrices indexed m[column][row]).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "../kpt.h"

#if defined(__has_include)
#if __has_include(<glm/glm.hpp>) && !defined(KPT_NO_GLM)
#include <glm/glm.hpp>
#define KPT_HAVE_GLM 1
#endif
#endif

namespace KittlesPT {

#ifdef KPT_HAVE_GLM
using Vec2 = glm::vec2;
using Vec3 = glm::vec3;
using Mat4 = glm::mat4;
#else
struct Vec2 { float x = 0.0f, y = 0.0f; };
struct Vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    Vec3() = default;
    Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit Vec3(float a) : x(a), y(a), z(a) {}
};
struct Mat4 {   // column-major, m[column][row], identity by default
    float m[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    float* operator[](int c) { return m[c]; }
    const float* operator[](int c) const { return m[c]; }
};
#endif

class Error : public std::runtime_error {
public:
    Error(kpt_status code, const std::string& msg) : std::runtime_error(msg), code(code) {}
    kpt_status code;
};

namespace detail {
inline void check(kpt_status s) {
    if (s != KPT_OK) throw Error(s, kpt_last_error());
}
template <class M>
inline std::array<float, 16> flat(const M& m) {   // column-major
    std::array<float, 16> a{};
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) a[4 * c + r] = m[c][r];
    return a;
}
inline Mat4 unflat(const float* a) {
    Mat4 m;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[c][r] = a[4 * c + r];
    return m;
}
}  // namespace detail

// pod_types.hpp:9-33
struct ExposureValues {
    ExposureValues() = default;
    ExposureValues(float aperture_f_num, int32_t iso, float shutter_secs, int32_t max_iso = 6400,
                   int32_t min_iso = 100, float max_shutter_secs = 0.0333f, float min_shutter_secs = 0.00025f)
        : aperture_f_num(aperture_f_num), ISO(static_cast<float>(iso)), shutter_speed_secs(shutter_secs),
          MAX_ISO(max_iso), MIN_ISO(min_iso), MIN_SHUTTER_SECS(min_shutter_secs), MAX_SHUTTER_SECS(max_shutter_secs) {}
    float aperture_f_num = 0.0f;
    float ISO = 0.0f;
    float shutter_speed_secs = 0.0f;
    int32_t MAX_ISO = 6400;
    int32_t MIN_ISO = 100;
    float MIN_SHUTTER_SECS = 0.00025f;
    float MAX_SHUTTER_SECS = 0.0333f;
};

// pod_types.hpp:37-44
struct ProceduralEnvironmentSettings {
    float sun_angular_diameter_rad = 0.0087f;
    float sun_phi_rad = 4.18879f;
    float sun_theta_rad = 17.0f * 3.14159265358979323846f / 180.0f;   // altitude
    float sun_emission_factor = 1.0f;
};

// pod_types.hpp:46-57
struct RendererSettings {
    int32_t integrator_max_ray_depth = 3;
    bool integrator_use_temporal_accumulation = false;
    bool bloom_generate_bloom = false;
    bool bloom_use_karis_average = false;
    float bloom_final_blend = 0.175f;
    float bloom_internal_blend = 0.65f;
    bool tonemapper_enable_auto_exposure = false;
    bool postprocess_enable_effects = false;
    bool upscale_enable = false;
    // the reference's build-time USE_FSR (kernels.cuh:3) as a setting: with
    // upscale_enable, FSR 1.0 (EASU + RCAS) instead of the bilinear upscale
    bool upscale_fsr = false;
};

// pod_types.hpp:60-123 (glTF 2.0 metallic-roughness material)
struct MaterialSceneEntity {
    MaterialSceneEntity() = default;
    MaterialSceneEntity(std::string_view name, int32_t albedo_texture_id, const Vec3& albedo, int32_t orm_texture_id,
                        float metallicity, float roughness, int32_t transmission_texture_id, float transmission,
                        float ior, int32_t emission_texture_id, const Vec3& emission_factor,
                        float emission_scale_nits, int32_t normal_texture_id, float normal_scale)
        : name(name), albedo_texture_id(albedo_texture_id), albedo_factor(albedo), ORM_texture_id(orm_texture_id),
          metallic_factor(metallicity), roughness_factor(roughness), transmission_texture_id(transmission_texture_id),
          transmission_factor(transmission), ior(ior), emission_texture_id(emission_texture_id),
          emission_factor(emission_factor), emission_scale_nits(emission_scale_nits),
          normal_texture_id(normal_texture_id), normal_scale(normal_scale) {}
    std::string name;
    int32_t albedo_texture_id = -1;
    Vec3 albedo_factor = Vec3(1.0f, 1.0f, 1.0f);
    int32_t ORM_texture_id = -1;
    float metallic_factor = 0.0f;
    float roughness_factor = 0.5f;
    int32_t transmission_texture_id = -1;
    float transmission_factor = 0.0f;
    float ior = 1.45f;
    int32_t emission_texture_id = -1;
    Vec3 emission_factor = Vec3(1.0f, 1.0f, 1.0f);
    float emission_scale_nits = 0.0f;
    int32_t normal_texture_id = -1;
    float normal_scale = 1.0f;
    bool isEmissive() const {
        return emission_factor.x * emission_scale_nits > 0.0f || emission_factor.y * emission_scale_nits > 0.0f ||
               emission_factor.z * emission_scale_nits > 0.0f;
    }
};

// pod_types.hpp:125-148
struct TriangleSceneEntity {
    TriangleSceneEntity(Vec3 p0, Vec3 p1, Vec3 p2, Vec3 n0, Vec3 n1, Vec3 n2, Vec2 t0, Vec2 t1, Vec2 t2,
                        int32_t material_id)
        : p0(p0), p1(p1), p2(p2), n0(n0), n1(n1), n2(n2), t0(t0), t1(t1), t2(t2), material_id(material_id) {}
    Vec3 p0, p1, p2;
    Vec3 n0, n1, n2;
    Vec2 t0, t1, t2;
    int32_t material_id = -1;
};

// pod_types.hpp:150-160
struct MeshSceneEntity {
    MeshSceneEntity(std::string_view name, const Mat4& model_transform) : name(name), model_matrix(model_transform) {}
    void addShape(const TriangleSceneEntity& shape) { shape_entities.push_back(shape); }
    std::string name;
    Mat4 model_matrix;
    std::vector<TriangleSceneEntity> shape_entities;
};

// pod_types.hpp:162-173
struct TextureSceneEntity {
    TextureSceneEntity(std::string_view name, const uint8_t* data, uint32_t width, uint32_t height,
                       uint32_t chl_count)
        : name(name), pixels_data(data, data + (size_t)width * height * chl_count), channels_count(chl_count),
          width(width), height(height) {}
    std::string name;
    std::vector<uint8_t> pixels_data;
    uint32_t channels_count = 0;
    uint32_t width = 0, height = 0;
};

// pod_types.hpp:175-182
struct CameraSceneEntity {
    CameraSceneEntity(std::string_view name, Mat4 view_transform, float yfov_rads)
        : name(name), y_fov_radians(yfov_rads), view_matrix(view_transform) {}
    std::string name;
    float y_fov_radians = 0.0f;
    Mat4 view_matrix;
};

// pod_types.hpp:188-212
struct BasicScene {
    void addTexture(const TextureSceneEntity& texture) { texture_entities.push_back(texture); }
    void addMaterial(const MaterialSceneEntity& material) { material_entities.push_back(material); }
    void addMesh(const MeshSceneEntity& msh) { mesh_entities.push_back(msh); }
    void addCamera(const CameraSceneEntity& cam) { camera_entities.push_back(cam); }
    std::vector<MaterialSceneEntity> material_entities;
    std::vector<MeshSceneEntity> mesh_entities;
    std::vector<CameraSceneEntity> camera_entities;
    std::vector<TextureSceneEntity> texture_entities;
};

// renderer.hpp:13-58 over include/kpt.h
class Renderer {
public:
    Renderer() = default;
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;
    ~Renderer() { shutdown(); }

    void initialize(int device = 0) {
        if (!m_ctx) detail::check(kpt_create(device, &m_ctx));
    }
    void shutdown() {
        if (m_ctx) kpt_destroy(m_ctx);
        m_ctx = nullptr;
    }

    void resizeResolution(uint32_t width, uint32_t height) {
        detail::check(kpt_resize(ctx(), (int)width, (int)height));
        m_width = width;
        m_height = height;
    }

    // one sample per pixel, as the reference's frame; then the post chain
    void executeRendering(float delta_time_ms) { executeRendering(delta_time_ms, 1); }
    void executeRendering(float delta_time_ms, int spp) { detail::check(kpt_render_frame(ctx(), spp, delta_time_ms)); }

    // headless getRenderTargetTexture: the display image, [height][width] RGBA float
    void getRenderTarget(float* rgba) const { detail::check(kpt_read_image(ctx(), rgba)); }
    std::vector<float> getRenderTarget() const {
        std::vector<float> img((size_t)m_width * m_height * 4);
        getRenderTarget(img.data());
        return img;
    }

    // getDebugRenderTargetTexture (renderer.cu:202-205): the reference's debug
    // texture, whose only write is commented out (kernels.cu:436-448), holds
    // zeros
    void getDebugRenderTarget(float* rgba) const {
        std::fill(rgba, rgba + (size_t)m_width * m_height * 4, 0.0f);
    }
    std::vector<float> getDebugRenderTarget() const { return std::vector<float>((size_t)m_width * m_height * 4, 0.0f); }

    size_t getMaterialsCount() const { return (size_t)counts()[0]; }
    size_t getMeshCount() const { return (size_t)counts()[2]; }   // the reference's meshes are instances here

    // renderer.cu:356-436: textures, materials, one mesh + instance per
    // MeshSceneEntity (the reference copies every mesh), and the first camera
    void loadScene(const BasicScene& scene) {
        kpt_context* c = ctx();
        detail::check(kpt_clear_scene(c));
        if (!scene.texture_entities.empty()) {
            std::vector<int32_t> desc;
            std::vector<uint8_t> pixels;
            for (const TextureSceneEntity& t : scene.texture_entities) {
                desc.insert(desc.end(), {(int32_t)t.width, (int32_t)t.height, (int32_t)t.channels_count,
                                         (int32_t)pixels.size()});
                pixels.insert(pixels.end(), t.pixels_data.begin(), t.pixels_data.end());
            }
            detail::check(kpt_set_textures(c, (int)scene.texture_entities.size(), desc.data(), pixels.size(),
                                           pixels.data()));
        }
        std::vector<kpt_material> mats;
        for (const MaterialSceneEntity& m : scene.material_entities) mats.push_back(to_c(m));
        detail::check(kpt_set_materials(c, (int)mats.size(), mats.data()));
        for (const MeshSceneEntity& me : scene.mesh_entities) {
            const size_t n = me.shape_entities.size();
            std::vector<float> pos(9 * n), nrm(9 * n), uv(6 * n);
            std::vector<int32_t> mat(n);
            for (size_t k = 0; k < n; ++k) {
                const TriangleSceneEntity& t = me.shape_entities[k];
                const Vec3 p[3] = {t.p0, t.p1, t.p2}, q[3] = {t.n0, t.n1, t.n2};
                const Vec2 w[3] = {t.t0, t.t1, t.t2};
                for (int v = 0; v < 3; ++v) {
                    pos[9 * k + 3 * v] = p[v].x; pos[9 * k + 3 * v + 1] = p[v].y; pos[9 * k + 3 * v + 2] = p[v].z;
                    nrm[9 * k + 3 * v] = q[v].x; nrm[9 * k + 3 * v + 1] = q[v].y; nrm[9 * k + 3 * v + 2] = q[v].z;
                    uv[6 * k + 2 * v] = w[v].x; uv[6 * k + 2 * v + 1] = w[v].y;
                }
                mat[k] = t.material_id;
            }
            int mesh = -1, inst = -1;
            detail::check(kpt_upload_mesh(c, (int)n, pos.data(), nrm.data(), uv.data(), mat.data(), &mesh));
            const std::array<float, 16> model = detail::flat(me.model_matrix);
            detail::check(kpt_add_instance(c, mesh, model.data(), -1, &inst));
        }
        detail::check(kpt_commit_scene(c));
        if (!scene.camera_entities.empty()) {
            // inverse of the view with its third column negated, inverse of a
            // left-handed perspective (y fov, 100 x 100, near 1, far 100)
            const CameraSceneEntity& cam = scene.camera_entities[0];
            std::array<float, 16> view = detail::flat(cam.view_matrix);
            for (int col = 0; col < 4; ++col) view[4 * col + 2] = -view[4 * col + 2];   // row 2 of V = column 2 of V^-1
            const float h = std::cos(0.5f * cam.y_fov_radians) / std::sin(0.5f * cam.y_fov_radians);
            const float w = h * 100.0f / 100.0f, zn = 1.0f, zf = 100.0f;
            std::array<float, 16> proj{};
            proj[0] = w;
            proj[5] = h;
            proj[10] = (zf + zn) / (zf - zn);
            proj[11] = 1.0f;
            proj[14] = -(2.0f * zf * zn) / (zf - zn);
            detail::check(kpt_set_view(c, proj.data(), view.data()));
        }
    }

    // renderer.cu:312-334
    void setExposure(const ExposureValues& v, float ev_comp, float white_point_ev, float black_point_ev) {
        kpt_exposure e{};
        e.aperture = v.aperture_f_num;
        e.iso = v.ISO;
        e.shutter = v.shutter_speed_secs;
        e.ev_comp = ev_comp;
        e.white_ev = white_point_ev;
        e.black_ev = black_point_ev;
        e.max_iso = (float)v.MAX_ISO;
        e.min_iso = (float)v.MIN_ISO;
        e.max_shutter = v.MAX_SHUTTER_SECS;
        e.min_shutter = v.MIN_SHUTTER_SECS;
        detail::check(kpt_set_exposure(ctx(), &e));
    }
    ExposureValues getExposure() const {
        kpt_exposure e{};
        detail::check(kpt_get_exposure(ctx(), &e));
        ExposureValues v;
        v.aperture_f_num = e.aperture;
        v.ISO = e.iso;
        v.shutter_speed_secs = e.shutter;
        v.MAX_ISO = (int32_t)e.max_iso;
        v.MIN_ISO = (int32_t)e.min_iso;
        v.MAX_SHUTTER_SECS = e.max_shutter;
        v.MIN_SHUTTER_SECS = e.min_shutter;
        return v;
    }

    // renderer.cu:207-248
    bool setMaterial(uint32_t index, const MaterialSceneEntity& material) {
        const kpt_material m = to_c(material);
        return kpt_set_material(ctx(), (int)index, &m) == KPT_OK;
    }
    MaterialSceneEntity getMaterial(uint32_t index) const {
        kpt_material m{};
        detail::check(kpt_get_material(ctx(), (int)index, &m));
        return MaterialSceneEntity("", m.albedo_tex, Vec3(m.albedo[0], m.albedo[1], m.albedo[2]), m.orm_tex,
                                   m.metallic, m.roughness, m.transmission_tex, m.transmission, m.ior, m.emission_tex,
                                   Vec3(m.emission[0], m.emission[1], m.emission[2]), m.emission_scale,
                                   m.normal_tex, m.normal_scale);
    }

    // renderer.cu:250-278
    bool setMeshTransform(uint32_t index, const Mat4& model_matrix) {
        const std::array<float, 16> a = detail::flat(model_matrix);
        return kpt_set_instance_transform(ctx(), (int)index, a.data()) == KPT_OK;
    }
    Mat4 getMeshTransform(uint32_t index) const {
        float a[16];
        detail::check(kpt_get_instance_transform(ctx(), (int)index, a));
        return detail::unflat(a);
    }

    // renderer.cu:290-310
    void setProceduralEnvironmentData(const ProceduralEnvironmentSettings& s) {
        kpt_environment e{};
        detail::check(kpt_get_environment(ctx(), &e));
        e.sun_angular_diameter = s.sun_angular_diameter_rad;
        e.sun_phi = s.sun_phi_rad;
        e.sun_theta = s.sun_theta_rad;
        e.sun_emission_factor = s.sun_emission_factor;
        detail::check(kpt_set_environment(ctx(), &e));
    }
    ProceduralEnvironmentSettings getProceduralEnvironmentData() const {
        kpt_environment e{};
        detail::check(kpt_get_environment(ctx(), &e));
        ProceduralEnvironmentSettings s;
        s.sun_angular_diameter_rad = e.sun_angular_diameter;
        s.sun_phi_rad = e.sun_phi;
        s.sun_theta_rad = e.sun_theta;
        s.sun_emission_factor = e.sun_emission_factor;
        return s;
    }

    void setRendererSettings(const RendererSettings& r) {
        kpt_settings s{};
        detail::check(kpt_get_settings(ctx(), &s));
        s.max_depth = r.integrator_max_ray_depth;
        s.bloom = r.bloom_generate_bloom;
        s.karis = r.bloom_use_karis_average;
        s.auto_exposure = r.tonemapper_enable_auto_exposure;
        s.bloom_final_blend = r.bloom_final_blend;
        s.bloom_internal_blend = r.bloom_internal_blend;
        s.temporal_accumulation = r.integrator_use_temporal_accumulation;
        s.postprocess_effects = r.postprocess_enable_effects;
        s.upscale = r.upscale_enable ? (r.upscale_fsr ? 2 : 1) : 0;
        detail::check(kpt_set_settings(ctx(), &s));
    }
    RendererSettings getRendererSettings() const {
        kpt_settings s{};
        detail::check(kpt_get_settings(ctx(), &s));
        RendererSettings r;
        r.integrator_max_ray_depth = s.max_depth;
        r.bloom_generate_bloom = s.bloom != 0;
        r.bloom_use_karis_average = s.karis != 0;
        r.tonemapper_enable_auto_exposure = s.auto_exposure != 0;
        r.bloom_final_blend = s.bloom_final_blend;
        r.bloom_internal_blend = s.bloom_internal_blend;
        r.integrator_use_temporal_accumulation = s.temporal_accumulation != 0;
        r.postprocess_enable_effects = s.postprocess_effects != 0;
        r.upscale_enable = s.upscale != 0;
        r.upscale_fsr = s.upscale == 2;
        return r;
    }

    // renderer.cu:342-354 (inverts both and resets the accumulation)
    void setView(const Mat4& projection_matrix, const Mat4& view_matrix) {
        const std::array<float, 16> p = detail::flat(projection_matrix), v = detail::flat(view_matrix);
        detail::check(kpt_set_view(ctx(), p.data(), v.data()));
    }

    void resetAccumulation() { detail::check(kpt_reset_accumulation(ctx())); }

    // the C-ABI context, for calls without a reference counterpart
    kpt_context* context() const { return m_ctx; }

private:
    kpt_context* ctx() const {
        if (!m_ctx) throw Error(KPT_ERR_STATE, "Renderer not initialized");
        return m_ctx;
    }
    std::array<int, 4> counts() const {
        std::array<int, 4> n{};
        detail::check(kpt_counts(ctx(), &n[0], &n[1], &n[2], &n[3]));
        return n;
    }
    static kpt_material to_c(const MaterialSceneEntity& m) {
        kpt_material c{};
        c.albedo[0] = m.albedo_factor.x; c.albedo[1] = m.albedo_factor.y; c.albedo[2] = m.albedo_factor.z;
        c.metallic = m.metallic_factor;
        c.roughness = m.roughness_factor;
        c.transmission = m.transmission_factor;
        c.ior = m.ior;
        c.emission[0] = m.emission_factor.x; c.emission[1] = m.emission_factor.y; c.emission[2] = m.emission_factor.z;
        c.emission_scale = m.emission_scale_nits;
        c.normal_scale = m.normal_scale;
        c.albedo_tex = m.albedo_texture_id;
        c.orm_tex = m.ORM_texture_id;
        c.transmission_tex = m.transmission_texture_id;
        c.emission_tex = m.emission_texture_id;
        c.normal_tex = m.normal_texture_id;
        return c;
    }

    kpt_context* m_ctx = nullptr;
    uint32_t m_width = 0, m_height = 0;
};

}  // namespace KittlesPT
