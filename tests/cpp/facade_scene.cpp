// Reference-style host code against the C++ facade (include/kittlespt_gb300/
// renderer.hpp): builds a BasicScene (ground quad, a faceted sphere, an
// emissive quad), loads it, sets settings, exposure, environment and a view,
// renders frames and writes the scene's arrays, the view matrices and the
// display image to a binary file, so that a test can rebuild the same scene
// through the C ABI and compare the images.  Exits 3 when no GPU context can be created.
//
// usage: facade_scene <out.bin> <width> <height> <frames>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kittlespt_gb300/renderer.hpp"

using namespace KittlesPT;

static void add_quad(MeshSceneEntity& m, float y, float half, bool up, int mat) {
    Vec3 a(-half, y, -half), b(half, y, -half), c(half, y, half), d(-half, y, half);
    Vec3 n(0.0f, up ? 1.0f : -1.0f, 0.0f);
    Vec2 t0{}, t1{}, t2{};
    if (up) {
        m.addShape(TriangleSceneEntity(a, c, b, n, n, n, t0, t1, t2, mat));
        m.addShape(TriangleSceneEntity(a, d, c, n, n, n, t0, t1, t2, mat));
    } else {
        m.addShape(TriangleSceneEntity(a, b, c, n, n, n, t0, t1, t2, mat));
        m.addShape(TriangleSceneEntity(a, c, d, n, n, n, t0, t1, t2, mat));
    }
}

static void add_sphere(MeshSceneEntity& m, int seg, int rings, float r, int mat) {
    auto p = [&](int i, int j) {
        float th = 3.14159265f * (float)j / (float)rings, ph = 6.28318531f * (float)i / (float)seg;
        return Vec3(r * std::sin(th) * std::cos(ph), r * std::cos(th), r * std::sin(th) * std::sin(ph));
    };
    auto nrm = [&](Vec3 v) { return Vec3(v.x / r, v.y / r, v.z / r); };
    Vec2 t{};
    for (int j = 0; j < rings; ++j)
        for (int i = 0; i < seg; ++i) {
            Vec3 a = p(i, j), b = p(i + 1, j), c = p(i + 1, j + 1), d = p(i, j + 1);
            if (j > 0) m.addShape(TriangleSceneEntity(a, b, c, nrm(a), nrm(b), nrm(c), t, t, t, mat));
            if (j < rings - 1) m.addShape(TriangleSceneEntity(a, c, d, nrm(a), nrm(c), nrm(d), t, t, t, mat));
        }
}

static Mat4 translate(float x, float y, float z) {
    Mat4 m;
    m[3][0] = x;
    m[3][1] = y;
    m[3][2] = z;
    return m;
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s out.bin width height frames\n", argv[0]);
        return 2;
    }
    const int W = std::atoi(argv[2]), H = std::atoi(argv[3]), frames = std::atoi(argv[4]);
    BasicScene scene;
    scene.addMaterial(MaterialSceneEntity("ground", -1, Vec3(0.5f, 0.5f, 0.5f), -1, 0.0f, 0.8f, -1, 0.0f, 1.45f, -1,
                                          Vec3(1.0f, 1.0f, 1.0f), 0.0f, -1, 1.0f));
    scene.addMaterial(MaterialSceneEntity("metal", -1, Vec3(0.95f, 0.64f, 0.54f), -1, 1.0f, 0.3f, -1, 0.0f, 1.45f, -1,
                                          Vec3(1.0f, 1.0f, 1.0f), 0.0f, -1, 1.0f));
    scene.addMaterial(MaterialSceneEntity("light", -1, Vec3(0.8f, 0.8f, 0.8f), -1, 0.0f, 0.5f, -1, 0.0f, 1.45f, -1,
                                          Vec3(1.0f, 0.9f, 0.8f), 20.0f, -1, 1.0f));
    MeshSceneEntity ground("ground", translate(0.0f, -1.0f, 0.0f));
    add_quad(ground, 0.0f, 10.0f, true, 0);
    MeshSceneEntity ball("ball", translate(0.3f, 0.0f, 0.0f));
    add_sphere(ball, 24, 12, 1.0f, 1);
    MeshSceneEntity lamp("lamp", translate(-1.5f, 2.0f, 0.5f));
    add_quad(lamp, 0.0f, 0.5f, false, 2);
    scene.addMesh(ground);
    scene.addMesh(ball);
    scene.addMesh(lamp);
    scene.addCamera(CameraSceneEntity("cam", translate(0.0f, -1.0f, -5.0f), 0.785398f));

    Renderer r;
    try {
        r.initialize(0);
    } catch (const Error& e) {
        std::printf("no GPU context: %s\n", e.what());
        return 3;
    }
    try {
        r.resizeResolution((uint32_t)W, (uint32_t)H);
        r.loadScene(scene);
        RendererSettings s = r.getRendererSettings();
        s.integrator_max_ray_depth = 4;
        s.bloom_generate_bloom = true;
        s.tonemapper_enable_auto_exposure = true;
        r.setRendererSettings(s);
        r.setExposure(ExposureValues(11.0f, 100, 0.004f), 0.0f, 6.5f, -10.0f);
        ProceduralEnvironmentSettings env = r.getProceduralEnvironmentData();
        env.sun_theta_rad = 0.5236f;
        r.setProceduralEnvironmentData(env);
        // the same camera through setView (renderer.cu:342-354): a left-handed
        // perspective and the view with its third row negated
        Mat4 P, V = translate(0.0f, -1.0f, -5.0f);
        {
            const float h = std::cos(0.5f * 0.785398f) / std::sin(0.5f * 0.785398f);
            for (int c = 0; c < 4; ++c)
                for (int k = 0; k < 4; ++k) P[c][k] = 0.0f;
            P[0][0] = h * (float)H / (float)W;
            P[1][1] = h;
            P[2][2] = 101.0f / 99.0f;
            P[2][3] = 1.0f;
            P[3][2] = -200.0f / 99.0f;
            for (int c = 0; c < 4; ++c) V[c][2] = -V[c][2];
        }
        r.setView(P, V);
        if (r.getMaterialsCount() != 3 || r.getMeshCount() != 3) {
            std::printf("bad counts\n");
            return 1;
        }
        if (r.setMaterial(7, scene.material_entities[0])) {   // out of range: false, as in the reference
            std::printf("setMaterial accepted a bad index\n");
            return 1;
        }
        for (int f = 0; f < frames; ++f) r.executeRendering(16.0f, 2);
        std::vector<float> img = r.getRenderTarget();
        const std::vector<float> dbg = r.getDebugRenderTarget();   // nothing writes it: zeros
        if (dbg.size() != img.size() || std::any_of(dbg.begin(), dbg.end(), [](float v) { return v != 0.0f; })) {
            std::printf("debug render target is not a zero image of the output size\n");
            return 1;
        }
        // arrays of the scene as the facade passed them, then the image
        FILE* fp = std::fopen(argv[1], "wb");
        if (!fp) return 1;
        int32_t hdr[4] = {W, H, frames, (int32_t)scene.mesh_entities.size()};
        std::fwrite(hdr, sizeof hdr, 1, fp);
        for (const MeshSceneEntity& m : scene.mesh_entities) {
            int32_t n = (int32_t)m.shape_entities.size();
            std::fwrite(&n, 4, 1, fp);
            for (const TriangleSceneEntity& t : m.shape_entities) {
                const Vec3 v[6] = {t.p0, t.p1, t.p2, t.n0, t.n1, t.n2};
                for (const Vec3& q : v) std::fwrite(&q, 12, 1, fp);
                std::fwrite(&t.material_id, 4, 1, fp);
            }
            float model[16];
            for (int c = 0; c < 4; ++c)
                for (int k = 0; k < 4; ++k) model[4 * c + k] = m.model_matrix[c][k];
            std::fwrite(model, sizeof model, 1, fp);
        }
        float pv[32];
        for (int c = 0; c < 4; ++c)
            for (int k = 0; k < 4; ++k) {
                pv[4 * c + k] = P[c][k];
                pv[16 + 4 * c + k] = V[c][k];
            }
        std::fwrite(pv, sizeof pv, 1, fp);
        std::fwrite(img.data(), sizeof(float), img.size(), fp);
        std::fclose(fp);
        std::printf("ok %d x %d, %d frames\n", W, H, frames);
    } catch (const Error& e) {
        std::printf("error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
