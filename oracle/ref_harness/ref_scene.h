// ref_scene.h -- builds a scene with the reference's own host code, as
// Renderer::loadScene (renderer.cu:356-436) followed by
// Renderer::setMeshTransform (renderer.cu:250-269) for every mesh, into the
// reference's buffers.  One difference: the mesh inverse is the reference's
// own Mat4::inverse of the model matrix rather than glm::inverse, so that the
// oracle and the harnesses share one inverse routine.  Shared by the host
// harness (ref_harness.cpp) and the GPU harness (ref_gpu_harness.cu); the
// including file has already included the reference's shaders, as_builder.cuh
// and pod_types.hpp.
//
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include "ref_records.h"

namespace {

using namespace KittlesPT;

struct RefScene {
    thrust::universal_vector<TLASNode> tlasnodes;
    thrust::universal_vector<BLAS2> blas;
    thrust::universal_vector<BVH2Node> nodes;
    thrust::universal_vector<int32_t> tri_index;
    thrust::universal_vector<TriangleMesh> meshes;
    thrust::universal_vector<Light> lights;
    thrust::universal_vector<Triangle> tris;
    thrust::universal_vector<Material> materials;
    thrust::universal_vector<Texture> textures;
    thrust::universal_vector<uint8_t> pixels;
    ShaderData sd;
};

inline Mat4 mat_from(const float* cm) {
    return Mat4(make_float4(cm[0], cm[1], cm[2], cm[3]), make_float4(cm[4], cm[5], cm[6], cm[7]),
                make_float4(cm[8], cm[9], cm[10], cm[11]), make_float4(cm[12], cm[13], cm[14], cm[15]));
}

inline void ref_replay_load_scene(RefScene* r, int ntris, const float* pos, const float* nrm, const float* uv,
                                  const int* mat, int nmeshes, const int* mesh_off, const int* mesh_cnt,
                                  const float* models, int nmaterials, const void* materials, int ntextures,
                                  const int* tex_desc, long long npixels, const unsigned char* pixels) {
    (void)ntris;
    const MaterialRecord* mr = (const MaterialRecord*)materials;
    for (int i = 0; i < nmaterials; ++i) {
        const MaterialRecord& m = mr[i];
        r->materials.push_back(Material(m.albedo_tex, make_float3(m.albedo[0], m.albedo[1], m.albedo[2]),
                                        m.orm_tex, m.metallic, m.roughness, m.transmission_tex, m.transmission,
                                        m.ior, m.emission_tex,
                                        make_float3(m.emission[0], m.emission[1], m.emission[2]),
                                        m.emission_scale, m.normal_tex, m.normal_scale));
    }
    for (int i = 0; i < ntextures; ++i)
        r->textures.push_back(Texture(tex_desc[4 * i], tex_desc[4 * i + 1], tex_desc[4 * i + 2], 8, tex_desc[4 * i + 3]));
    if (npixels > 0) r->pixels.assign(pixels, pixels + npixels);

    BLASBuilder builder(&r->tris, &r->tri_index, &r->nodes);
    for (int mi = 0; mi < nmeshes; ++mi) {
        size_t start = r->tris.size();
        for (int k = 0; k < mesh_cnt[mi]; ++k) {
            int i = mesh_off[mi] + k;
            const MaterialRecord& m = mr[mat[i]];
            glm::vec3 p[3], n[3];
            glm::vec2 t[3];
            for (int v = 0; v < 3; ++v) {
                p[v] = glm::vec3(pos[9 * i + 3 * v], pos[9 * i + 3 * v + 1], pos[9 * i + 3 * v + 2]);
                n[v] = glm::vec3(nrm[9 * i + 3 * v], nrm[9 * i + 3 * v + 1], nrm[9 * i + 3 * v + 2]);
                t[v] = glm::vec2(uv[6 * i + 2 * v], uv[6 * i + 2 * v + 1]);
            }
            TriangleSceneEntity tri(p[0], p[1], p[2], n[0], n[1], n[2], t[0], t[1], t[2], mat[i]);
            MaterialSceneEntity mse;
            mse.emission_factor = glm::vec3(m.emission[0], m.emission[1], m.emission[2]);
            mse.emission_scale_nits = m.emission_scale;
            int32_t light_id = -1;
            if (mse.isEmissive()) {
                int32_t prim_id = (int32_t)r->tris.size();
                r->lights.push_back(Light(tri.getArea(), prim_id, make_float3(m.emission[0], m.emission[1], m.emission[2]),
                                          m.emission_scale));
                light_id = (int32_t)r->lights.size() - 1;
            }
            r->tris.push_back(Triangle(Vertex(make_float3(p[0].x, p[0].y, p[0].z), make_float3(n[0].x, n[0].y, n[0].z), make_float2(t[0].x, t[0].y)),
                                       Vertex(make_float3(p[1].x, p[1].y, p[1].z), make_float3(n[1].x, n[1].y, n[1].z), make_float2(t[1].x, t[1].y)),
                                       Vertex(make_float3(p[2].x, p[2].y, p[2].z), make_float3(n[2].x, n[2].y, n[2].z), make_float2(t[2].x, t[2].y)),
                                       mat[i], light_id, mi));
        }
        Mat4 model = mat_from(models + 16 * mi);
        Mat4 inv = model.inverse();
        TriangleMesh tm((int)start, mesh_cnt[mi], inv);
        tm.blas_index = (int32_t)r->blas.size();
        r->blas.push_back(builder.build(tm, mi));
        r->meshes.push_back(tm);
    }
    // setMeshTransform for every mesh (renderer.cu:250-269)
    for (int mi = 0; mi < nmeshes; ++mi) {
        Mat4 model = mat_from(models + 16 * mi);
        TriangleMesh tm = r->meshes[mi];
        tm.setTransform(model.inverse());
        r->meshes[mi] = tm;
        BLAS2 b = r->blas[tm.blas_index];
        b.setTransform(model);
        r->blas[tm.blas_index] = b;
    }
    TLASBuilder tb(&r->blas, &r->tlasnodes);
    r->sd.top_level_acceleration_structure = tb.build();
}

}  // namespace
