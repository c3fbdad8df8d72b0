// kpt_scene.h -- host-side scene build: BLAS and TLAS construction and the
// packing of the device records (IEEE single precision, no contraction).
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "kpt_device.cuh"

namespace kpt {

struct HostMesh {                    // one uploaded mesh (BLAS geometry)
    std::vector<float> pos;          // 9 per triangle
    std::vector<float> nrm;          // 9 per triangle
    std::vector<float> uv;           // 6 per triangle
    std::vector<int> material;       // 1 per triangle
    // built
    std::vector<BvhNode> nodes;      // interior nodes, local indices
    std::vector<int> order;          // leaf order -> mesh triangle
    int root = -1, leaf_first = 0, leaf_count = 0;
    float lo[3], hi[3];              // object-space bounds (BLAS2::original_bounds)
    int max_depth = 0;
    int ntris() const { return (int)material.size(); }
};

struct HostInstance {
    int mesh;
    float model[16];                 // column-major
    int material;                    // override or -1
    float prev_model[16];            // the transform before the last change (TriangleMesh prev, triangle.cuh:142-146)
};

// Binned SAH build of the reference (as_builder.cuh:110-261).
void build_blas(HostMesh& m);

// A node of the reference's BLAS array: interior (count 0) with children at
// left_first and left_first + 1, or a leaf of `count` triangles
// order[left_first ..].  Node 0 is the root.
struct BlasNode {
    int left_first;
    int count;
    float lo[3], hi[3];
};

// Packs a reference-form tree (nodes, triangle order) into m: device nodes
// in depth-first order (left first), leaf ranges, root, bounds and depth.
void pack_blas(HostMesh& m, const std::vector<BlasNode>& nodes, std::vector<int>&& order);

// The same build on the GPU (kpt_build.cu): identical nodes, boxes and
// triangle order.  Returns a CUDA error code (0 on success).
int build_blas_device(HostMesh& m, cudaStream_t stream);

// Refit on the GPU after m.pos (and m.nrm) changed, same tree: recomputes
// the child boxes of the mesh's nodes at node_base of the scene's device
// node array bottom up, rewrites its triangle records and the geometric
// normals of its shading records at tri_base, and updates m.nodes' boxes
// and m.lo / m.hi.  Returns a CUDA error code (0 on success).
int refit_blas_device(HostMesh& m, BvhNode* d_nodes, int node_base, float4* d_tris, int tri_base, TriShade* d_shade,
                      cudaStream_t stream);

// World bounds of an instance: the 8 transformed corners of the mesh bounds
// (BLAS2::setTransform, blas.cuh:338-348).
void instance_bounds(const HostMesh& m, const float* model, float* lo, float* hi);

// Agglomerative TLAS (as_builder.cuh:312-392) converted to the device node
// format.  Returns the nodes; root_leaf is set for a single instance.
std::vector<BvhNode> build_tlas(const std::vector<float>& lo, const std::vector<float>& hi, int n,
                                float* root_lo, float* root_hi, int* root_leaf, int* max_depth);

// Closed-form 4x4 inverse of the reference (matrix_maths.cuh:304-354),
// identity when |det| < 1e-6.  Column-major in and out.
void inverse4(const float* m, float* out);

// Local geometric normal of a triangle (Triangle constructor,
// triangle.cuh:51-64) and its area (pod_types.hpp:143-146).
void tri_normal_area(const float* p, const float* n, float* gn, float* area);

}  // namespace kpt
