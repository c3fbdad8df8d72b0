// kpt_trace.cuh -- two-level BVH2 traversal (closest hit and any hit).
//
// Follows TLAS::intersect / TLAS::intersectP (shaders/tlas.cu:8-125),
// BLAS2::intersect / BLAS2::intersectP (shaders/blas.cuh:198-336),
// Bounds3f::intersectP (maths/bounds.cuh:38-57) and Triangle::intersect
// (shaders/triangle.cuh:66-102): the same visiting order (near child popped
// first, children culled against the closest hit so far), the same absolute
// epsilons, IEEE arithmetic.  Differences from the reference, none of which
// changes a result:
//   * child boxes live in the parent node, so the boxes tested when a node
//     is popped are the ones the reference tests, read in one record;
//   * the stacks hold 48 (BLAS) and 32 (TLAS) entries instead of 16 (the
//     reference overflows its 16-entry stacks on deep trees, which is
//     undefined behaviour); a ray that would overflow stops and is counted
//     in `overflow`.
#pragma once
#include <cooperative_groups.h>

#include "kpt_device.cuh"

namespace kpt {

namespace cg = cooperative_groups;

struct XRay { float3 o, d, inv; };

__device__ __forceinline__ XRay make_xray(float3 o, float3 d) {
    XRay r;
    r.o = o;
    r.d = d;
    r.inv = make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
    return r;
}

// Ray::transform (shaders/ray.cuh:28-31): object ray = M (o,1), M (d,0),
// direction not renormalised so that t is shared with the world ray.
__device__ __forceinline__ XRay transform_xray(const XRay& r, const float4* inv) {
    float3 o = make_float3(xrow(inv[0], r.o, 1.0f), xrow(inv[1], r.o, 1.0f), xrow(inv[2], r.o, 1.0f));
    float3 d = make_float3(xrow(inv[0], r.d, 0.0f), xrow(inv[1], r.d, 0.0f), xrow(inv[2], r.d, 0.0f));
    return make_xray(o, d);
}

// Slab test against one child box of a node.
__device__ __forceinline__ bool slab(float lx, float ly, float lz, float hx, float hy, float hz,
                                     const XRay& r, float tmin, float tmax, float* tenter_out) {
    float t0x = xm(xs(lx, r.o.x), r.inv.x), t1x = xm(xs(hx, r.o.x), r.inv.x);
    float t0y = xm(xs(ly, r.o.y), r.inv.y), t1y = xm(xs(hy, r.o.y), r.inv.y);
    float t0z = xm(xs(lz, r.o.z), r.inv.z), t1z = xm(xs(hz, r.o.z), r.inv.z);
    float tenter = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float texit = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    bool hit = (tenter <= texit) && (texit >= tmin) && (tenter <= tmax);
    *tenter_out = hit ? tenter : __int_as_float(0x7f800000);
    return hit;
}

__device__ __forceinline__ void node_slabs(const BvhNode& n, const XRay& r, float tmin, float tmax,
                                           bool* h1, float* t1, bool* h2, float* t2) {
    *h1 = slab(n.a.x, n.a.y, n.a.z, n.a.w, n.b.x, n.b.y, r, tmin, tmax, t1);
    *h2 = slab(n.b.z, n.b.w, n.c.x, n.c.y, n.c.z, n.c.w, r, tmin, tmax, t2);
}

__device__ __forceinline__ BvhNode load_node(const BvhNode* p) {
    BvhNode n;
    const float4* q = reinterpret_cast<const float4*>(p);
    n.a = __ldg(q);
    n.b = __ldg(q + 1);
    n.c = __ldg(q + 2);
    n.d = __ldg(reinterpret_cast<const int4*>(q + 3));
    return n;
}

// Moeller-Trumbore with the reference's epsilons; returns t or +inf.
__device__ __forceinline__ float tri_test(const float4* tri, const XRay& r, float tmin, float tmax,
                                          float* bu, float* bv, int* local_id) {
    float4 a = __ldg(tri), b = __ldg(tri + 1), c = __ldg(tri + 2);
    float3 v0 = make_float3(a.x, a.y, a.z);
    float3 e1 = make_float3(b.x, b.y, b.z);
    float3 e2 = make_float3(c.x, c.y, c.z);
    const float INF = __int_as_float(0x7f800000);
    float3 pv = xcross(r.d, e2);
    float det = xdot(e1, pv);
    if (det > -TRI_EPS && det < TRI_EPS) return INF;
    float inv = __frcp_rn(det);
    float3 tv = xsub3(r.o, v0);
    float u = xm(inv, xdot(tv, pv));
    if (u < 0.0f || u > 1.0f) return INF;
    float3 qv = xcross(tv, e1);
    float v = xm(inv, xdot(r.d, qv));
    if (v < 0.0f || xa(u, v) > 1.0f) return INF;
    float t = xm(inv, xdot(e2, qv));
    if (t > TRI_EPS && t < tmax && t > tmin) {
        *bu = u;
        *bv = v;
        *local_id = __float_as_int(a.w);
        return t;
    }
    return INF;
}

struct Hit {
    float t;
    int inst;       // instance, -1: miss
    int tri;        // local triangle id (mesh order)
    float u, v;
};

struct TraceStats {
    unsigned box_tests, tri_tests, inst_xforms, overflow;
};

// Stack entries: >= 0 interior node index; < 0 leaf, encoded as
// -(2 * parent + slot) - 1, whose triangle range is read back from the
// parent node when it is popped (the node is still in L1).
__device__ __forceinline__ int leaf_code(int parent, int slot) { return -(2 * parent + slot) - 1; }

// BLAS2::intersect (blas.cuh:261-336) for one instance, merged into `best`
// the way TLAS::intersect does (tlas.cu:116-121).
__device__ __forceinline__ void blas_closest(const SceneView& s, int inst, const XRay& wr, float tmin, float tmax,
                                             Hit& best, TraceStats& st, int* stack) {
    const InstRec& ir = s.inst[inst];
    const MeshRec m = s.meshes[ir.mesh];
    float4 inv[3] = {__ldg(&ir.inv[0]), __ldg(&ir.inv[1]), __ldg(&ir.inv[2])};
    XRay r = transform_xray(wr, inv);
    st.inst_xforms++;
    Hit loc;
    loc.t = __int_as_float(0x7f800000);
    loc.tri = -1;
    loc.u = loc.v = 0.0f;
    int sp = 0;
    int first = m.leaf_first, count = m.leaf_count;
    bool leaf = m.node_root < 0;
    if (!leaf) stack[sp++] = m.node_root;
    for (;;) {
        if (!leaf) {
            if (sp == 0) break;
            int e = stack[--sp];
            if (e < 0) {
                int c = -e - 1;
                int4 d = __ldg(reinterpret_cast<const int4*>(s.nodes + (c >> 1)) + 3);
                first = (c & 1) ? d.z : d.x;
                count = (c & 1) ? d.w : d.y;
                leaf = true;
            } else {
                BvhNode n = load_node(s.nodes + e);
                bool h1, h2;
                float t1, t2;
                node_slabs(n, r, tmin, tmax, &h1, &t1, &h2, &t2);
                st.box_tests += 2;
                bool p1 = h1 && t1 < loc.t, p2 = h2 && t2 < loc.t;
                if (sp + 2 > BLAS_STACK) { st.overflow++; break; }
                int c1 = n.d.y ? leaf_code(e, 0) : n.d.x;
                int c2 = n.d.w ? leaf_code(e, 1) : n.d.z;
                if (t1 > t2) {
                    if (p1) stack[sp++] = c1;
                    if (p2) stack[sp++] = c2;
                } else {
                    if (p2) stack[sp++] = c2;
                    if (p1) stack[sp++] = c1;
                }
                continue;
            }
        }
        for (int i = 0; i < count; ++i) {
            float u, v;
            int lid;
            float t = tri_test(s.tris + 3 * (size_t)(first + i), r, tmin, tmax, &u, &v, &lid);
            st.tri_tests++;
            if (t < loc.t) {
                loc.t = t;
                loc.tri = lid;
                loc.u = u;
                loc.v = v;
                tmax = t;
            }
        }
        leaf = false;
        if (m.node_root < 0) break;
    }
    if (loc.t < best.t) {
        best = loc;
        best.inst = inst;
    }
}

// TLAS::intersect (tlas.cu:60-125).
__device__ __forceinline__ Hit trace_closest(const SceneView& s, const XRay& r, float tmin, float tmax,
                                             TraceStats& st, int* stack) {
    Hit best;
    best.t = __int_as_float(0x7f800000);
    best.inst = -1;
    best.tri = -1;
    best.u = best.v = 0.0f;
    float te;
    st.box_tests++;
    if (s.ninst == 0 ||
        !slab(s.tlas_lo.x, s.tlas_lo.y, s.tlas_lo.z, s.tlas_hi.x, s.tlas_hi.y, s.tlas_hi.z, r, tmin, tmax, &te))
        return best;
    if (s.tlas_root_leaf) {
        blas_closest(s, 0, r, tmin, tmax, best, st, stack);
        return best;
    }
    int* tstack = stack + BLAS_STACK;
    int sp = 0;
    tstack[sp++] = 0;
    while (sp > 0) {
        int e = tstack[--sp];
        if (e >= 0) {
            BvhNode n = load_node(s.tlas + e);
            bool h1, h2;
            float t1, t2;
            node_slabs(n, r, tmin, tmax, &h1, &t1, &h2, &t2);
            st.box_tests += 2;
            bool p1 = h1 && t1 < best.t, p2 = h2 && t2 < best.t;
            if (sp + 2 > TLAS_STACK) { st.overflow++; break; }
            int c1 = n.d.y ? -n.d.x - 1 : n.d.x;   // TLAS leaves hold one instance
            int c2 = n.d.w ? -n.d.z - 1 : n.d.z;
            if (t1 > t2) {
                if (p1) tstack[sp++] = c1;
                if (p2) tstack[sp++] = c2;
            } else {
                if (p2) tstack[sp++] = c2;
                if (p1) tstack[sp++] = c1;
            }
        } else {
            blas_closest(s, -e - 1, r, tmin, tmax, best, st, stack);
        }
    }
    return best;
}

// BLAS2::intersectP (blas.cuh:198-259).
__device__ __forceinline__ bool blas_any(const SceneView& s, int inst, const XRay& wr, float tmin, float tmax,
                                         TraceStats& st, int* stack) {
    const InstRec& ir = s.inst[inst];
    const MeshRec m = s.meshes[ir.mesh];
    float4 inv[3] = {__ldg(&ir.inv[0]), __ldg(&ir.inv[1]), __ldg(&ir.inv[2])};
    XRay r = transform_xray(wr, inv);
    st.inst_xforms++;
    int sp = 0;
    int first = m.leaf_first, count = m.leaf_count;
    bool leaf = m.node_root < 0;
    if (!leaf) stack[sp++] = m.node_root;
    for (;;) {
        if (!leaf) {
            if (sp == 0) return false;
            int e = stack[--sp];
            if (e < 0) {
                int c = -e - 1;
                int4 d = __ldg(reinterpret_cast<const int4*>(s.nodes + (c >> 1)) + 3);
                first = (c & 1) ? d.z : d.x;
                count = (c & 1) ? d.w : d.y;
            } else {
                BvhNode n = load_node(s.nodes + e);
                bool h1, h2;
                float t1, t2;
                node_slabs(n, r, tmin, tmax, &h1, &t1, &h2, &t2);
                st.box_tests += 2;
                if (sp + 2 > BLAS_STACK) { st.overflow++; return false; }
                int c1 = n.d.y ? leaf_code(e, 0) : n.d.x;
                int c2 = n.d.w ? leaf_code(e, 1) : n.d.z;
                // near child pushed last, popped first
                if (t1 > t2) {
                    if (h1) stack[sp++] = c1;
                    if (h2) stack[sp++] = c2;
                } else {
                    if (h2) stack[sp++] = c2;
                    if (h1) stack[sp++] = c1;
                }
                continue;
            }
        }
        for (int i = 0; i < count; ++i) {
            float u, v;
            int lid;
            float t = tri_test(s.tris + 3 * (size_t)(first + i), r, tmin, tmax, &u, &v, &lid);
            st.tri_tests++;
            if (t < __int_as_float(0x7f800000)) return true;
        }
        leaf = false;
        if (m.node_root < 0) return false;
    }
}

// TLAS::intersectP (tlas.cu:8-58).
__device__ __forceinline__ bool trace_any(const SceneView& s, const XRay& r, float tmin, float tmax,
                                          TraceStats& st, int* stack) {
    float te;
    st.box_tests++;
    if (s.ninst == 0 ||
        !slab(s.tlas_lo.x, s.tlas_lo.y, s.tlas_lo.z, s.tlas_hi.x, s.tlas_hi.y, s.tlas_hi.z, r, tmin, tmax, &te))
        return false;
    if (s.tlas_root_leaf) return blas_any(s, 0, r, tmin, tmax, st, stack);
    int* tstack = stack + BLAS_STACK;
    int sp = 0;
    tstack[sp++] = 0;
    while (sp > 0) {
        int e = tstack[--sp];
        if (e >= 0) {
            BvhNode n = load_node(s.tlas + e);
            bool h1, h2;
            float t1, t2;
            node_slabs(n, r, tmin, tmax, &h1, &t1, &h2, &t2);
            st.box_tests += 2;
            if (sp + 2 > TLAS_STACK) { st.overflow++; return false; }
            int c1 = n.d.y ? -n.d.x - 1 : n.d.x;
            int c2 = n.d.w ? -n.d.z - 1 : n.d.z;
            if (t1 > t2) {
                if (h1) tstack[sp++] = c1;
                if (h2) tstack[sp++] = c2;
            } else {
                if (h2) tstack[sp++] = c2;
                if (h1) tstack[sp++] = c1;
            }
        } else if (blas_any(s, -e - 1, r, tmin, tmax, st, stack)) {
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Queue traversal: a persistent warp walks a queue of rays.  Each lane runs
// its own ray and, when the ray is done, fetches the next queue entry (one
// atomic per group of lanes fetching together), so no lane waits for the
// longest ray of its warp.  One loop iteration is one step of a lane's ray --
// a node (TLAS and BLAS share the node format), one triangle, entering or
// leaving an instance -- so lanes at different depths of the two levels keep
// issuing together.  The visiting order and culling are those of
// trace_closest / trace_any above (the BLAS keeps its local closest hit and
// culls against it, and is merged into the ray's closest hit when left), so
// every result is identical to theirs.
//
// Src supplies the queue:  void ray(int i, float3& o, float3& d, float& tmin, float& tmax);
//                          bool closest(int i, const Hit& h, float3& o, float3& d);   (ANY == false)
//                          void any(int i, bool occluded);      (ANY == true)
// closest() may return true with the next ray of entry i (a bounce chain):
// the lane traces it at once, with the same tmin and tmax.  TRI triangles of
// a leaf are tested per loop iteration (in order; 1 is fastest on the
// instanced full frame, 2 on one BLAS of 2M random triangles).  ROOTS: the
// queue spans several scenes merged into `s` (a batch), each entry's TLAS
// root supplied by
//                          void root(int i, float4& lo, float4& hi, int& root, int& ninst);
// (root: a node index of s.tlas, or -(instance) - 1 for a single-instance scene).
template <bool ANY, class Src, int TRI = 1, bool ROOTS = false>
__device__ __forceinline__ void trace_queue(const SceneView& s, int n, int* next, Src& src, TraceStats& st,
                                            int* stack) {
    const float INF = __int_as_float(0x7f800000);
    XRay w, r;               // world ray; current ray (object space inside an instance)
    float tmin = 0.0f, tmax0 = INF;
    Hit best, loc;           // closest hit of the ray; of the instance being traversed
    int ray = -1;            // queue entry, -1: fetch the next one
    int inst = -1;           // instance being traversed, -1: in the TLAS
    int base = 0;            // stack height when the instance was entered
    int sp = 0;
    // the top of the stack lives in a register: a node step keeps its near
    // child here instead of pushing and popping it through local memory
    constexpr int NONE = (int)0x80000000;
    int top = NONE;
    int first = 0, count = 0;   // triangles of the leaf being tested
    best.t = loc.t = INF;
    best.inst = best.tri = loc.inst = loc.tri = -1;
    best.u = best.v = loc.u = loc.v = 0.0f;
    // a new ray: the TLAS root box (TLAS::intersect, tlas.cu:60-75), then its root
    auto start = [&](float3 o, float3 d) {
        w = make_xray(o, d);
        r = w;
        best.t = INF;
        best.inst = best.tri = -1;
        best.u = best.v = 0.0f;
        inst = -1;
        sp = 0;
        top = NONE;
        count = 0;
        float te;
        st.box_tests++;
        if constexpr (ROOTS) {
            float4 lo, hi;
            int root, ninst;
            src.root(ray, lo, hi, root, ninst);
            if (ninst > 0 && slab(lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, w, tmin, tmax0, &te)) top = root;
        } else {
            if (s.ninst > 0 &&
                slab(s.tlas_lo.x, s.tlas_lo.y, s.tlas_lo.z, s.tlas_hi.x, s.tlas_hi.y, s.tlas_hi.z, w, tmin, tmax0, &te))
                top = s.tlas_root_leaf ? -1 : 0;   // TLAS entries: node index, or -(instance) - 1
        }
    };
    bool occluded = false;   // ANY: a triangle blocked the ray
    for (;;) {
        // a lane whose ray is done waits until fetch_batch lanes of the warp
        // are (or all are): the result write and the next fetch and set-up
        // then run for those lanes together instead of one lane at a time
        const bool fin = ray < 0 || (count == 0 && inst < 0 && top == NONE && sp == 0);
        const unsigned act = __activemask();
        const unsigned idle = __ballot_sync(act, fin);
        if (fin) {
            if (idle != act && __popc(idle) < s.fetch_batch) continue;
            if (ray >= 0) {
                float3 o, d;
                if (ANY) {
                    src.any(ray, occluded);
                    ray = -1;
                } else if (src.closest(ray, best, o, d)) {
                    start(o, d);   // the next ray of a bounce chain
                    continue;
                } else {
                    ray = -1;
                }
            }
            cg::coalesced_group g = cg::coalesced_threads();
            int b = 0;
            if (g.thread_rank() == 0) b = atomicAdd(next, (int)g.size());
            ray = g.shfl(b, 0) + (int)g.thread_rank();
            if (ray >= n) break;
            float3 o, d;
            src.ray(ray, o, d, tmin, tmax0);
            start(o, d);
            occluded = false;
        } else if (count > 0) {
            // TRI triangles of the leaf, in order (BLAS2::intersect /
            // intersectP leaf loop)
#pragma unroll
            for (int k = 0; k < TRI; ++k) {
                if (count == 0) break;
                float u, v;
                int lid;
                const float tmx = ANY ? tmax0 : fminf(tmax0, loc.t);
                float t = tri_test(s.tris + 3 * (size_t)first, r, tmin, tmx, &u, &v, &lid);
                st.tri_tests++;
                ++first;
                --count;
                if (ANY) {
                    if (t < INF) {   // blocked: the ray is done
                        occluded = true;
                        count = 0;
                        inst = -1;
                        top = NONE;
                        sp = 0;
                    }
                } else if (t < loc.t) {
                    loc.t = t;
                    loc.tri = lid;
                    loc.u = u;
                    loc.v = v;
                }
            }
        } else if (inst >= 0 && top == NONE && sp == base) {
            // leaving the instance: merge its closest hit (tlas.cu:116-121)
            if (!ANY && loc.t < best.t) {
                best = loc;
                best.inst = inst;
            }
            inst = -1;
            r = w;
        } else {
            const int e = top != NONE ? top : stack[--sp];
            top = NONE;
            if (e >= 0) {
                // interior node of the TLAS or of the instance's BLAS
                const bool in_blas = inst >= 0;
                const BvhNode nd = load_node((in_blas ? s.nodes : s.tlas) + e);
                const float cull = ANY ? INF : (in_blas ? loc.t : best.t);
                const float tmx = (ANY || !in_blas) ? tmax0 : fminf(tmax0, loc.t);
                bool h1, h2;
                float t1, t2;
                node_slabs(nd, r, tmin, tmx, &h1, &t1, &h2, &t2);
                st.box_tests += 2;
                const bool p1 = h1 && t1 < cull, p2 = h2 && t2 < cull;
                if (in_blas ? (sp - base + 1 > BLAS_STACK) : (sp + 1 > TLAS_STACK)) {
                    st.overflow++;
                    sp = in_blas ? base : 0;   // the reference's stack would overflow: end this level
                } else {
                    const int c1 = nd.d.y ? (in_blas ? leaf_code(e, 0) : -nd.d.x - 1) : nd.d.x;
                    const int c2 = nd.d.w ? (in_blas ? leaf_code(e, 1) : -nd.d.z - 1) : nd.d.z;
                    // near child popped first: the far one goes to memory, the
                    // near one stays in the register
                    const bool far1 = t1 > t2;
                    const int ca = far1 ? c1 : c2, cb = far1 ? c2 : c1;
                    const bool pa = far1 ? p1 : p2, pb = far1 ? p2 : p1;
                    if (pa && pb) stack[sp++] = ca;
                    // the child visited next: a BLAS leaf starts at once, its
                    // triangle range is in this node (no push, pop, setup step)
                    const int cn = pb ? (far1 ? 1 : 0) : (far1 ? 0 : 1);
                    const int ncount = cn ? nd.d.w : nd.d.y;
                    if ((pa || pb) && in_blas && ncount > 0) {
                        first = cn ? nd.d.z : nd.d.x;
                        count = ncount;
                        top = NONE;
                    } else {
                        top = pb ? cb : (pa ? ca : NONE);
                    }
                }
            } else if (inst < 0) {
                // entering an instance (TLAS leaf): object-space ray (Ray::transform)
                inst = -e - 1;
                const InstRec& ir = s.inst[inst];
                const MeshRec m = s.meshes[ir.mesh];
                const float4 inv[3] = {__ldg(&ir.inv[0]), __ldg(&ir.inv[1]), __ldg(&ir.inv[2])};
                r = transform_xray(w, inv);
                st.inst_xforms++;
                base = sp;
                loc.t = INF;
                loc.tri = -1;
                loc.u = loc.v = 0.0f;
                if (m.node_root < 0) {
                    first = m.leaf_first;
                    count = m.leaf_count;
                } else {
                    top = m.node_root;
                }
            } else {
                // BLAS leaf: its triangle range is read back from the parent node
                const int c = -e - 1;
                const int4 d = __ldg(reinterpret_cast<const int4*>(s.nodes + (c >> 1)) + 3);
                first = (c & 1) ? d.z : d.x;
                count = (c & 1) ? d.w : d.y;
            }
        }
    }
}

}  // namespace kpt
