// kpt_scene.cpp -- host-side acceleration-structure build.
//
// The BLAS builder is the reference's binned SAH (as_builder.cuh:110-261:
// 8 bins on each axis, centroid = (v0+v1+v2)*0.3333f, split search on
// centroid bounds, partition in place, leaves of at most 8 triangles, a
// split that leaves one side empty ends the recursion), so the tree -- and
// with it the traversal order and tie-breaking of closest hits -- is the
// reference's.  The result is packed into the device format: interior nodes
// only, each holding both child boxes, triangles reordered into leaf order.
// The TLAS is the reference's agglomerative clustering on half surface area
// (as_builder.cuh:312-392).  Compiled with -ffp-contract=off so that x86-64
// and aarch64 builds produce the same floats.
#include "kpt_scene.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <utility>

namespace kpt {

namespace {

struct V3 { float x, y, z; };
inline V3 vmin(V3 a, V3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }

struct Box {
    V3 lo = {FLT_MAX, FLT_MAX, FLT_MAX}, hi = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(V3 p) { lo = vmin(lo, p); hi = vmax(hi, p); }
    void grow(const Box& b) { grow(b.hi); grow(b.lo); }   // bounds.cuh:22-26 (max first)
    float area() const {
        V3 d = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
        return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
    }
};

struct RefNode { int left_first = -1; uint32_t count = 0; Box b; };

struct Builder {
    const float* pos;
    std::vector<V3> cen;
    std::vector<int> idx;
    std::vector<RefNode> nodes;

    V3 vert(int t, int k) const { return {pos[9 * t + 3 * k], pos[9 * t + 3 * k + 1], pos[9 * t + 3 * k + 2]}; }
    static float comp(V3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

    void bounds(int ni) {
        RefNode& n = nodes[ni];
        n.b = Box();
        for (uint32_t i = 0; i < n.count; ++i) {
            int t = idx[n.left_first + i];
            n.b.grow(vert(t, 0)); n.b.grow(vert(t, 1)); n.b.grow(vert(t, 2));
        }
    }
    void best_split(const RefNode& n, int* axis, float* pos_) {
        const int B = 8;
        float best = INFINITY;
        for (int a = 0; a < 3; ++a) {
            float mn = INFINITY, mx = -INFINITY;
            for (uint32_t i = 0; i < n.count; ++i) {
                float c = comp(cen[idx[n.left_first + i]], a);
                mn = fminf(mn, c);
                mx = fmaxf(mx, c);
            }
            if (mn == mx) continue;
            Box bb[B];
            uint32_t bn[B] = {0};
            float scale = (float)B / (mx - mn);
            for (uint32_t i = 0; i < n.count; ++i) {
                int t = idx[n.left_first + i];
                int bi = std::min(B - 1, (int)((comp(cen[t], a) - mn) * scale));
                bn[bi]++;
                bb[bi].grow(vert(t, 0)); bb[bi].grow(vert(t, 1)); bb[bi].grow(vert(t, 2));
            }
            const int P = B - 1;
            float la[P], ra[P];
            int lc[P], rc[P];
            Box lb, rb;
            int ls = 0, rs = 0;
            for (int i = 0; i < P; ++i) {
                ls += bn[i]; lc[i] = ls; lb.grow(bb[i]); la[i] = lb.area();
                rs += bn[P - i]; rc[P - 1 - i] = rs; rb.grow(bb[P - i]); ra[P - 1 - i] = rb.area();
            }
            scale = (mx - mn) / (float)B;
            for (int i = 0; i < P; ++i) {
                float cost = lc[i] * la[i] + rc[i] * ra[i];
                if (cost < best) { *axis = a; *pos_ = mn + scale * (i + 1); best = cost; }
            }
        }
    }
    // iterative form of BLASBuilder::subdivide (as_builder.cuh:181-233); the
    // children are created in the same order, so node numbering matches
    void subdivide(int root, uint32_t* next) {
        std::vector<int> work;
        work.push_back(root);
        while (!work.empty()) {
            int ni = work.back();
            work.pop_back();
            RefNode& p = nodes[ni];
            if (p.count <= 8) continue;
            int axis = -1;
            float sp = 0.0f;
            best_split(p, &axis, &sp);
            int i = p.left_first, j = i + (int)p.count - 1;
            while (i <= j) {
                if (comp(cen[idx[i]], axis) < sp) i++;
                else std::swap(idx[i], idx[j--]);
            }
            uint32_t lcount = (uint32_t)(i - p.left_first);
            if (lcount == 0 || lcount == p.count) continue;
            int lid = (int)(*next)++, rid = (int)(*next)++;
            RefNode l, r;
            l.left_first = p.left_first; l.count = lcount;
            r.left_first = i; r.count = p.count - lcount;
            p.count = 0;
            p.left_first = lid;
            nodes[lid] = l;
            nodes[rid] = r;
            bounds(lid);
            bounds(rid);
            // recursion order: left subtree completely, then right
            work.push_back(rid);
            work.push_back(lid);
        }
    }
};

inline void pack_child(const Box& b, float* dst6) {
    dst6[0] = b.lo.x; dst6[1] = b.lo.y; dst6[2] = b.lo.z; dst6[3] = b.hi.x; dst6[4] = b.hi.y; dst6[5] = b.hi.z;
}
inline BvhNode make_node(const Box& b1, int r1, int c1, const Box& b2, int r2, int c2) {
    float v[12];
    pack_child(b1, v);
    pack_child(b2, v + 6);
    BvhNode n;
    n.a = make_float4(v[0], v[1], v[2], v[3]);
    n.b = make_float4(v[4], v[5], v[6], v[7]);
    n.c = make_float4(v[8], v[9], v[10], v[11]);
    n.d = make_int4(r1, c1, r2, c2);
    return n;
}

}  // namespace

void pack_blas(HostMesh& m, const std::vector<BlasNode>& nodes, std::vector<int>&& order) {
    const BlasNode& rb = nodes[0];
    for (int k = 0; k < 3; ++k) {
        m.lo[k] = rb.lo[k];
        m.hi[k] = rb.hi[k];
    }
    m.order = std::move(order);
    m.nodes.clear();
    m.max_depth = 0;
    if (nodes[0].count != 0) {       // the root is a leaf
        m.root = -1;
        m.leaf_first = 0;
        m.leaf_count = nodes[0].count;
        return;
    }
    // interior nodes in depth-first order (left first)
    std::vector<int> dev(nodes.size(), -1);
    std::vector<std::pair<int, int>> stack;   // (reference node, depth)
    stack.push_back({0, 1});
    std::vector<int> seq;
    while (!stack.empty()) {
        auto [ni, dep] = stack.back();
        stack.pop_back();
        m.max_depth = std::max(m.max_depth, dep);
        dev[ni] = (int)seq.size();
        seq.push_back(ni);
        const BlasNode& n = nodes[ni];
        int l = n.left_first, r = n.left_first + 1;
        if (nodes[r].count == 0) stack.push_back({r, dep + 1});
        if (nodes[l].count == 0) stack.push_back({l, dep + 1});
    }
    auto box = [](const BlasNode& n) {
        Box b;
        b.lo = {n.lo[0], n.lo[1], n.lo[2]};
        b.hi = {n.hi[0], n.hi[1], n.hi[2]};
        return b;
    };
    m.nodes.resize(seq.size());
    for (size_t k = 0; k < seq.size(); ++k) {
        const BlasNode& n = nodes[seq[k]];
        const BlasNode& l = nodes[n.left_first];
        const BlasNode& r = nodes[n.left_first + 1];
        int lr = l.count ? l.left_first : dev[n.left_first];
        int rr = r.count ? r.left_first : dev[n.left_first + 1];
        m.nodes[k] = make_node(box(l), lr, l.count, box(r), rr, r.count);
    }
    m.root = 0;
}

void build_blas(HostMesh& m) {
    const int N = m.ntris();
    Builder b;
    b.pos = m.pos.data();
    b.cen.resize(N);
    for (int t = 0; t < N; ++t) {
        V3 a = b.vert(t, 0), c = b.vert(t, 1), d = b.vert(t, 2);
        V3 s = {a.x + c.x, a.y + c.y, a.z + c.z};
        s = {s.x + d.x, s.y + d.y, s.z + d.z};
        b.cen[t] = {s.x * 0.3333f, s.y * 0.3333f, s.z * 0.3333f};
    }
    b.idx.resize(N);
    for (int t = 0; t < N; ++t) b.idx[t] = t;
    b.nodes.assign(N > 0 ? 2 * N - 1 : 1, RefNode());
    b.nodes[0].count = (uint32_t)N;
    b.nodes[0].left_first = 0;
    b.bounds(0);
    uint32_t next = 1;
    b.subdivide(0, &next);
    std::vector<BlasNode> nodes(next);
    for (uint32_t k = 0; k < next; ++k) {
        const RefNode& r = b.nodes[k];
        nodes[k] = {r.left_first, (int)r.count, {r.b.lo.x, r.b.lo.y, r.b.lo.z}, {r.b.hi.x, r.b.hi.y, r.b.hi.z}};
    }
    pack_blas(m, nodes, std::move(b.idx));
}

void inverse4(const float* m, float* out) {
    struct F4 { float x, y, z, w; };
    F4 c0 = {m[0], m[1], m[2], m[3]}, c1 = {m[4], m[5], m[6], m[7]};
    F4 c2 = {m[8], m[9], m[10], m[11]}, c3 = {m[12], m[13], m[14], m[15]};
    float s00 = c2.z * c3.w - c3.z * c2.w;
    float s01 = c2.y * c3.w - c3.y * c2.w;
    float s02 = c2.y * c3.z - c3.y * c2.z;
    float s03 = c2.x * c3.w - c3.x * c2.w;
    float s04 = c2.x * c3.z - c3.x * c2.z;
    float s05 = c2.x * c3.y - c3.x * c2.y;
    float det = c0.x * (c1.y * s00 - c1.z * s01 + c1.w * s02) -
                c0.y * (c1.x * s00 - c1.z * s03 + c1.w * s04) +
                c0.z * (c1.x * s01 - c1.y * s03 + c1.w * s05) -
                c0.w * (c1.x * s02 - c1.y * s04 + c1.z * s05);
    if (fabsf(det) < 1e-6f) {
        for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0f : 0.0f;
        return;
    }
    float id = 1.0f / det;
    float r[16];
    r[0] = (c1.y * s00 - c1.z * s01 + c1.w * s02) * id;
    r[1] = -(c0.y * s00 - c0.z * s01 + c0.w * s02) * id;
    r[2] = (c0.y * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.y * c3.w - c1.w * c3.y) + c0.w * (c1.y * c3.z - c1.z * c3.y)) * id;
    r[3] = -(c0.y * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.y * c2.w - c1.w * c2.y) + c0.w * (c1.y * c2.z - c1.z * c2.y)) * id;
    r[4] = -(c1.x * s00 - c1.z * s03 + c1.w * s04) * id;
    r[5] = (c0.x * s00 - c0.z * s03 + c0.w * s04) * id;
    r[6] = -(c0.x * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.z - c1.z * c3.x)) * id;
    r[7] = (c0.x * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.z - c1.z * c2.x)) * id;
    r[8] = (c1.x * s01 - c1.y * s03 + c1.w * s05) * id;
    r[9] = -(c0.x * s01 - c0.y * s03 + c0.w * s05) * id;
    r[10] = (c0.x * (c1.y * c3.w - c1.w * c3.y) - c0.y * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.y - c1.y * c3.x)) * id;
    r[11] = -(c0.x * (c1.y * c2.w - c1.w * c2.y) - c0.y * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.y - c1.y * c2.x)) * id;
    r[12] = -(c1.x * s02 - c1.y * s04 + c1.z * s05) * id;
    r[13] = (c0.x * s02 - c0.y * s04 + c0.z * s05) * id;
    r[14] = -(c0.x * (c1.y * c3.z - c1.z * c3.y) - c0.y * (c1.x * c3.z - c1.z * c3.x) + c0.z * (c1.x * c3.y - c1.y * c3.x)) * id;
    r[15] = (c0.x * (c1.y * c2.z - c1.z * c2.y) - c0.y * (c1.x * c2.z - c1.z * c2.x) + c0.z * (c1.x * c2.y - c1.y * c2.x)) * id;
    std::memcpy(out, r, sizeof r);
}

void instance_bounds(const HostMesh& m, const float* M, float* lo, float* hi) {
    Box b;
    for (int i = 0; i < 8; ++i) {
        float x = (i & 1) ? m.hi[0] : m.lo[0], y = (i & 2) ? m.hi[1] : m.lo[1], z = (i & 4) ? m.hi[2] : m.lo[2];
        // Matrix4x4 * (x, y, z, 1) (matrix_maths.cuh:258-267)
        V3 p = {M[0] * x + M[4] * y + M[8] * z + M[12] * 1.0f,
                M[1] * x + M[5] * y + M[9] * z + M[13] * 1.0f,
                M[2] * x + M[6] * y + M[10] * z + M[14] * 1.0f};
        b.grow(p);
    }
    lo[0] = b.lo.x; lo[1] = b.lo.y; lo[2] = b.lo.z;
    hi[0] = b.hi.x; hi[1] = b.hi.y; hi[2] = b.hi.z;
}

std::vector<BvhNode> build_tlas(const std::vector<float>& lo, const std::vector<float>& hi, int n,
                                float* root_lo, float* root_hi, int* root_leaf, int* max_depth) {
    struct TN { Box b; uint32_t lr = 0; int blas = -1; };
    std::vector<TN> tn(2 * (size_t)std::max(n, 1));
    std::vector<int> ids(n);
    int next = 1, left = n;
    for (int i = 0; i < n; ++i) {
        ids[i] = next;
        tn[next].b.lo = {lo[3 * i], lo[3 * i + 1], lo[3 * i + 2]};
        tn[next].b.hi = {hi[3 * i], hi[3 * i + 1], hi[3 * i + 2]};
        tn[next].blas = i;
        tn[next++].lr = 0;
    }
    auto best_match = [&](int cnt, int A) {
        float smallest = INFINITY;
        int bestB = -1;
        for (int B = 0; B < cnt; ++B) {
            if (B == A) continue;
            V3 mx = vmax(tn[ids[A]].b.hi, tn[ids[B]].b.hi), mn = vmin(tn[ids[A]].b.lo, tn[ids[B]].b.lo);
            V3 e = {mx.x - mn.x, mx.y - mn.y, mx.z - mn.z};
            float sa = e.x * e.y + e.y * e.z + e.z * e.x;
            if (sa < smallest) { smallest = sa; bestB = B; }
        }
        return bestB;
    };
    int A = 0, B = best_match(left, A);
    while (left > 1) {
        int C = best_match(left, B);
        if (A == C) {
            int na = ids[A], nb = ids[B];
            TN& nn = tn[next];
            nn.lr = (uint32_t)(na + (nb << 16));
            nn.b.lo = vmin(tn[na].b.lo, tn[nb].b.lo);
            nn.b.hi = vmax(tn[na].b.hi, tn[nb].b.hi);
            ids[A] = next++;
            ids[B] = ids[left - 1];
            B = best_match(--left, A);
        } else {
            A = B;
            B = C;
        }
    }
    tn[0] = tn[ids[A]];
    root_lo[0] = tn[0].b.lo.x; root_lo[1] = tn[0].b.lo.y; root_lo[2] = tn[0].b.lo.z;
    root_hi[0] = tn[0].b.hi.x; root_hi[1] = tn[0].b.hi.y; root_hi[2] = tn[0].b.hi.z;
    std::vector<BvhNode> out;
    *max_depth = 1;
    if (tn[0].lr == 0) {
        *root_leaf = 1;
        return out;
    }
    *root_leaf = 0;
    std::vector<int> dev(next, -1);
    std::vector<std::pair<int, int>> stack;
    std::vector<int> order;
    stack.push_back({0, 1});
    while (!stack.empty()) {
        auto [ni, dep] = stack.back();
        stack.pop_back();
        *max_depth = std::max(*max_depth, dep);
        dev[ni] = (int)order.size();
        order.push_back(ni);
        int i1 = tn[ni].lr & 0xFFFF, i2 = (tn[ni].lr >> 16) & 0xFFFF;
        if (tn[i2].lr != 0) stack.push_back({i2, dep + 1});
        if (tn[i1].lr != 0) stack.push_back({i1, dep + 1});
    }
    out.resize(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        const TN& t = tn[order[k]];
        int i1 = t.lr & 0xFFFF, i2 = (t.lr >> 16) & 0xFFFF;
        const TN &a = tn[i1], &b2 = tn[i2];
        int r1 = a.lr ? dev[i1] : a.blas, r2 = b2.lr ? dev[i2] : b2.blas;
        out[k] = make_node(a.b, r1, a.lr ? 0 : 1, b2.b, r2, b2.lr ? 0 : 1);
    }
    return out;
}

void tri_normal_area(const float* p, const float* n, float* gn, float* area) {
    V3 p0 = {p[0], p[1], p[2]}, p1 = {p[3], p[4], p[5]}, p2 = {p[6], p[7], p[8]};
    V3 e0 = {p1.x - p0.x, p1.y - p0.y, p1.z - p0.z}, e1 = {p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
    V3 g = {e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x};
    V3 s = {n[0] + n[3], n[1] + n[4], n[2] + n[5]};
    s = {s.x + n[6], s.y + n[7], s.z + n[8]};
    V3 avg = {s.x / 3.f, s.y / 3.f, s.z / 3.f};
    float d = g.x * avg.x + g.y * avg.y + g.z * avg.z;
    V3 o = (d < 0.0f) ? V3{-g.x, -g.y, -g.z} : g;
    float inv = 1.0f / sqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
    gn[0] = o.x * inv; gn[1] = o.y * inv; gn[2] = o.z * inv;
    *area = 0.5f * sqrtf(g.x * g.x + g.y * g.y + g.z * g.z);
}

}  // namespace kpt
