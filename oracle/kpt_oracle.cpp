// kpt_oracle.cpp -- CPU restatement of the KittlesPT path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the parity tests,
// the smoke check and the CPU baseline of the benchmark compare the CUDA
// library against.  Nothing in the product (kittlespt_gb300/) links or calls
// it.  It restates the reference algorithm in FP32 with the reference's
// operation order; every function cites the reference file:line it follows
// (paths relative to the reference repository, KittlesPT/src/...).
//
// Floating point model: IEEE single precision, no contraction
// (-ffp-contract=off), no fast-math.  fminf/fmaxf are the IEEE
// (NaN-suppressing) C functions, min(float,float) is fminf and rsqrtf(x) is
// 1/sqrtf(x): this is what the reference's host and device code resolve to
// under nvcc, where helper_math's host fallbacks are compiled out.  Where the
// reference writes a double literal inside a float expression (GGX D, Yxy ->
// XYZ) the expression is evaluated in double as C++ requires.
//
// Order of RNG draws: the reference writes three calls whose argument
// evaluation order C++ leaves unspecified.  `rng_order` is a bit mask, a set
// bit meaning right to left: 1 = the pair of get2D (samplers.cuh:37-40),
// 2 = the sun-disc offset (integrator.cuh:155), 4 = the BSDF sample's two
// pairs (integrator.cuh:382).  The reference's GPU build evaluates them as
// 0, its host build (g++) as 7.

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// vector maths (semantics of maths/vector_types_extension.cuh)

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

static inline f2 F2(float x, float y) { return {x, y}; }
static inline f3 F3(float x, float y, float z) { return {x, y, z}; }
static inline f3 F3(float s) { return {s, s, s}; }
static inline f4 F4(float x, float y, float z, float w) { return {x, y, z, w}; }
static inline f4 F4(f3 a, float w) { return {a.x, a.y, a.z, w}; }
static inline f3 xyz(f4 a) { return {a.x, a.y, a.z}; }

static inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
static inline f3 operator*(f3 a, float b) { return {a.x * b, a.y * b, a.z * b}; }
static inline f3 operator*(float b, f3 a) { return {b * a.x, b * a.y, b * a.z}; }
static inline f3 operator/(f3 a, float b) { return {a.x / b, a.y / b, a.z / b}; }
static inline f3 operator/(float b, f3 a) { return {b / a.x, b / a.y, b / a.z}; }
static inline f3 operator+(f3 a, float b) { return {a.x + b, a.y + b, a.z + b}; }
static inline f3 operator-(f3 a, float b) { return {a.x - b, a.y - b, a.z - b}; }
static inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
static inline f2 operator+(f2 a, f2 b) { return {a.x + b.x, a.y + b.y}; }
static inline f2 operator*(float b, f2 a) { return {b * a.x, b * a.y}; }
static inline f4 operator+(f4 a, f4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
static inline f4 operator-(f4 a, f4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
static inline f4 operator*(float b, f4 a) { return {b * a.x, b * a.y, b * a.z, b * a.w}; }
static inline f4 operator*(f4 a, float b) { return {a.x * b, a.y * b, a.z * b, a.w * b}; }

static inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float length(f3 v) { return sqrtf(dot(v, v)); }
static inline float rsqrt_(float x) { return 1.0f / sqrtf(x); }
static inline f3 normalize(f3 v) { float inv = rsqrt_(dot(v, v)); return v * inv; }
static inline f3 fmin3(f3 a, f3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
static inline f3 fmax3(f3 a, f3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
static inline float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
static inline float saturate(float v) { return clampf(v, 0.0f, 1.0f); }
static inline float lerpf(float a, float b, float t) { return a + t * (b - a); }
static inline f4 lerp4(f4 a, f4 b, float t) { return a + t * (b - a); }
static inline f3 reflect(f3 i, f3 n) { return i - 2.0f * n * dot(n, i); }
static inline float Sqr(float v) { return v * v; }
static inline float pow5(float v) { return v * v * v * v * v; }
static inline float AbsDot(f3 a, f3 b) { return fabsf(dot(a, b)); }
static inline float distance3(f3 a, f3 b) { return length(a - b); }
static inline bool nonzero(f3 v) { return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f; }
static inline float smoothstepf(float a, float b, float x) {
    float y = clampf((x - a) / (b - a), 0.0f, 1.0f);
    return y * y * (3.0f - (2.0f * y));
}

static const float PI = 3.14159265358979323846f;
static const float INV_PI = 0.31830988618379067154f;
static const float INV_UINT32MAX = 1.0f / float(UINT32_MAX);
static const float INV_255 = 0.00392156862f;
static const float TRI_EPS = 1.0e-5f;     // maths/constants.cuh:20
static const float HIT_EPS = 0.001f;      // maths/constants.cuh:21

// ---------------------------------------------------------------------------
// matrices, column-major (maths/matrix_maths.cuh:13-396)

struct M3 { f3 c[3]; };
struct M4 { f4 c[4]; };

static inline f3 mul(const M3& m, f3 v) {  // matrix_maths.cuh:91-99
    return {m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z,
            m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z};
}
static inline M3 transpose(const M3& m) {  // matrix_maths.cuh:126-132
    M3 r;
    r.c[0] = {m.c[0].x, m.c[1].x, m.c[2].x};
    r.c[1] = {m.c[0].y, m.c[1].y, m.c[2].y};
    r.c[2] = {m.c[0].z, m.c[1].z, m.c[2].z};
    return r;
}
static inline f4 mul(const M4& m, f4 v) {  // matrix_maths.cuh:258-267
    return {m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w,
            m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w,
            m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w};
}
static M4 identity4() {
    M4 m;
    m.c[0] = {1, 0, 0, 0}; m.c[1] = {0, 1, 0, 0}; m.c[2] = {0, 0, 1, 0}; m.c[3] = {0, 0, 0, 1};
    return m;
}
// Closed-form adjugate inverse, identity when |det| < 1e-6
// (matrix_maths.cuh:304-354).
static M4 inverse(const M4& m) {
    const f4 &c0 = m.c[0], &c1 = m.c[1], &c2 = m.c[2], &c3 = m.c[3];
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
    if (fabsf(det) < 1e-6f) return identity4();
    float id = 1.0f / det;
    M4 r;
    r.c[0].x = (c1.y * s00 - c1.z * s01 + c1.w * s02) * id;
    r.c[0].y = -(c0.y * s00 - c0.z * s01 + c0.w * s02) * id;
    r.c[0].z = (c0.y * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.y * c3.w - c1.w * c3.y) + c0.w * (c1.y * c3.z - c1.z * c3.y)) * id;
    r.c[0].w = -(c0.y * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.y * c2.w - c1.w * c2.y) + c0.w * (c1.y * c2.z - c1.z * c2.y)) * id;
    r.c[1].x = -(c1.x * s00 - c1.z * s03 + c1.w * s04) * id;
    r.c[1].y = (c0.x * s00 - c0.z * s03 + c0.w * s04) * id;
    r.c[1].z = -(c0.x * (c1.z * c3.w - c1.w * c3.z) - c0.z * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.z - c1.z * c3.x)) * id;
    r.c[1].w = (c0.x * (c1.z * c2.w - c1.w * c2.z) - c0.z * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.z - c1.z * c2.x)) * id;
    r.c[2].x = (c1.x * s01 - c1.y * s03 + c1.w * s05) * id;
    r.c[2].y = -(c0.x * s01 - c0.y * s03 + c0.w * s05) * id;
    r.c[2].z = (c0.x * (c1.y * c3.w - c1.w * c3.y) - c0.y * (c1.x * c3.w - c1.w * c3.x) + c0.w * (c1.x * c3.y - c1.y * c3.x)) * id;
    r.c[2].w = -(c0.x * (c1.y * c2.w - c1.w * c2.y) - c0.y * (c1.x * c2.w - c1.w * c2.x) + c0.w * (c1.x * c2.y - c1.y * c2.x)) * id;
    r.c[3].x = -(c1.x * s02 - c1.y * s04 + c1.z * s05) * id;
    r.c[3].y = (c0.x * s02 - c0.y * s04 + c0.z * s05) * id;
    r.c[3].z = -(c0.x * (c1.y * c3.z - c1.z * c3.y) - c0.y * (c1.x * c3.z - c1.z * c3.x) + c0.z * (c1.x * c3.y - c1.y * c3.x)) * id;
    r.c[3].w = (c0.x * (c1.y * c2.z - c1.z * c2.y) - c0.y * (c1.x * c2.z - c1.z * c2.x) + c0.z * (c1.x * c2.y - c1.y * c2.x)) * id;
    return r;
}
static M4 m4_from(const float* colmajor) {
    M4 m;
    for (int c = 0; c < 4; ++c)
        m.c[c] = {colmajor[4 * c + 0], colmajor[4 * c + 1], colmajor[4 * c + 2], colmajor[4 * c + 3]};
    return m;
}
// Frisvad orthonormal basis, columns (t, b, n) (matrix_maths.cuh:375-396).
static M3 onb_frisvad(f3 n) {
    M3 r;
    f3 c0, c2;
    if (n.z < -0.999805696f) {
        c0 = {0.0f, -1.0f, 0.0f};
        c2 = {-1.0f, 0.0f, 0.0f};
    } else {
        float a = 1.0f / (1.0f + n.z);
        float b = -n.x * n.y * a;
        c0 = {1.0f - n.x * n.x * a, b, -n.x};
        c2 = {b, 1.0f - n.y * n.y * a, -n.y};
    }
    r.c[0] = c0; r.c[1] = c2; r.c[2] = n;
    return r;
}

// ---------------------------------------------------------------------------
// RNG (shaders/samplers.cuh:9-48)

static inline uint32_t pcg_hash(uint32_t input) {  // samplers.cuh:12-17
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
struct Sampler {
    uint32_t seed;
    int order;  // bit 0: the pair's argument evaluation order (0 left to right)
    // samplers.cuh:24-29: seed = pixel index scaled by max(frame, 1) in float
    void init(int px, int py, int width, int index, int dimension = 0) {
        seed = (uint32_t)(px + py * width);
        float f = (index == 0) ? 1.0f : (float)index;
        seed = (uint32_t)((float)seed * f);
        seed += (uint32_t)dimension;
    }
    float get1D() {  // samplers.cuh:31-35
        seed = pcg_hash(seed);
        return (float)seed * INV_UINT32MAX;
    }
    f2 get2D() {  // samplers.cuh:37-40
        if ((order & 1) == 0) { float a = get1D(); float b = get1D(); return {a, b}; }
        float b = get1D(); float a = get1D(); return {a, b};
    }
};

// ---------------------------------------------------------------------------
// rays and bounds (shaders/ray.cuh:6-33, maths/bounds.cuh:38-57)

struct Ray {
    f3 o, d, inv;
};
static inline Ray make_ray(f3 o, f3 d) { return {o, d, 1.0f / d}; }
static inline Ray transform_ray(const Ray& r, const M4& m) {  // ray.cuh:28-31
    return make_ray(xyz(mul(m, F4(r.o, 1.0f))), xyz(mul(m, F4(r.d, 0.0f))));
}
static inline f3 point_at(const Ray& r, float t) { return r.o + (t * r.d); }

struct Bounds {
    f3 pmin = {FLT_MAX, FLT_MAX, FLT_MAX};
    f3 pmax = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(f3 p) { pmin = fmin3(pmin, p); pmax = fmax3(pmax, p); }
    void grow(const Bounds& b) { grow(b.pmax); grow(b.pmin); }  // bounds.cuh:22-26
    float area() const {  // bounds.cuh:16-20
        f3 d = pmax - pmin;
        return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
    }
};
// Slab test (bounds.cuh:38-57).
static inline bool slab(const Bounds& b, const Ray& r, float tmin_, float tmax_, float* h0, float* h1) {
    f3 t0 = (b.pmin - r.o) * r.inv;
    f3 t1 = (b.pmax - r.o) * r.inv;
    f3 tmn = fmin3(t0, t1), tmx = fmax3(t0, t1);
    float tenter = fmaxf(fmaxf(tmn.x, tmn.y), tmn.z);
    float texit = fminf(fminf(tmx.x, tmx.y), tmx.z);
    bool hit = (tenter <= texit) && (texit >= tmin_) && (tenter <= tmax_);
    if (hit) { *h0 = tenter; *h1 = texit; }
    return hit;
}

// ---------------------------------------------------------------------------
// scene records (reference layouts, one triangle copy per mesh)

struct Tri {       // shaders/triangle.cuh:38-130
    f3 p[3], n[3];
    f2 uv[3];
    f3 local_gn;
    int material, light, mesh;
};
struct Node {      // shaders/blas.cuh:9-35
    int left_first = -1;
    uint32_t count = 0;
    Bounds b;
};
struct Blas {      // shaders/blas.cuh:193-355
    Bounds b, original;
    int64_t root = -1;
    int mesh_id = -1;
    M4 inv_model;
};
struct TlasNode {  // shaders/blas.cuh:357-386
    Bounds b;
    uint32_t lr = 0;
    int blas = -1;
};
struct Mesh {      // shaders/triangle.cuh:132-154
    M4 inv_model;
    int blas = -1;
    uint32_t count = 0;
    int offset = -1;
};
struct Material {  // shaders/material.cuh:91-145; same layout as the C-ABI record
    float albedo[3]; float metallic, roughness, transmission, ior;
    float emission[3]; float emission_scale, normal_scale;
    int albedo_tex, orm_tex, transmission_tex, emission_tex, normal_tex, pad;
};
struct Light {     // shaders/light.cuh:70-94
    int prim;
    f3 emission;
    float nits, area;
};
struct Texture { int w, h, ch, offset; };  // shaders/texture.cuh:25-72

struct Env {       // procedural environment + Nishita coefficients (C-ABI layout)
    float sun_angular_diameter, sun_phi, sun_theta, sun_emission_factor;
    float rayleigh[3]; float mie, mie_absorption, rayleigh_height, mie_height, pad;
};
struct Settings {
    int max_depth, bloom, karis, auto_exposure;
    float bloom_final_blend, bloom_internal_blend, frame_delta_ms, pad;
};
struct Exposure {
    float aperture, iso, shutter, ev_comp, white_ev, black_ev;
    float max_iso, min_iso, max_shutter, min_shutter, pad0, pad1;
};

struct Counters {  // algorithmic work, summed per call
    int64_t box_tests = 0, tri_tests = 0, inst_xforms = 0, sky_evals = 0,
            hits = 0, rays = 0, max_stack = 0, stack_overflow = 0;
    void add(const Counters& o) {
        box_tests += o.box_tests; tri_tests += o.tri_tests; inst_xforms += o.inst_xforms;
        sky_evals += o.sky_evals; hits += o.hits; rays += o.rays;
        max_stack = std::max(max_stack, o.max_stack); stack_overflow += o.stack_overflow;
    }
};

struct Scene {
    std::vector<Tri> tris;
    std::vector<Node> nodes;
    std::vector<int32_t> tri_index;
    std::vector<Blas> blas;
    std::vector<TlasNode> tlas_nodes;
    Bounds tlas_bounds;
    int tlas_root = -1;
    std::vector<Mesh> meshes;
    std::vector<Material> materials;
    std::vector<Light> lights;
    std::vector<Texture> textures;
    std::vector<uint8_t> pixels;
    std::vector<M4> mesh_model;     // inverse of the mesh inverse (per-hit in the reference)
};

// ---------------------------------------------------------------------------
// BLAS builder: binned SAH, 8 bins on each axis, leaves of <= 8 triangles
// (as_builder.cuh:11-261).

struct BlasBuilder {
    Scene& s;
    std::vector<f3> centroid;
    int offset = 0;
    uint32_t count = 0;
    explicit BlasBuilder(Scene& sc) : s(sc) {}

    static float comp(f3 v, int idx) { return (idx == 0) ? v.x : (idx == 1) ? v.y : v.z; }

    void update_bounds(uint32_t ni) {  // as_builder.cuh:49-62
        Node& n = s.nodes[ni];
        n.b.pmin = F3(FLT_MAX);
        n.b.pmax = F3(-FLT_MAX);
        for (uint32_t i = 0; i < n.count; ++i) {
            const Tri& t = s.tris[s.tri_index[n.left_first + i]];
            n.b.grow(t.p[0]); n.b.grow(t.p[1]); n.b.grow(t.p[2]);
        }
    }
    float best_split(const Node& n, int* axis, float* pos) {  // as_builder.cuh:110-179
        const int BINS = 8;
        float best = INFINITY;
        for (int a = 0; a < 3; ++a) {
            float bmin = INFINITY, bmax = -INFINITY;
            for (uint32_t i = 0; i < n.count; ++i) {
                f3 c = centroid[s.tri_index[n.left_first + i]];
                bmin = fminf(bmin, comp(c, a));
                bmax = fmaxf(bmax, comp(c, a));
            }
            if (bmin == bmax) continue;
            Bounds bin_b[BINS];
            uint32_t bin_n[BINS] = {0};
            float scale = (float)BINS / (bmax - bmin);
            for (uint32_t i = 0; i < n.count; ++i) {
                int ti = s.tri_index[n.left_first + i];
                int bi = std::min(BINS - 1, (int32_t)((comp(centroid[ti], a) - bmin) * scale));
                bin_n[bi]++;
                const Tri& t = s.tris[ti];
                bin_b[bi].grow(t.p[0]); bin_b[bi].grow(t.p[1]); bin_b[bi].grow(t.p[2]);
            }
            const int P = BINS - 1;
            float la[P], ra[P];
            int32_t lc[P], rc[P];
            Bounds lb, rb;
            int32_t ls = 0, rs = 0;
            for (int i = 0; i < P; ++i) {
                ls += bin_n[i]; lc[i] = ls; lb.grow(bin_b[i]); la[i] = lb.area();
                rs += bin_n[P - i]; rc[P - 1 - i] = rs; rb.grow(bin_b[P - i]); ra[P - 1 - i] = rb.area();
            }
            scale = (bmax - bmin) / (float)BINS;
            for (int i = 0; i < P; ++i) {
                float cost = lc[i] * la[i] + rc[i] * ra[i];
                if (cost < best) { *axis = a; *pos = bmin + scale * (i + 1); best = cost; }
            }
        }
        return best;
    }
    void subdivide(uint32_t ni, uint32_t* next) {  // as_builder.cuh:181-233
        Node& p = s.nodes[ni];
        if (p.count <= 8) return;   // the split search before this test has no effect
        int axis = -1;
        float pos = 0;
        best_split(p, &axis, &pos);
        int32_t i = p.left_first, j = i + (int32_t)p.count - 1;
        while (i <= j) {
            if (comp(centroid[s.tri_index[i]], axis) < pos) i++;
            else std::swap(s.tri_index[i], s.tri_index[j--]);
        }
        int32_t split = i;
        Node l, r;
        l.count = (uint32_t)(split - p.left_first);
        if (l.count == 0 || l.count == p.count) return;
        int32_t lid = (int32_t)(*next)++;
        int32_t rid = (int32_t)(*next)++;
        l.left_first = p.left_first;
        r.left_first = split;
        r.count = p.count - l.count;
        p.count = 0;
        p.left_first = lid;
        s.nodes[lid] = l;
        s.nodes[rid] = r;
        update_bounds(lid);
        update_bounds(rid);
        subdivide(lid, next);
        subdivide(rid, next);
    }
    Blas build(const Mesh& m, int mesh_id) {  // as_builder.cuh:26-35, 235-261
        offset = m.offset;
        count = m.count;
        for (uint32_t i = 0; i < count; ++i) {
            const Tri& t = s.tris[offset + i];
            centroid.push_back((t.p[0] + t.p[1] + t.p[2]) * 0.3333f);
        }
        int32_t root = (int32_t)s.nodes.size();
        s.nodes.resize(s.nodes.size() + (2 * count - 1));
        size_t base = s.tri_index.size();
        s.tri_index.resize(base + count);
        for (uint32_t i = 0; i < count; ++i) s.tri_index[base + i] = offset + (int32_t)i;
        Blas b;
        b.root = root;
        Node& rn = s.nodes[root];
        rn.count = count;
        rn.left_first = offset;
        update_bounds(root);
        b.b = s.nodes[root].b;
        uint32_t next = root + 1;
        subdivide(root, &next);
        b.original = b.b;
        b.inv_model = m.inv_model;
        b.mesh_id = mesh_id;
        return b;
    }
};

// BLAS2::setTransform (blas.cuh:338-348): inverse and world bounds of the
// 8 transformed corners of the object-space bounds.
static void blas_set_transform(Blas& b, const M4& model) {
    b.inv_model = inverse(model);
    f3 mn = b.original.pmin, mx = b.original.pmax;
    b.b = Bounds();
    for (int i = 0; i < 8; ++i)
        b.b.grow(xyz(mul(model, F4((i & 1) ? mx.x : mn.x, (i & 2) ? mx.y : mn.y, (i & 4) ? mx.z : mn.z, 1.0f))));
}

// TLAS: agglomerative clustering on half surface area (as_builder.cuh:312-392).
static int tlas_best_match(const Scene& s, const std::vector<int32_t>& ids, int32_t n, int32_t A) {
    float smallest = INFINITY;
    int32_t bestB = -1;
    for (int32_t B = 0; B < n; ++B) {
        if (B == A) continue;
        f3 bmax = fmax3(s.tlas_nodes[ids[A]].b.pmax, s.tlas_nodes[ids[B]].b.pmax);
        f3 bmin = fmin3(s.tlas_nodes[ids[A]].b.pmin, s.tlas_nodes[ids[B]].b.pmin);
        f3 e = bmax - bmin;
        float sa = e.x * e.y + e.y * e.z + e.z * e.x;
        if (sa < smallest) { smallest = sa; bestB = B; }
    }
    return bestB;
}
static void build_tlas(Scene& s) {
    uint32_t n = (uint32_t)s.blas.size();
    s.tlas_nodes.assign(2 * n, TlasNode());
    std::vector<int32_t> ids(n);
    int32_t next = 1, left = (int32_t)n;
    for (uint32_t i = 0; i < n; ++i) {
        ids[i] = next;
        s.tlas_nodes[next].b = s.blas[i].b;
        s.tlas_nodes[next].blas = (int)i;
        s.tlas_nodes[next++].lr = 0u;
    }
    int A = 0, B = tlas_best_match(s, ids, left, A);
    while (left > 1) {
        int C = tlas_best_match(s, ids, left, B);
        if (A == C) {
            int32_t na = ids[A], nb = ids[B];
            TlasNode& nn = s.tlas_nodes[next];
            nn.lr = (uint32_t)(na + (nb << 16));
            nn.b.pmin = fmin3(s.tlas_nodes[na].b.pmin, s.tlas_nodes[nb].b.pmin);
            nn.b.pmax = fmax3(s.tlas_nodes[na].b.pmax, s.tlas_nodes[nb].b.pmax);
            ids[A] = next++;
            ids[B] = ids[left - 1];
            B = tlas_best_match(s, ids, --left, A);
        } else {
            A = B; B = C;
        }
    }
    s.tlas_root = 0;
    s.tlas_nodes[0] = s.tlas_nodes[ids[A]];
    s.tlas_bounds = s.tlas_nodes[0].b;
    s.tlas_nodes.resize(next);
}

// ---------------------------------------------------------------------------
// traversal

struct Hit {
    float t = INFINITY;
    int prim = -1, inst = -1;
    f3 bary = {0, 0, 0};
};

// Moeller-Trumbore with the reference's absolute epsilons (triangle.cuh:66-102).
static inline void tri_intersect(const Tri& tr, const Ray& r, float tmin, float tmax, Hit* h) {
    h->t = INFINITY;
    f3 e1 = tr.p[1] - tr.p[0];
    f3 e2 = tr.p[2] - tr.p[0];
    f3 pv = cross(r.d, e2);
    float det = dot(e1, pv);
    if (det > -TRI_EPS && det < TRI_EPS) return;
    float inv = 1.0f / det;
    f3 tv = r.o - tr.p[0];
    float u = inv * dot(tv, pv);
    if (u < 0.0f || u > 1.0f) return;
    f3 qv = cross(tv, e1);
    float v = inv * dot(r.d, qv);
    if (v < 0.0f || u + v > 1.0f) return;
    float t = inv * dot(e2, qv);
    if (t > TRI_EPS && t < tmax && t > tmin) {
        h->t = t;
        h->bary = {1.0f - u - v, u, v};
    }
}

static const int STACK = 64;       // the reference stops at 16 (blas.cuh:185, tlas.cuh:10)
static const int REF_STACK = 16;

// BLAS2::intersect (blas.cuh:261-336).
static Hit blas_intersect(const Scene& s, const Blas& b, const Ray& ray, float tmin, float tmax, Counters& c) {
    if (b.root < 0) return Hit();
    c.inst_xforms++;
    Ray r = transform_ray(ray, b.inv_model);
    uint32_t st[STACK];
    int sp = 0;
    st[sp++] = (uint32_t)b.root;
    Hit closest, h;
    while (sp > 0) {
        const Node& n = s.nodes[st[--sp]];
        if (n.count == 0) {
            float h1 = INFINITY, h2 = INFINITY, x1 = 0, x2 = 0;
            const Node& c1 = s.nodes[n.left_first];
            const Node& c2 = s.nodes[n.left_first + 1];
            bool hit1 = slab(c1.b, r, tmin, tmax, &h1, &x1);
            bool hit2 = slab(c2.b, r, tmin, tmax, &h2, &x2);
            c.box_tests += 2;
            if (h1 > h2) {
                if (hit1 && h1 < closest.t) st[sp++] = (uint32_t)n.left_first;
                if (hit2 && h2 < closest.t) st[sp++] = (uint32_t)n.left_first + 1;
            } else {
                if (hit2 && h2 < closest.t) st[sp++] = (uint32_t)n.left_first + 1;
                if (hit1 && h1 < closest.t) st[sp++] = (uint32_t)n.left_first;
            }
            if (sp > c.max_stack) c.max_stack = sp;
            if (sp > REF_STACK) c.stack_overflow++;
        } else {
            for (uint32_t i = 0; i < n.count; ++i) {
                int32_t pi = s.tri_index[n.left_first + i];
                tri_intersect(s.tris[pi], r, tmin, tmax, &h);
                c.tri_tests++;
                if (h.t < INFINITY && h.t < tmax && h.t > tmin && h.t < closest.t) {
                    closest = h;
                    closest.prim = pi;
                    closest.inst = b.mesh_id;
                    tmax = closest.t;
                }
            }
        }
    }
    return closest;
}

// BLAS2::intersectP (blas.cuh:198-259).
static bool blas_occluded(const Scene& s, const Blas& b, const Ray& ray, float tmin, float tmax, Counters& c) {
    if (b.root < 0) return false;
    c.inst_xforms++;
    Ray r = transform_ray(ray, b.inv_model);
    uint32_t st[STACK];
    int sp = 0;
    st[sp++] = (uint32_t)b.root;
    Hit h;
    while (sp > 0) {
        const Node& n = s.nodes[st[--sp]];
        if (n.count == 0) {
            float h1 = INFINITY, h2 = INFINITY, x1 = 0, x2 = 0;
            bool hit1 = slab(s.nodes[n.left_first].b, r, tmin, tmax, &h1, &x1);
            bool hit2 = slab(s.nodes[n.left_first + 1].b, r, tmin, tmax, &h2, &x2);
            c.box_tests += 2;
            if (hit1) st[sp++] = (uint32_t)n.left_first;
            if (hit2) st[sp++] = (uint32_t)n.left_first + 1;
            if (sp > c.max_stack) c.max_stack = sp;
            if (sp > REF_STACK) c.stack_overflow++;
        } else {
            for (uint32_t i = 0; i < n.count; ++i) {
                tri_intersect(s.tris[s.tri_index[n.left_first + i]], r, tmin, tmax, &h);
                c.tri_tests++;
                if (h.t < INFINITY && h.t < tmax && h.t > tmin) return true;
            }
        }
    }
    return false;
}

// TLAS::intersect (tlas.cu:60-125).
static Hit tlas_intersect(const Scene& s, const Ray& r, float tmin, float tmax, Counters& c) {
    c.rays++;
    if (s.tlas_root < 0) return Hit();
    float h1 = INFINITY, h2 = INFINITY;
    c.box_tests++;
    if (!slab(s.tlas_bounds, r, tmin, tmax, &h1, &h2)) return Hit();
    h1 = INFINITY; h2 = INFINITY;
    int32_t st[STACK];
    int sp = 0;
    st[sp++] = s.tlas_root;
    Hit closest;
    while (sp > 0) {
        const TlasNode& n = s.tlas_nodes[st[--sp]];
        if (n.lr != 0) {
            uint32_t i1 = n.lr & 0xFFFF, i2 = (n.lr >> 16) & 0xFFFF;
            float x1 = 0, x2 = 0;
            bool hit1 = slab(s.tlas_nodes[i1].b, r, tmin, tmax, &h1, &x1);
            bool hit2 = slab(s.tlas_nodes[i2].b, r, tmin, tmax, &h2, &x2);
            c.box_tests += 2;
            if (h1 > h2) {
                if (hit1 && h1 < closest.t) st[sp++] = (int32_t)i1;
                if (hit2 && h2 < closest.t) st[sp++] = (int32_t)i2;
            } else {
                if (hit2 && h2 < closest.t) st[sp++] = (int32_t)i2;
                if (hit1 && h1 < closest.t) st[sp++] = (int32_t)i1;
            }
        } else {
            Hit h = blas_intersect(s, s.blas[n.blas], r, tmin, tmax, c);
            if (h.t < closest.t) closest = h;
        }
    }
    if (closest.prim >= 0) c.hits++;
    return closest;
}

// TLAS::intersectP (tlas.cu:8-58).
static bool tlas_occluded(const Scene& s, const Ray& r, float tmin, float tmax, Counters& c) {
    c.rays++;
    if (s.tlas_root < 0) return false;
    float h1 = INFINITY, h2 = INFINITY;
    c.box_tests++;
    if (!slab(s.tlas_bounds, r, tmin, tmax, &h1, &h2)) return false;
    int32_t st[STACK];
    int sp = 0;
    st[sp++] = s.tlas_root;
    while (sp > 0) {
        const TlasNode& n = s.tlas_nodes[st[--sp]];
        if (n.lr != 0) {
            uint32_t i1 = n.lr & 0xFFFF, i2 = (n.lr >> 16) & 0xFFFF;
            float x1 = 0, x2 = 0;
            bool hit1 = slab(s.tlas_nodes[i1].b, r, tmin, tmax, &h1, &x1);
            bool hit2 = slab(s.tlas_nodes[i2].b, r, tmin, tmax, &h2, &x2);
            c.box_tests += 2;
            if (hit1) st[sp++] = (int32_t)i1;
            if (hit2) st[sp++] = (int32_t)i2;
        } else if (blas_occluded(s, s.blas[n.blas], r, tmin, tmax, c)) {
            return true;
        }
    }
    return false;
}

// Brute force closest hit over every mesh and triangle (the reference's
// INTERSECT_DEBUG path, integrator.cuh:69-94).
static Hit brute_intersect(const Scene& s, const Ray& ray, float tmin, float tmax) {
    Hit closest, h;
    for (size_t mi = 0; mi < s.meshes.size(); ++mi) {
        const Mesh& m = s.meshes[mi];
        Ray r = transform_ray(ray, s.blas[m.blas].inv_model);
        for (int p = m.offset; p < m.offset + (int)m.count; ++p) {
            tri_intersect(s.tris[p], r, tmin, tmax, &h);
            if (h.t < INFINITY && h.t < tmax && h.t > tmin && h.t < closest.t) {
                closest = h; closest.prim = p; closest.inst = (int)mi;
            }
        }
    }
    return closest;
}

// ---------------------------------------------------------------------------
// textures (shaders/texture.cuh:34-66), colour helpers (shaders/color.cuh)

static f3 texture_eval(const Scene& s, int tex_id, f2 uv) {
    const Texture& t = s.textures[tex_id];
    if (t.offset < 0 || (size_t)t.offset >= s.pixels.size()) return F3(0.0f);
    size_t px_stride = (size_t)t.ch;
    size_t row_stride = (size_t)t.w * px_stride;
    f2 st = {uv.x - floorf(uv.x), uv.y - floorf(uv.y)};
    int32_t x = (int32_t)(st.x * t.w) % t.w;
    int32_t y = (int32_t)(st.y * t.h) % t.h;
    if (x < 0) x += t.w;
    if (y < 0) y += t.h;
    size_t off = (size_t)y * row_stride + (size_t)x * px_stride;
    if (off + 3 >= s.pixels.size()) return F3(0.0f);
    const uint8_t* p = &s.pixels[(size_t)t.offset + off];
    return {p[0] * INV_255, p[1] * INV_255, p[2] * INV_255};
}
static float srgb_decode(float v) {  // color.cuh:428-433
    return (v <= 0.04045f) ? (v / 12.92f) : powf((v + 0.055f) / (1 + 0.055f), 2.4f);
}
static float srgb_encode(float v) {  // color.cuh:421-426
    return (v <= 0.0031308f) ? (12.92f * v) : ((1 + 0.055f) * powf(v, 1.0f / 2.4f) - 0.055f);
}
static float luminance(f3 c) { return (0.2126f * c.x) + (0.7152f * c.y) + (0.0722f * c.z); }
static f3 clamp_output(f3 v) {  // color.cuh:295-302
    if (std::isnan(v.x) || std::isnan(v.y) || std::isnan(v.z) ||
        std::isinf(v.x) || std::isinf(v.y) || std::isinf(v.z))
        return F3(0.0f);
    return {clampf(v.x, 0.0f, 1.0e8f), clampf(v.y, 0.0f, 1.0e8f), clampf(v.z, 0.0f, 1.0e8f)};
}

// ---------------------------------------------------------------------------
// GGX microfacet model and the unified BSDF (shaders/bsdf.cuh)

struct GGX {
    float alpha = 0.25f;
    bool smooth() const { return alpha < 0.001f; }  // bsdf.cuh:76-78
    float D(f3 wm) const {  // bsdf.cuh:26-37
        float a = alpha;
        if (smooth()) a = fmaxf(a, 1.0e-3f);
        float a2 = Sqr(a);
        float ndh = Sqr(saturate(wm.z));
        float b = (float)((double)ndh * ((double)a2 - 1.0) + 1.0);
        return a2 / (PI * Sqr(b));
    }
    float G(f3 wo, f3 wi) const {  // bsdf.cuh:45-57
        float nv = fmaxf(wo.z, 0.0f);
        float nl = fabsf(wi.z);
        float tv = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nv));
        float tl = sqrtf(Sqr(alpha) + (1.0f - Sqr(alpha)) * Sqr(nl));
        float g1v = (2.0f * nv) / (nv + tv);
        float g1l = (2.0f * nl) / (nl + tl);
        return g1v * g1l;
    }
    // xs (rounding-sensitivity probe only, 1 otherwise) scales the cosine
    // before the inverse cosine
    f3 sample_wm(f2 u, float xs = 1.0f) const {  // bsdf.cuh:59-74
        float a2 = Sqr(alpha);
        float x = sqrtf((1.0f - u.x) / ((a2 - 1.0f) * u.x + 1.0f));
        if (xs != 1.0f) x = fminf(x * xs, 1.0f);
        float theta = acosf(x);
        float phi = 2.0f * PI * u.y;
        f3 wm = {sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta)};
        return normalize(wm);
    }
    void regularize() {  // bsdf.cuh:80-84
        if (alpha < 0.3f) alpha = clampf(2.0f * alpha, 0.1f, 0.3f);
    }
};

enum { ABSORBED = 0, REFLECTED = 2, TRANSMITTED = 4, DIFFUSE = 8, GLOSSY = 16, SPECULAR = 32 };
struct BSDFSample { int scatter = ABSORBED; f3 f = {0, 0, 0}; f3 wi = {0, 0, 0}; float pdf = 0.0f; };

static float fresnel_dielectric(float cos_t, float ior) {  // bsdf.cuh:122-141
    cos_t = clampf(cos_t, -1.0f, 1.0f);
    if (cos_t < 0.0f) { ior = 1.0f / ior; cos_t = -cos_t; }
    float s2 = (1.0f - cos_t * cos_t);
    float s2t = s2 / (ior * ior);
    if (s2t >= 1.0f) return 1.0f;
    float ct = sqrtf(1.0f - s2t);
    float rp = (ior * cos_t - ct) / (ior * cos_t + ct);
    float rs = (cos_t - ior * ct) / (cos_t + ior * ct);
    return (rp * rp + rs * rs) * 0.5f;
}
static f3 fresnel_schlick(float c, f3 F0) {  // bsdf.cuh:144-148
    f3 F = F0 + (F3(1.0f) - F0) * pow5(1.0f - c);
    return {clampf(F.x, 0.0f, 1.0f), clampf(F.y, 0.0f, 1.0f), clampf(F.z, 0.0f, 1.0f)};
}
static float microfacet_brdf(f3 wo, f3 wi, f3 wm, const GGX& g) {  // bsdf.cuh:151-164
    float nv = saturate(wo.z);
    float nl = saturate(wi.z);
    float D = g.D(wm);
    float G = g.G(wo, wi);
    float f = (D * G) / (4.0f * fmaxf(nv, 1.0e-3f) * nl);
    if (wi.z <= 0.0f || dot(wi, wm) <= 0.0f) f = 0.0f;
    return f;
}
static bool refract_(f3 wi, f3 n, float ior, f3* wt) {  // maths/vector_maths.cuh:46-65
    float c = dot(wi, n);
    if (c < 0.0f) { ior = 1.0f / ior; c *= -1.0f; n = n * -1.0f; }
    float s2 = (1.0f - c * c);
    float s2t = s2 / (ior * ior);
    if (s2t >= 1.0f) return false;
    float ct = sqrtf(1.0f - s2t);
    *wt = (-1.0f * wi) / ior + (c / ior - ct) * n;
    return true;
}
static inline bool same_hemi_z(f3 a, f3 b) { return (a.z * b.z) > 0.0f; }  // vector_maths.cuh:71-74 with n = z

struct BSDF {  // UnifiedBSDF, bsdf.cuh:166-624
    GGX ggx;
    M3 basis;
    f3 albedo = {1.0f, 0.0f, 1.0f};
    float roughness = 0.5f, metallic = 0.0f, transmission = 0.0f, ior = 1.45f;
    bool backface = false;

    void regularize() {  // bsdf.cuh:271-276
        if (roughness < 0.3f) roughness = clampf(2.0f * roughness, 0.1f, 0.3f);
        ggx.regularize();
    }
    bool non_specular() const { return !ggx.smooth(); }

    // BxDFs, bsdf.cuh:542-610
    float f_diffuse(f3 wo, f3 wi) const { return ((wo.z * wi.z > 0) ? 1.0f : 0.0f) * INV_PI; }
    float pdf_diffuse(f3, f3 wi) const { return wi.z * INV_PI; }
    f3 f_glossy(f3 wo, f3 wi, f3 wm) const {
        float M = microfacet_brdf(wo, wi, wm, ggx);
        float F = fresnel_dielectric(dot(wo, wm), ior);
        return F3(F * M);
    }
    float pdf_glossy(f3 wo, f3, f3 wm) const {
        float voh = fmaxf(dot(wo, wm), 0.0f);
        float noh = fmaxf(wm.z, 0.0f);
        float D = ggx.D(wm);
        return (D * noh) / (4.0f * voh);
    }
    float pdf_btdf(f3 wo, f3 wi, f3 ht, float eta) const {
        float temp = dot(wi, ht) * eta + dot(wo, ht);
        float dwm = AbsDot(wi, ht) / (temp * temp);
        float noh = fabsf(ht.z);
        float D = ggx.D(ht);
        float F = fresnel_dielectric(AbsDot(wo, ht), eta);
        return (D * noh) * dwm * (1.0f - F);
    }
    f3 f_btdf(f3 wo, f3 wi, f3 ht, float eta) const {
        float temp = dot(wi, ht) * eta + dot(wo, ht);
        float F = fresnel_dielectric(AbsDot(wo, ht), eta);
        float T = ggx.D(ht) * ggx.G(wo, wi) * fabsf(dot(wi, ht) * dot(wo, ht) / (wi.z * wo.z * temp * temp));
        return (albedo * (1.0f - F)) * T;
    }
    // lobes, bsdf.cuh:298-537
    f3 f_opaque(f3 wo, f3 wi) const {
        f3 wm = normalize(wo + wi);
        f3 glossy = f_glossy(wo, wi, wm);
        f3 wd = F3(1.0f) - glossy;
        f3 diffuse = wd * (albedo * f_diffuse(wo, wi));
        return diffuse + glossy;
    }
    float pdf_opaque(f3 wo, f3 wi) const {
        f3 wm = normalize(wo + wi);
        float ps = pdf_glossy(wo, wi, wm);
        float pd = pdf_diffuse(wo, wi);
        return 0.5f * (ps + pd);
    }
    BSDFSample sample_opaque(f3 wo, f2 u, float X, float xs = 1.0f) const {
        BSDFSample bs;
        if (X < 0.5f) {
            f3 wm = ggx.sample_wm(u, xs);
            f3 wi = reflect(-wo, wm);
            f3 f = f_glossy(wo, wi, wm) * 2.0f;
            bs.scatter = GLOSSY | REFLECTED; bs.f = f; bs.wi = wi; bs.pdf = pdf_glossy(wo, wi, wm);
            return bs;
        }
        float phi = 2.0f * PI * u.x;   // sampleCosineWeightedHemisphere, samplers.cuh:88-95
        float ct = sqrtf(u.y);
        float stt = sqrtf(1.0f - u.y);
        f3 wi = {stt * cosf(phi), stt * sinf(phi), ct};
        f3 f = (albedo * f_diffuse(wo, wi)) * 2.0f;
        bs.scatter = DIFFUSE | REFLECTED; bs.f = f; bs.wi = wi; bs.pdf = pdf_diffuse(wo, wi);
        return bs;
    }
    f3 f_conductor(f3 wo, f3 wi) const {
        f3 wm = normalize(wo + wi);
        float nv = clampf(wo.z, 0.0f, 1.0f);
        float nl = clampf(wi.z, 0.0f, 1.0f);
        if (nv == 0.0f || nl == 0.0f) return F3(0.0f);
        float voh = clampf(dot(wo, wm), 0.0f, 1.0f);
        f3 M = F3(0.0f);
        if (nl > 0.0f && voh > 0.0f) {
            f3 F = fresnel_schlick(voh, albedo);
            M = F * microfacet_brdf(wo, wi, wm, ggx);
        }
        return M;
    }
    float pdf_conductor(f3 wo, f3 wi) const { return pdf_glossy(wo, wi, normalize(wo + wi)); }
    BSDFSample sample_conductor(f3 wo, f2 u, float xs = 1.0f) const {
        f3 wm = ggx.sample_wm(u, xs);
        f3 wi = reflect(-wo, wm);
        BSDFSample bs;
        bs.scatter = GLOSSY | REFLECTED; bs.f = f_conductor(wo, wi); bs.wi = wi;
        bs.pdf = pdf_glossy(wo, wi, wm);
        return bs;
    }
    BSDFSample sample_transparent(f3 wo, f2 u, float X, float xs = 1.0f) const {
        bool inside = backface;
        float eta = inside ? (1.0f / ior) : ior;
        f3 ht = ggx.sample_wm(u, xs);
        f3 wi = {0, 0, 0};
        bool tir = !refract_(wo, ht, eta, &wi);
        BSDFSample bs;
        if ((X < 0.5f && !inside) || (tir && inside)) {
            wi = reflect(-wo, ht);
            if (!same_hemi_z(wi, wo)) return bs;
            float M = microfacet_brdf(wo, wi, ht, ggx);
            float F = fresnel_dielectric(dot(wo, ht), eta);
            f3 f = F3(F * M);
            if (!tir) f = f * 2.0f;
            bs.scatter = REFLECTED | GLOSSY; bs.f = f; bs.wi = wi; bs.pdf = pdf_glossy(wo, wi, ht);
            return bs;
        }
        if (tir || same_hemi_z(wi, wo) || wi.z == 0.0f) return bs;
        float pdf = pdf_btdf(wo, wi, ht, eta);
        f3 f = f_btdf(wo, wi, ht, eta);
        if (!inside) f = f * 2.0f;
        bs.scatter = TRANSMITTED | GLOSSY; bs.f = f; bs.wi = wi; bs.pdf = pdf;
        return bs;
    }
    f3 f_transparent(f3 wo, f3 wi) const {
        float co = wo.z, ci = wi.z;
        bool refl = (co * ci) > 0.0f;
        float eta = 1.0f;
        if (!refl) eta = (!backface) ? ior : (1.0f / ior);
        f3 wm = (eta * wi + wo);
        wm = normalize((wm.z > 0) ? wm : -wm);
        if ((dot(wm, wi) * ci < 0.0f) || (dot(wm, wo) * co < 0.0f)) return F3(0.0f);
        float F = fresnel_dielectric(fabsf(dot(wo, wm)), ior);
        float T = 1.0f - F;
        if (refl) return F3(F * microfacet_brdf(wo, wi, wm, ggx));
        float temp = dot(wi, wm) * eta + dot(wo, wm);
        float dwm = fabsf(dot(wi, wm)) * fabsf(dot(wo, wm)) / (temp * temp);
        float Tss = ggx.D(wm) * ggx.G(wo, wi) * dwm / (fabsf(ci * co));
        return (T * albedo) * Tss;
    }
    float pdf_transparent(f3 wo, f3 wi) const {
        float co = wo.z, ci = wi.z;
        bool refl = co * ci > 0.0f;
        float eta = 1.0f;
        if (!refl) eta = (!backface) ? ior : 1.0f / ior;
        f3 wm = (eta * wi + wo);
        wm = normalize((wm.z > 0) ? wm : -wm);
        if (dot(wm, wi) * ci < 0.0f || dot(wm, wo) * co < 0.0f) return 0.0f;
        float F = fresnel_dielectric(fabsf(dot(wo, wm)), ior);
        float T = 1.0f - F;
        if (refl) return pdf_glossy(wo, wi, wm) * F;
        float temp = dot(wi, wm) + dot(wo, wm) / eta;
        float dwm = fabsf(dot(wo, wm)) / (temp * temp);
        float noh = fmaxf(wm.z, 0.0f);
        float D = ggx.D(wm);
        return D * noh * dwm * T;
    }
    // UnifiedBSDF::f / pdf / sampleF, bsdf.cuh:191-268
    f3 f(f3 w_wo, f3 w_wi) const {
        M3 ib = transpose(basis);
        f3 wo = mul(ib, w_wo), wi = mul(ib, w_wi);
        float wm_ = metallic;
        float wt = (1.0f - wm_) * transmission;
        float wd = (1.0f - wm_) * (1.0f - transmission);
        f3 F = F3(0.0f);
        if (wm_ > 0.0f) F = F + (f_conductor(wo, wi) * wm_);
        if (wt > 0.0f) F = F + (f_transparent(wo, wi) * wt);
        if (wd > 0.0f) F = F + (f_opaque(wo, wi) * wd);
        return F;
    }
    float pdf(f3 w_wo, f3 w_wi) const {
        M3 ib = transpose(basis);
        f3 wi = mul(ib, w_wi), wo = mul(ib, w_wo);
        float wm_ = metallic;
        float wt = (1.0f - wm_) * transmission;
        float wd = (1.0f - wm_) * (1.0f - transmission);
        float p = 0.0f;
        if (wm_ > 0.0f) p += wm_ * pdf_conductor(wo, wi);
        if (wt > 0.0f) p += wt * pdf_transparent(wo, wi);
        if (wd > 0.0f) p += wd * pdf_opaque(wo, wi);
        return p;
    }
    BSDFSample sample(f3 w_wo, f2 u, f2 X, float xs = 1.0f) const {
        f3 wo = mul(transpose(basis), w_wo);
        float pm = metallic;
        float pt = (1.0f - pm) * transmission;
        BSDFSample bs;
        if (X.x < pm) bs = sample_conductor(wo, u, xs);
        else if (X.x < pt) bs = sample_transparent(wo, u, X.y, xs);
        else bs = sample_opaque(wo, u, X.y, xs);
        bs.wi = mul(basis, bs.wi);
        return bs;
    }
};

// ---------------------------------------------------------------------------
// Nishita single-scattering atmosphere (shaders/atmosphere.cuh:30-311); the
// coefficients and scale heights are parameters with the reference's values
// as defaults.

struct Atmosphere {
    f3 sun_dir;
    float emission;
    float Re = 6378137.0f, Ra = 6438137.0f;
    float Hr, Hm;
    f3 sR;
    float sM, aM;
};
static Atmosphere make_atmosphere(const Env& e, f3 sun_dir) {
    Atmosphere a;
    a.sun_dir = sun_dir;
    a.emission = e.sun_emission_factor;
    a.Hr = e.rayleigh_height;
    a.Hm = e.mie_height;
    a.sR = {e.rayleigh[0], e.rayleigh[1], e.rayleigh[2]};
    a.sM = e.mie;
    a.aM = e.mie_absorption;
    return a;
}
static bool intersect_sphere(const Ray& r, float radius, float* t0, float* t1) {  // atmosphere.cuh:30-57
    f3 oc = F3(0.0f) - r.o;
    float a = dot(r.d, r.d);
    float b = -2.0f * dot(r.d, oc);
    float c = dot(oc, oc) - Sqr(radius);
    float disc = Sqr(b) - 4.0f * a * c;
    if (disc < 0.0f) return false;
    float sq = sqrtf(disc);
    *t0 = (-b - sq) / (2.0f * a);
    *t1 = (-b + sq) / (2.0f * a);
    if (*t0 > *t1) std::swap(*t0, *t1);
    if (*t1 < 0.0f) return false;
    return true;
}
static f3 sky(const Atmosphere& A, const Ray& r) {  // atmosphere.cuh:132-223
    float tmin = 0.0f, tmax = INFINITY;
    {
        float te, tx;
        if (!intersect_sphere(r, A.Ra, &te, &tx) || tx < 0.0f) return F3(0.0f);
        if (te > tmin && te > 0.0f) tmin = te;
        if (tx < tmax) tmax = tx;
    }
    const float depth = tmax - tmin;
    const float step = depth / 16u;
    float t = tmin;
    f3 iR = F3(0.0f), iM = F3(0.0f);
    float oR = 0.0f, oM = 0.0f;
    for (uint32_t i = 0; i < 16u; ++i) {
        const f3 sp = point_at(r, t + (step * 0.5f));
        const float alt = length(sp) - A.Re;
        const float pR = expf(-alt / A.Hr) * step;
        const float pM = expf(-alt / A.Hm) * step;
        oR += pR;
        oM += pM;
        float lte, ltx;
        Ray rl = make_ray(sp, A.sun_dir);
        intersect_sphere(rl, A.Ra, &lte, &ltx);
        const float lstep = ltx / 8u;
        float lt = 0.0f, lR = 0.0f, lM = 0.0f;
        uint8_t j;
        for (j = 0; j < 8u; ++j) {
            const f3 spl = point_at(rl, lt + (lstep * 0.5f));
            const float altl = length(spl) - A.Re;
            if (altl < 0.0f) break;
            lR += expf(-altl / A.Hr) * lstep;
            lM += expf(-altl / A.Hm) * lstep;
            lt += lstep;
        }
        if (j == 8u) {
            const f3 tR = A.sR + 0.0f;
            const f3 tM = F3(A.sM + A.aM);
            const f3 tau = tR * (oR + lR) + tM * (oM + lM);
            const f3 Tr = {expf(-tau.x), expf(-tau.y), expf(-tau.z)};
            iR = iR + Tr * pR;
            iM = iM + Tr * pM;
        }
        t += step;
    }
    const float mu = dot(r.d, A.sun_dir);
    const float ray_phase = (3.0f * (1.0f + Sqr(mu))) / (16.0f * PI);
    const float g = 0.76f;
    const float denom = (8.0f * PI) * ((2.0f + Sqr(g)) * powf(1.0f + Sqr(g) - 2.0f * g * mu, 1.5f));
    const float mie_phase = 3.0f * ((1.0f - Sqr(g)) * (1.0f + Sqr(mu))) / denom;
    const f3 L = (A.sR * iR * ray_phase + F3(A.sM) * iM * mie_phase);
    return L * 6.0e5f * A.emission;
}
static f3 sun_direction(const Env& e) {  // integrator.cuh:222-230
    float phi = e.sun_phi, th = e.sun_theta;
    return normalize(F3(cosf(phi) * cosf(th), sinf(th), sinf(phi) * cosf(th)));
}

// ---------------------------------------------------------------------------
// integrator (shaders/integrator.cuh:61-417 and the surrounding device code)

struct Surface {   // shaders/interaction.cuh:223-275
    int prim = -1, inst = -1, light = -1, material = -1;
    f3 wo = {0, 0, 0};
    float distance = INFINITY;
    f2 uv = {0, 0};
    f3 pos = {0, 0, 0}, ng = {0, 0, 0};
    bool backface = false;
};

// Intersection::getSurfaceInteraction (interaction.cu:11-38).
static Surface surface_interaction(const Scene& s, const Hit& h, const Ray& r) {
    Surface si;
    si.prim = h.prim;
    si.inst = h.inst;
    si.distance = h.t;
    si.wo = -r.d;
    const Tri& t = s.tris[h.prim];
    const M4& model = s.mesh_model[h.inst];
    si.material = t.material;
    si.pos = point_at(r, h.t);
    si.ng = normalize(xyz(mul(model, F4(t.local_gn, 0.0f))));
    f2 uv = (h.bary.x * t.uv[0]) + (h.bary.y * t.uv[1]);
    si.uv = uv + (h.bary.z * t.uv[2]);
    if (!(dot(si.ng, si.wo) > 0.0f)) { si.ng = si.ng * -1.0f; si.backface = true; }
    si.light = t.light;
    return si;
}
static f3 light_L(const Scene& s, const Light& l, f2 uv) {  // light.cu:21-33
    const Material& m = s.materials[s.tris[l.prim].material];
    f3 em = F3(m.emission[0], m.emission[1], m.emission[2]) * m.emission_scale;
    if (m.emission_tex >= 0) {
        f3 t = texture_eval(s, m.emission_tex, uv);
        t = {powf(t.x, 2.2f), powf(t.y, 2.2f), powf(t.z, 2.2f)};
        em = em * t;
    }
    return em;
}
// Material::getBSDF (material.cu:17-70).
static BSDF material_bsdf(const Scene& s, const Surface& si) {
    const Material& m = s.materials[si.material];
    f3 alb = {m.albedo[0], m.albedo[1], m.albedo[2]};
    float rough = m.roughness, metal = m.metallic, trans = m.transmission;
    f3 n = si.ng;
    if (m.albedo_tex >= 0) {
        f3 t = texture_eval(s, m.albedo_tex, si.uv);
        alb = alb * F3(srgb_decode(t.x), srgb_decode(t.y), srgb_decode(t.z));
    }
    if (m.orm_tex >= 0) {
        f3 t = texture_eval(s, m.orm_tex, si.uv);
        rough *= t.y;
        metal *= t.z;
    }
    if (m.transmission_tex >= 0) trans *= texture_eval(s, m.transmission_tex, si.uv).x;
    if (m.normal_tex >= 0) {
        f3 t = texture_eval(s, m.normal_tex, si.uv);
        f3 mn = (t * 2.0f) - 1.0f;
        mn.x *= m.normal_scale;
        mn.y *= m.normal_scale;
        M3 fr = onb_frisvad(n);
        f3 sn = mul(fr, normalize(mn));
        n = (dot(si.wo, sn) > 0.0f) ? sn : n;
    }
    BSDF b;
    b.basis = onb_frisvad(n);
    b.albedo = alb;
    b.metallic = metal;
    b.roughness = rough;
    b.transmission = trans;
    b.ior = m.ior;
    b.backface = si.backface;
    b.ggx.alpha = Sqr(rough);
    return b;
}
static inline float power_heuristic(float f, float g) {  // maths/sampling.cuh:13-17
    return Sqr(f) / (Sqr(f) + Sqr(g));
}
// SurfaceInteraction::spawnRayTo (interaction.cuh:53-63) + Unoccluded (integrator.cuh:124-131).
static bool unoccluded(const Scene& s, const Surface& si, f3 target, Counters& c) {
    f3 o = si.backface ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
    Ray r = make_ray(o, normalize(target - o));
    float tmax = distance3(target, r.o) - 0.11f;
    return !tlas_occluded(s, r, 0.0f, tmax, c);
}

struct PathResult {
    f3 L;
    f3 albedo;          // visible surface albedo (G-buffer)
    int first_prim, first_inst;
    float first_t;
};

struct Frame {
    const Scene* s;
    Env env;
    Settings set;
    M4 inv_proj, inv_view;
    f3 cam_pos;
    f3 sun_dir;
    Atmosphere atm;
    int rng_order;
};

// Rounding-sensitivity probe (test support, not part of the reference's
// algorithm): when given to Li, the quantities a fast-maths build computes
// with rounding that differs from this one -- every scattered ray direction,
// geometric normal, area-light sample point, surface point and the path
// throughput -- are moved by a relative amount of at most eps (directions,
// normals, throughput) or eps_pos (points) in a pseudo-random direction drawn
// from its own stream.  The inputs of the computations that amplify rounding
// are moved by eps_pos too: the interpolated texture coordinates (a texel
// edge) and the random numbers that the BSDF and the light sampler map to a
// direction or a point, and by a few ulps the cosine of the sampled GGX
// microfacet normal (near the lobe's axis its inverse cosine turns one ulp of
// a value next to 1 into ~1e-4 of angle, ~1e-3 at roughness 0.01); the
// numbers that choose a lobe, a light
// or the sun, and Russian roulette's, are the same in every build and are
// not moved.  Camera rays, traversal and the sun's target are computed
// exactly alike everywhere and are not moved either.  A
// sample whose radiance moves by more than the parity tolerance under such a
// perturbation of a few ulps sits at a decision that rounding can flip (a ray
// grazing a triangle edge or silhouette, a shadow ray grazing an occluder, a
// hemisphere or total-internal-reflection test, a Russian-roulette draw next
// to its threshold) or is ill-conditioned (a near-specular lobe).
struct Perturb {
    uint32_t state;
    float eps, eps_pos;
    float next() {   // in [-1, 1]
        state = pcg_hash(state);
        return (float)state * INV_UINT32MAX * 2.0f - 1.0f;
    }
    f3 vec() { float a = next(); float b = next(); float c = next(); return {a, b, c}; }
    f3 dir(f3 d) { return d + vec() * eps; }   // not renormalised: a unit vector off by a few ulps
    f3 point(f3 p) {
        float m = fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))) + 1.0f;
        return p + vec() * (eps_pos * m);
    }
    f3 scale(f3 v) {
        float a = next(); float b = next(); float c = next();
        return {v.x * (1.0f + eps * a), v.y * (1.0f + eps * b), v.z * (1.0f + eps * c)};
    }
    f2 uv(f2 v) {   // relative eps_pos, kept in [0, 1] where the value was
        float a = next(); float b = next();
        f2 r = {v.x * (1.0f + eps_pos * a), v.y * (1.0f + eps_pos * b)};
        if (v.x <= 1.0f && r.x > 1.0f) r.x = v.x;
        if (v.y <= 1.0f && r.y > 1.0f) r.y = v.y;
        return r;
    }
};

// Integrator::Li (integrator.cuh:241-402) including LeSun (:135-143),
// sampleLdSun (:147-186) and sampleLd (:188-220).  P (test support) is null
// except under the rounding-sensitivity probe.
static PathResult Li(const Frame& F, const Ray& ray_in, Sampler& S, Counters& c, Perturb* P = nullptr) {
    const Scene& s = *F.s;
    const int max_depth = F.set.max_depth;
    f3 L = F3(0.0f), beta = F3(1.0f);
    int depth = 0;
    float p_b = 1.0f;
    f3 prev_pos = {0, 0, 0};
    const Atmosphere& A = F.atm;
    const f3 observer = {0.0f, A.Re + 1.0f, 0.0f};
    const size_t nl = s.lights.size();
    PathResult out;
    out.albedo = F3(0.0f);
    out.first_prim = -1; out.first_inst = -1; out.first_t = INFINITY;
    bool any_non_specular = false;
    Ray ray = ray_in;
    while (nonzero(beta)) {
        S.seed = S.seed + (uint32_t)depth;
        bool first = (depth == 0);
        if (P && !first) ray = make_ray(ray.o, P->dir(ray.d));
        Hit h = tlas_intersect(s, ray, 0.0f, INFINITY, c);
        if (h.prim < 0) {
            f3 sk = sky(A, make_ray(observer, ray.d));
            c.sky_evals++;
            if (first) {
                float min_sim = cosf(F.env.sun_angular_diameter / 2.0f);
                float sim = dot(ray.d, A.sun_dir);
                bool sun_surface = sim > min_sim;
                float sr = F.env.sun_emission_factor * 6.0e5f;
                f3 lesun = F3(sr * powf(1.0f / sr, (float)(!sun_surface)));
                sk = sk * lesun;
                out.albedo = sk;
            }
            L = L + sk * beta;
            break;
        }
        if (first) { out.first_prim = h.prim; out.first_inst = h.inst; out.first_t = h.t; }
        Surface si = surface_interaction(s, h, ray);
        if (P) { si.pos = P->point(si.pos); si.ng = P->dir(si.ng); si.uv = P->uv(si.uv); }
        f3 Le = F3(0.0f);
        if (si.light >= 0) Le = light_L(s, s.lights[si.light], si.uv);
        if (nonzero(Le)) {
            float w_l = 1.0f;
            if (si.light >= 0 && !first) {
                const Light& lt = s.lights[si.light];
                float pmf = (nl < 1) ? 0.0f : (1.0f / (float)nl);
                float area_pdf = 1.0f / lt.area;
                float dist = distance3(si.pos, prev_pos);
                float cosl = AbsDot(normalize(si.pos - prev_pos), si.ng);
                float lpdf = pmf * (area_pdf / (cosl / Sqr(dist)));
                w_l = power_heuristic(p_b, lpdf);
            }
            L = L + Le * w_l * beta;
        }
        BSDF bsdf = material_bsdf(s, si);
        if (first) {
            out.albedo = nonzero(Le) ? Le : bsdf.albedo;
            bsdf.albedo = F3(1.0f);
        }
        if (any_non_specular) bsdf.regularize();
        f3 wo = -ray.d;
        if (bsdf.non_specular()) {
            if (S.get1D() < 0.5f) {
                // sampleLdSun
                f3 Ld = F3(0.0f);
                f3 sd = A.sun_dir;
                const float dist_sun = 149.597e9f;
                f3 sun_pos = sd * dist_sun;
                float sun_r = (2.0f * dist_sun * tanf(F.env.sun_angular_diameter / 2.0f)) / 2.0f;
                f3 off;
                if ((F.rng_order & 2) == 0) {
                    f2 a = S.get2D(); float b = S.get1D();
                    off = {a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f};
                } else {
                    float b = S.get1D(); f2 a = S.get2D();
                    off = {a.x * 2.0f - 1.0f, a.y * 2.0f - 1.0f, b * 2.0f - 1.0f};
                }
                f3 target = sun_pos + (off * sun_r);
                f3 fcos = bsdf.f(wo, sd) * fmaxf(0.0f, dot(sd, (si.backface ? -1.0f : 1.0f) * si.ng));
                if (nonzero(fcos)) {
                    f3 srad = sky(A, make_ray(observer, sd));
                    c.sky_evals++;
                    if (nonzero(srad) && unoccluded(s, si, target, c)) {
                        float area = PI * Sqr(sun_r);
                        f3 sn = normalize(target - sun_pos), wi = normalize(target - si.pos);
                        float th = AbsDot(sn, -wi);
                        float pdf = (1.0f / area) / (th / Sqr(dist_sun));
                        Ld = (fcos * srad * 6.0e5f) / pdf;
                    }
                }
                L = L + Ld * beta / 0.5f;
            } else {
                // sampleLd
                f3 Ld = F3(0.0f);
                float X = S.get1D();
                if (nl >= 1) {
                    int li = std::min((int)(X * (float)nl), (int)(nl - 1));
                    const Light& lt = s.lights[li];
                    float prob = 1.0f / (float)nl;
                    f2 u = S.get2D();
                    if (P) u = P->uv(u);
                    // Light::sampleLi (light.cu:35-45) + Triangle::sample (triangle.cuh:104-118)
                    const Tri& tr = s.tris[lt.prim];
                    const M4& model = s.mesh_model[tr.mesh];
                    f3 bary;
                    {
                        f2 b;
                        if (u.x < u.y) { b.x = u.x / 2.0f; b.y = u.y - b.x; }
                        else { b.y = u.y / 2.0f; b.x = u.x - b.y; }
                        bary = {b.x, b.y, 1.0f - b.x - b.y};
                    }
                    f2 luv = (bary.x * tr.uv[0]) + (bary.y * tr.uv[1]);
                    luv = luv + (bary.z * tr.uv[2]);
                    f3 p = (tr.p[0] * bary.x) + (tr.p[1] * bary.y);
                    p = p + (tr.p[2] * bary.z);
                    p = xyz(mul(model, F4(p, 1.0f)));
                    if (P) p = P->point(p);
                    f3 gn = xyz(mul(model, F4(tr.local_gn, 0.0f)));
                    float tri_area = 0.5f * length(cross(tr.p[1] - tr.p[0], tr.p[2] - tr.p[0]));
                    float pdf = 1.0f / tri_area;
                    pdf *= Sqr(distance3(p, si.pos));
                    pdf /= AbsDot(normalize(p - si.pos), gn);
                    f3 wi = normalize(p - si.pos);
                    f3 Lem = light_L(s, lt, luv);
                    if (!(pdf <= 0 || !nonzero(Lem))) {
                        f3 fcos = bsdf.f(wo, wi) * fmaxf(0.0f, dot(wi, (si.backface ? -1.0f : 1.0f) * si.ng));
                        if (nonzero(fcos) && unoccluded(s, si, p, c)) {
                            float p_l = prob * pdf;
                            float pb = bsdf.pdf(wo, wi);
                            float w_l = power_heuristic(p_l, pb);
                            Ld = (Lem * fcos * w_l) / p_l;
                        }
                    }
                }
                L = L + Ld * beta / (1.0f - 0.5f);
            }
        }
        if (depth++ == max_depth) break;
        f2 u, X;
        if ((F.rng_order & 4) == 0) { u = S.get2D(); X = S.get2D(); }
        else { X = S.get2D(); u = S.get2D(); }
        float xs = 1.0f;
        if (P) {
            u = P->uv(u);
            if (P->eps > 0.0f) xs = 1.0f + 4.0f * FLT_EPSILON * P->next();   // a few ulps of the microfacet cosine
        }
        BSDFSample bs = bsdf.sample(wo, u, X, xs);
        if (bs.scatter == ABSORBED || !nonzero(bs.f)) break;
        beta = beta * (bs.f * AbsDot(si.ng, bs.wi) / bs.pdf);
        if (P) beta = P->scale(beta);
        p_b = bsdf.pdf(wo, bs.wi);
        any_non_specular |= !(bs.scatter & SPECULAR);
        prev_pos = si.pos;
        f3 o = (bs.scatter & TRANSMITTED) ? (si.pos - (si.ng * HIT_EPS)) : (si.pos + (si.ng * HIT_EPS));
        ray = make_ray(o, bs.wi);
        // russianRoulette (maths/sampling.cuh:19-31)
        float mx = fmaxf(beta.x, fmaxf(beta.y, beta.z));
        if (mx < 1 && depth > 1) {
            float q = fmaxf(0.0f, 1.0f - mx);
            if (S.get1D() < q) break;
            beta = beta / (1.0f - q);
        }
    }
    out.L = L;
    return out;
}

// Camera::generateRay (camera.cuh:16-25).
static Ray camera_ray(const Frame& F, f2 ndc) {
    f4 tcs = mul(F.inv_proj, F4(ndc.x, ndc.y, 1.0f, 1.0f));
    f4 tws = mul(F.inv_view, F4(normalize(xyz(tcs) / tcs.w), 0.0f));
    return make_ray(F.cam_pos, normalize(xyz(tws)));
}

// One sample of the megakernel body (kernels.cu:385-413): seed, discarded
// filter draw, camera ray, Li, clampOutput.
static PathResult megakernel_sample(const Frame& F, int x, int y, int W, int H, int frame_index, Counters& c,
                                    Perturb* P = nullptr) {
    Sampler S;
    S.order = F.rng_order;
    S.init(x, y, W, frame_index);
    S.get2D();  // BoxFilter::sample, result discarded (kernels.cu:397-402)
    f2 uv = {((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H};
    f2 ndc = {2.0f * uv.x - 1.0f, 2.0f * uv.y - 1.0f};
    Ray r = camera_ray(F, ndc);
    PathResult pr = Li(F, r, S, c, P);
    pr.L = clamp_output(F3(1.0f) * 1.0f * pr.L);
    return pr;
}

template <class Fn>
static void parallel_rows(int n, int nthreads, Fn fn) {
    if (nthreads <= 1 || n < 2) { for (int i = 0; i < n; ++i) fn(i, 0); return; }
    nthreads = std::min(nthreads, n);
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t] { for (int i; (i = next.fetch_add(1)) < n;) fn(i, t); });
    for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// post chain (kernels.cu:453-504, histogram.cu, bloom.cu,
// autoexposure_program.hpp, film.cuh, color.cuh)

struct Image {
    int w = 0, h = 0;
    std::vector<f4> px;
    f4 at(int x, int y) const {  // surf2Dread with cudaBoundaryModeClamp
        x = std::min(std::max(x, 0), w - 1);
        y = std::min(std::max(y, 0), h - 1);
        return px[(size_t)y * w + x];
    }
    // DeviceTextureBuffer::textureReadBilinear (device_texture_buffer.cuh:42-80)
    f4 bilinear(f2 pc) const {
        int dx = (int)pc.x, dy = (int)pc.y;
        int s0 = dx, s1 = dx + 1, t0 = dy, t1 = dy + 1;
        float ws = pc.x - (float)dx, wt = pc.y - (float)dy;
        f4 c0 = at(s0, t0), c1 = at(s1, t0), c2 = at(s0, t1), c3 = at(s1, t1);
        f4 a = lerp4(c0, c1, ws), b = lerp4(c2, c3, ws);
        return lerp4(a, b, wt);
    }
};

static f4 karis(f4 a, f4 b, f4 c, f4 d) {  // bloom.cu:6-15
    float w0 = 1.0f / luminance(xyz(a)), w1 = 1.0f / luminance(xyz(b));
    float w2 = 1.0f / luminance(xyz(c)), w3 = 1.0f / luminance(xyz(d));
    float nw = 1.0f / (w0 + w1 + w2 + w3);
    return (a * w0 + b * w1 + c * w2 + d * w3) * nw;
}
static f4 read36(const Image& t, f2 p, bool ka) {  // bloom.cu:17-74
    auto T = [&](float ox, float oy) { return t.bilinear(F2(p.x + ox, p.y + oy)); };
    f4 a = T(-2, 2), b = T(0, 2), c = T(2, 2), d = T(-2, 0), e = t.bilinear(p), f = T(2, 0);
    f4 g = T(-2, -2), h = T(0, -2), i = T(2, -2);
    auto box = [&](f4 p0, f4 p1, f4 p2, f4 p3) {
        return ka ? karis(p0, p1, p2, p3) : lerp4(lerp4(p0, p1, 0.5f), lerp4(p2, p3, 0.5f), 0.5f);
    };
    f4 hb1 = box(a, b, d, e), hb2 = box(b, c, e, f), hb3 = box(d, e, g, h), hb4 = box(e, f, h, i);
    f4 j = T(-1, 1), k = T(1, 1), l = T(-1, -1), m = T(1, -1);
    f4 hb5 = box(j, k, l, m);
    return lerp4(hb5, lerp4(lerp4(hb1, hb2, 0.5f), lerp4(hb3, hb4, 0.5f), 0.5f), 0.5f);
}
static void bloom_down(const Image& src, Image& dst, bool ka) {  // bloom.cu:90-110
    for (int y = 0; y < dst.h; ++y)
        for (int x = 0; x < dst.w; ++x) {
            f2 uv = {(float)x / (float)dst.w, (float)y / (float)dst.h};
            f2 sp = {uv.x * (float)src.w, uv.y * (float)src.h};
            f4 c = read36(src, sp, ka);
            dst.px[(size_t)y * dst.w + x] = F4(clamp_output(xyz(c)), 1.0f);
        }
}
static void bloom_up(const Image& src, Image& dst, float blend) {  // bloom.cu:112-146
    static const float K[3][3] = {{1.0f / 16.0f, 2.0f / 16.0f, 1.0f / 16.0f},
                                  {2.0f / 16.0f, 4.0f / 16.0f, 2.0f / 16.0f},
                                  {1.0f / 16.0f, 2.0f / 16.0f, 1.0f / 16.0f}};
    for (int y = 0; y < dst.h; ++y)
        for (int x = 0; x < dst.w; ++x) {
            f2 uv = {(float)x / (float)dst.w, (float)y / (float)dst.h};
            f2 sp = {uv.x * (float)src.w, uv.y * (float)src.h};
            f4 m = {0, 0, 0, 0};
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i)
                    m = m + K[j + 1][i + 1] * src.bilinear(F2(sp.x + (float)i, sp.y + (float)j));
            f4 prev = dst.px[(size_t)y * dst.w + x];
            m = lerp4(prev, m, blend);
            dst.px[(size_t)y * dst.w + x] = F4(clamp_output(xyz(m)), 1.0f);
        }
}

// Fixed-point (2^24) histogram weights: the deterministic form of the
// reference's float-atomic histogram (histogram.cu:18-90).
static const double HIST_ONE = 16777216.0;

// luminanceToBin (histogram.cu:18-33) decided exactly: the bin is the count
// of thresholds 2^(black + range*k/254), k = 1..254, at or below Y (with the
// 0.005 black cut-off), thresholds evaluated in double and rounded up to float.
static void bin_thresholds(float black_ev, float white_ev, float* thr /*255*/) {
    double range = (double)white_ev - (double)black_ev;
    thr[0] = 0.005f;
    for (int k = 1; k < 255; ++k) {
        double v = exp2((double)black_ev + range * (double)k / 254.0);
        float f = (float)v;
        if ((double)f < v) f = nextafterf(f, INFINITY);
        thr[k] = f;
    }
}
static int bin_of(float Y, const float* thr) {
    if (!(Y >= thr[0])) return 0;
    int b = 1;
    for (int k = 1; k < 255; ++k) if (Y >= thr[k]) b = k + 1;
    return b > 255 ? 255 : b;
}
// centerMeteringWeight (histogram.cu:35-48) with IEEE-rounded operations.
static float metering_weight(int W, int H, int x, int y) {
    int cx = (int)((float)W / 2.0f), cy = (int)((float)H / 2.0f);
    float dx = (float)(cx - x), dy = (float)(cy - y);
    float dist = sqrtf(dx * dx + dy * dy);
    dist *= (1.0f / 0.4f);
    float maxd = fminf((float)W, (float)H) / 2.0f;
    float nd = dist / maxd;
    float w = 1.0f - smoothstepf(0.0f, 1.0f, nd);
    return clampf(w, 0.0f, 1.0f);
}
// Which bins of a 16x16 histogram block reach the global histogram: bin b
// is flushed by thread b, which exits early when its own pixel lies outside
// the image (histogram.cu:55-90).
static inline bool bin_flushed(int W, int H, int x, int y, int b) {
    int bx = (x / 16) * 16 + (b & 15), by = (y / 16) * 16 + (b >> 4);
    return bx < W && by < H;
}

struct ExposureOut { float avg_bin, avg_lum, adapted, exposure_scalar, iso, shutter; };

// Average of the histogram and eye adaptation (histogram.cu:93-154), then the
// host AutoExposureProgram (autoexposure_program.hpp:18-94) and setExposure
// (renderer.cu:312-329), all in double.
static ExposureOut exposure_from_hist(const uint64_t* hist, const Exposure& ex, float last_lum, float delta_ms) {
    uint64_t total = 0, wsum = 0;
    for (int b = 0; b < 256; ++b) { total += hist[b]; wsum += hist[b] * (uint64_t)b; }
    double nonblack = (double)(total - hist[0]) / HIST_ONE;
    if (nonblack < 0.001) nonblack = 0.001;
    double avg_bin = ((double)wsum / HIST_ONE) / nonblack;
    double range = (double)ex.white_ev - (double)ex.black_ev;
    double t = (avg_bin - 1.0) / 254.0;
    t = t < 0 ? 0 : (t > 1 ? 1 : t);
    double avg_lum = exp2(t * range + (double)ex.black_ev);
    double k = 1.0 - exp(-(double)delta_ms * 0.5);
    double adapted = (double)last_lum + k * (avg_lum - (double)last_lum);
    float adapted_f = (float)adapted;
    double ev = log2(((double)adapted_f * 100.0) / 12.5) - (double)ex.ev_comp + 6.0;
    double N = ex.aperture;
    double shutter = 1.0 / (0.1 * 1000.0);
    double iso = (N * N * 100.0) / (shutter * exp2(ev));
    iso = std::min(std::max(iso, (double)ex.min_iso), (double)ex.max_iso);
    double evdiff = ev - log2((N * N * 100.0) / (shutter * iso));
    shutter = shutter * exp2(-evdiff);
    shutter = std::min(std::max(shutter, (double)ex.min_shutter), (double)ex.max_shutter);
    float isof = (float)iso, shf = (float)shutter;
    double lavg = (10.0 / 0.65) * ((N * N) / ((double)isof * (double)shf));
    ExposureOut o;
    o.avg_bin = (float)avg_bin;
    o.avg_lum = (float)avg_lum;
    o.adapted = adapted_f;
    o.exposure_scalar = (float)(0.18 / lavg);
    o.iso = isof;
    o.shutter = shf;
    return o;
}

// AgX (film.cuh:79-194).
static f3 agx(f3 c, float white_ev, float black_ev) {
    const float MG = 0.18f;
    const float mn = log2f(exp2f(black_ev) * MG), mx = log2f(exp2f(white_ev) * MG);
    const float dr = mx - mn;
    // LINEAR_SRGB_TO_LINEAR_REC2020 (columns), film.cuh:34-37
    M3 to2020 = {{{0.6274f, 0.0691f, 0.0164f}, {0.3293f, 0.9195f, 0.0880f}, {0.0433f, 0.0113f, 0.8956f}}};
    M3 inset = {{{0.856627153315983f, 0.137318972929847f, 0.11189821299995f},
                 {0.0951212405381588f, 0.761241990602591f, 0.0767994186031903f},
                 {0.0482516061458583f, 0.101439036467562f, 0.811302368396859f}}};
    M3 outset = {{{1.9648846919172409596f, -0.29937618452442253746f, -0.16440106280678278299f},
                  {-0.85594737466675834968f, 1.3263980951083531115f, -0.23819967517076844919f},
                  {-0.10883731725048386702f, -0.02702191058393112346f, 1.4025007379775505276f}}};
    f3 r2020 = mul(to2020, c);
    r2020 = fmax3(r2020, F3(0.0f));
    f3 ins = mul(inset, r2020);
    f3 lg = {clampf(log2f(ins.x), mn, mx), clampf(log2f(ins.y), mn, mx), clampf(log2f(ins.z), mn, mx)};
    f3 x = (lg - mn) / dr;
    // AgXDefaultContrastApprox (film.cuh:57-69)
    f3 x2 = x * x, x4 = x2 * x2;
    f3 v = 15.5f * x4 * x2 - 40.14f * x4 * x + 31.96f * x4 - 6.868f * x2 * x + 0.4298f * x2 + 0.1191f * x - 0.00232f;
    // AgXLook, Punchy (film.cuh:123-148)
    float luma = dot(v, F3(0.2126f, 0.7152f, 0.0722f));
    f3 nv = {powf(v.x * 1.0f + 0.0f, 1.05f), powf(v.y * 1.0f + 0.0f, 1.05f), powf(v.z * 1.0f + 0.0f, 1.05f)};
    f3 look = (nv - luma) * 1.25f;
    look = {luma + look.x, luma + look.y, luma + look.z};
    // AgXFittedEOTF (film.cuh:155-172)
    f3 lin = {powf(look.x, 2.4f), powf(look.y, 2.4f), powf(look.z, 2.4f)};
    f3 srgb = mul(outset, lin);
    srgb = fmax3(srgb, F3(0.0f));
    return {srgb_encode(srgb.x), srgb_encode(srgb.y), srgb_encode(srgb.z)};
}
// computePostProcess body (kernels.cu:475-504): bloom lerp, Yxy exposure, AgX.
static f3 post_pixel(f3 c, f3 bloom, bool use_bloom, float final_blend, float expo, float white, float black) {
    if (use_bloom) c = c + final_blend * (bloom - c);
    f3 xyz_;
    xyz_.x = dot(F3(0.4124564f, 0.3575761f, 0.1804375f), c);
    xyz_.y = dot(F3(0.2126729f, 0.7151522f, 0.0721750f), c);
    xyz_.z = dot(F3(0.0193339f, 0.1191920f, 0.9503041f), c);
    float inv = 1.0f / dot(xyz_, F3(1.0f, 1.0f, 1.0f));
    f3 Yxy = {xyz_.y, xyz_.x * inv, xyz_.y * inv};
    Yxy.x *= expo;
    f3 X;
    X.x = Yxy.x * Yxy.y / Yxy.z;
    X.y = Yxy.x;
    X.z = (float)((double)Yxy.x * (1.0 - (double)Yxy.y - (double)Yxy.z) / (double)Yxy.z);
    f3 rgb;
    rgb.x = dot(F3(3.2404542f, -1.5371385f, -0.4985314f), X);
    rgb.y = dot(F3(-0.9692660f, 1.8760108f, 0.0415560f), X);
    rgb.z = dot(F3(0.0556434f, -0.2040259f, 1.0572252f), X);
    return agx(rgb, white, black);
}

}  // namespace orc

// ===========================================================================
// C ABI

using namespace orc;

extern "C" {

struct orc_handle { Scene s; };

// Scene from per-mesh triangle lists (one mesh per reference MeshSceneEntity)
// following Renderer::loadScene (renderer.cu:356-436) with
// Renderer::setMeshTransform (renderer.cu:250-269) applied to every mesh so
// that the TLAS sees world-space bounds.  `models` are column-major 4x4.
void* orc_scene_create(int ntris, const float* pos, const float* nrm, const float* uv, const int* mat,
                       int nmeshes, const int* mesh_off, const int* mesh_cnt, const float* models,
                       int nmaterials, const void* materials,
                       int ntextures, const int* tex_desc, long long npixels, const unsigned char* pixels) {
    orc_handle* h = new orc_handle();
    Scene& s = h->s;
    s.materials.resize(nmaterials);
    std::memcpy(s.materials.data(), materials, sizeof(Material) * (size_t)nmaterials);
    for (int i = 0; i < ntextures; ++i)
        s.textures.push_back({tex_desc[4 * i], tex_desc[4 * i + 1], tex_desc[4 * i + 2], tex_desc[4 * i + 3]});
    if (npixels > 0) s.pixels.assign(pixels, pixels + npixels);
    s.tris.resize(ntris);
    for (int mi = 0; mi < nmeshes; ++mi) {
        for (int k = 0; k < mesh_cnt[mi]; ++k) {
            int i = mesh_off[mi] + k;
            Tri& t = s.tris[i];
            for (int v = 0; v < 3; ++v) {
                t.p[v] = {pos[9 * i + 3 * v], pos[9 * i + 3 * v + 1], pos[9 * i + 3 * v + 2]};
                t.n[v] = {nrm[9 * i + 3 * v], nrm[9 * i + 3 * v + 1], nrm[9 * i + 3 * v + 2]};
                t.uv[v] = {uv[6 * i + 2 * v], uv[6 * i + 2 * v + 1]};
            }
            t.material = mat[i];
            t.mesh = mi;
            t.light = -1;
            // Triangle constructor, triangle.cuh:51-64
            f3 e0 = t.p[1] - t.p[0], e1 = t.p[2] - t.p[0];
            f3 g = cross(e0, e1);
            f3 avg = (t.n[0] + t.n[1] + t.n[2]) / 3.f;
            t.local_gn = normalize((dot(g, avg) < 0.0f) ? -g : g);
            // emissive material -> light (renderer.cu:393-401, pod_types.hpp:118-122)
            const Material& m = s.materials[t.material];
            f3 emit = F3(m.emission[0], m.emission[1], m.emission[2]) * m.emission_scale;
            if (emit.x > 0.0f || emit.y > 0.0f || emit.z > 0.0f) {
                f3 a = t.p[1] - t.p[0], b = t.p[2] - t.p[0];
                float area = 0.5f * length(cross(a, b));
                s.lights.push_back({i, F3(m.emission[0], m.emission[1], m.emission[2]), m.emission_scale, area});
                t.light = (int)s.lights.size() - 1;
            }
        }
    }
    BlasBuilder bb(s);
    for (int mi = 0; mi < nmeshes; ++mi) {
        M4 model = m4_from(models + 16 * mi);
        Mesh m;
        m.offset = mesh_off[mi];
        m.count = (uint32_t)mesh_cnt[mi];
        m.inv_model = inverse(model);
        m.blas = (int)s.blas.size();
        s.blas.push_back(bb.build(m, mi));
        s.meshes.push_back(m);
        blas_set_transform(s.blas.back(), model);
    }
    build_tlas(s);
    s.mesh_model.resize(s.meshes.size());
    for (size_t i = 0; i < s.meshes.size(); ++i) s.mesh_model[i] = inverse(s.meshes[i].inv_model);
    return h;
}

void orc_scene_destroy(void* h) { delete (orc_handle*)h; }

// counts: [0] bvh nodes (allocated), [1] tri index entries, [2] tlas nodes,
// [3] lights, [4] meshes
void orc_scene_counts(void* hp, long long* out) {
    Scene& s = ((orc_handle*)hp)->s;
    out[0] = (long long)s.nodes.size();
    out[1] = (long long)s.tri_index.size();
    out[2] = (long long)s.tlas_nodes.size();
    out[3] = (long long)s.lights.size();
    out[4] = (long long)s.meshes.size();
}

// BVH arrays: per node (left_first, count) and bounds (pmin, pmax); the
// triangle index buffer; per BLAS (root, world bounds, inv model).
void orc_scene_bvh(void* hp, int* left_first, unsigned* count, float* bounds, int* tri_index,
                   long long* blas_root, float* blas_bounds, float* blas_inv) {
    Scene& s = ((orc_handle*)hp)->s;
    for (size_t i = 0; i < s.nodes.size(); ++i) {
        left_first[i] = s.nodes[i].left_first;
        count[i] = s.nodes[i].count;
        const Bounds& b = s.nodes[i].b;
        float v[6] = {b.pmin.x, b.pmin.y, b.pmin.z, b.pmax.x, b.pmax.y, b.pmax.z};
        std::memcpy(bounds + 6 * i, v, sizeof v);
    }
    std::memcpy(tri_index, s.tri_index.data(), sizeof(int32_t) * s.tri_index.size());
    for (size_t i = 0; i < s.blas.size(); ++i) {
        blas_root[i] = s.blas[i].root;
        const Bounds& b = s.blas[i].b;
        float v[6] = {b.pmin.x, b.pmin.y, b.pmin.z, b.pmax.x, b.pmax.y, b.pmax.z};
        std::memcpy(blas_bounds + 6 * i, v, sizeof v);
        std::memcpy(blas_inv + 16 * i, &s.blas[i].inv_model, 64);
    }
}

void orc_scene_tlas(void* hp, unsigned* lr, int* blas, float* bounds) {
    Scene& s = ((orc_handle*)hp)->s;
    for (size_t i = 0; i < s.tlas_nodes.size(); ++i) {
        lr[i] = s.tlas_nodes[i].lr;
        blas[i] = s.tlas_nodes[i].blas;
        const Bounds& b = s.tlas_nodes[i].b;
        float v[6] = {b.pmin.x, b.pmin.y, b.pmin.z, b.pmax.x, b.pmax.y, b.pmax.z};
        std::memcpy(bounds + 6 * i, v, sizeof v);
    }
}

// Closest hit for n rays.  counters (optional, 8 int64): box tests, triangle
// tests, instance transforms, sky evaluations, hits, rays, max stack,
// rays past the reference's 16-entry stack.
void orc_trace(void* hp, int n, const float* o, const float* d, float tmin, float tmax,
               int* prim, int* inst, float* t, float* bary, int brute, long long* counters, int nthreads) {
    Scene& s = ((orc_handle*)hp)->s;
    std::vector<Counters> cs(std::max(nthreads, 1));
    const int CH = 256;
    parallel_rows((n + CH - 1) / CH, nthreads, [&](int blk, int tid) {
        for (int i = blk * CH; i < std::min(n, (blk + 1) * CH); ++i) {
            Ray r = make_ray(F3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), F3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            Counters& c = cs[tid];
            int64_t ov = c.stack_overflow;
            Hit h = brute ? brute_intersect(s, r, tmin, tmax) : tlas_intersect(s, r, tmin, tmax, c);
            if (c.stack_overflow != ov) c.stack_overflow = ov + 1;   // count rays, not pushes
            prim[i] = h.prim; inst[i] = h.inst; t[i] = h.t;
            if (bary) { bary[3 * i] = h.bary.x; bary[3 * i + 1] = h.bary.y; bary[3 * i + 2] = h.bary.z; }
        }
    });
    if (counters) {
        Counters tot;
        for (auto& c : cs) tot.add(c);
        int64_t v[8] = {tot.box_tests, tot.tri_tests, tot.inst_xforms, tot.sky_evals, tot.hits, tot.rays, tot.max_stack, tot.stack_overflow};
        for (int k = 0; k < 8; ++k) counters[k] = v[k];
    }
}

void orc_occluded(void* hp, int n, const float* o, const float* d, float tmin, const float* tmax,
                  unsigned char* out, int nthreads) {
    Scene& s = ((orc_handle*)hp)->s;
    const int CH = 256;
    parallel_rows((n + CH - 1) / CH, nthreads, [&](int blk, int) {
        Counters c;
        for (int i = blk * CH; i < std::min(n, (blk + 1) * CH); ++i) {
            Ray r = make_ray(F3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), F3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            out[i] = tlas_occluded(s, r, tmin, tmax[i], c) ? 1 : 0;
        }
    });
}

// Diffuse bounce chain of the traversal workload: from each closest hit, a
// cosine-weighted direction about the geometric normal facing the incoming
// ray (Malley's method: a uniform point on the unit disk, rejection-sampled
// from pairs of PCG draws, lifted to the hemisphere, then rotated by the
// Frisvad basis), origin offset by 1e-3 along the normal.  The sampler is
// seeded with 4 * ray index + bounce.  Only IEEE +, -, *, / and sqrt are
// used, so every implementation produces the same rays.  Writes
// (nbounces+1) x n hits.
static f3 bounce_dir(uint32_t seed, f3 n) {
    Sampler S; S.order = 0;
    S.seed = seed;
    float x = 0.0f, y = 0.0f, r2 = 0.0f;
    for (int k = 0; k < 64; ++k) {
        float u0 = S.get1D(), u1 = S.get1D();
        float a = 2.0f * u0 - 1.0f, b = 2.0f * u1 - 1.0f;
        float q = a * a + b * b;
        if (q < 1.0f) { x = a; y = b; r2 = q; break; }
    }
    f3 l = {x, y, sqrtf(1.0f - r2)};
    return mul(onb_frisvad(n), l);
}
static void bounce_ray(const Scene& s, const Hit& h, Ray& r, uint32_t idx, int b) {
    const Tri& tr = s.tris[h.prim];
    f3 n = normalize(xyz(mul(s.mesh_model[h.inst], F4(tr.local_gn, 0.0f))));
    if (dot(n, r.d) > 0.0f) n = -n;
    f3 p = point_at(r, h.t);
    f3 w = bounce_dir(idx * 4u + (uint32_t)b, n);
    r = make_ray(p + n * HIT_EPS, w);
}
void orc_trace_bounces(void* hp, int n, const float* o, const float* d, int nbounces,
                       int* prim, float* t, long long* counters, int nthreads) {
    Scene& s = ((orc_handle*)hp)->s;
    std::vector<Counters> cs(std::max(nthreads, 1));
    const int CH = 256;
    parallel_rows((n + CH - 1) / CH, nthreads, [&](int blk, int tid) {
        Counters& c = cs[tid];
        for (int i = blk * CH; i < std::min(n, (blk + 1) * CH); ++i) {
            Ray r = make_ray(F3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), F3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            for (int b = 0; b <= nbounces; ++b) {
                size_t k = (size_t)b * n + i;
                Hit h = tlas_intersect(s, r, 0.0f, INFINITY, c);
                prim[k] = h.prim; t[k] = h.t;
                if (h.prim < 0) {
                    for (int bb = b + 1; bb <= nbounces; ++bb) { prim[(size_t)bb * n + i] = -1; t[(size_t)bb * n + i] = INFINITY; }
                    break;
                }
                if (b < nbounces) bounce_ray(s, h, r, (uint32_t)i, b);
            }
        }
    });
    if (counters) {
        Counters tot;
        for (auto& c : cs) tot.add(c);
        int64_t v[8] = {tot.box_tests, tot.tri_tests, tot.inst_xforms, tot.sky_evals, tot.hits, tot.rays, tot.max_stack, tot.stack_overflow};
        for (int k = 0; k < 8; ++k) counters[k] = v[k];
    }
}

// Per-sample radiance of the plain method: sample k of pixel (x, y) is the
// megakernel's output for frame_index = sample0 + k (the reference renders
// one sample per frame).  radiance: [nsamples][H][W][3]; albedo: [H][W][3]
// visible-surface albedo (from the last sample); first_hit: [H][W] (prim,
// inst) of sample 0 and first_t [H][W].
void orc_render_samples(void* hp, const float* inv_proj, const float* inv_view, const void* env,
                        const void* settings, int W, int H, int sample0, int nsamples, int rng_order,
                        int row0, int nrows, float* radiance, float* albedo, int* first_hit, float* first_t,
                        long long* counters, int nthreads) {
    Frame F;
    F.s = &((orc_handle*)hp)->s;
    std::memcpy(&F.env, env, sizeof(Env));
    std::memcpy(&F.set, settings, sizeof(Settings));
    F.inv_proj = m4_from(inv_proj);
    F.inv_view = m4_from(inv_view);
    F.cam_pos = xyz(F.inv_view.c[3]);
    F.sun_dir = sun_direction(F.env);
    F.atm = make_atmosphere(F.env, F.sun_dir);
    F.rng_order = rng_order;
    if (nrows <= 0) nrows = H - row0;
    std::vector<Counters> cs(std::max(nthreads, 1));
    parallel_rows(nrows, nthreads, [&](int ry, int tid) {
        int y = row0 + ry;
        for (int x = 0; x < W; ++x) {
            for (int k = 0; k < nsamples; ++k) {
                PathResult pr = megakernel_sample(F, x, y, W, H, sample0 + k, cs[tid]);
                if (radiance) {
                    size_t o = (((size_t)k * nrows + ry) * W + x) * 3;
                    radiance[o] = pr.L.x; radiance[o + 1] = pr.L.y; radiance[o + 2] = pr.L.z;
                }
                if (k == nsamples - 1) {
                    size_t p = (size_t)ry * W + x;
                    if (albedo) { albedo[3 * p] = pr.albedo.x; albedo[3 * p + 1] = pr.albedo.y; albedo[3 * p + 2] = pr.albedo.z; }
                    if (first_hit) { first_hit[2 * p] = pr.first_prim; first_hit[2 * p + 1] = pr.first_inst; }
                    if (first_t) first_t[p] = pr.first_t;
                }
            }
        }
    });
    if (counters) {
        Counters tot;
        for (auto& c : cs) tot.add(c);
        int64_t v[8] = {tot.box_tests, tot.tri_tests, tot.inst_xforms, tot.sky_evals, tot.hits, tot.rays, tot.max_stack, tot.stack_overflow};
        for (int k = 0; k < 8; ++k) counters[k] = v[k];
    }
}

// The rounding-sensitivity probe over the samples of orc_render_samples
// (test support): for every sample, `ncopies` renders under Perturb with
// relative sizes eps and eps_pos (streams seeded from the sample, the pixel and the copy),
// compared with the unperturbed sample: response = the largest over copies
// and channels of |L' - L| / max(max channel of |L|, 1e-3), the relative
// error measure of the parity tests.  radiance (may be null) receives the
// unperturbed samples as orc_render_samples does.
void orc_render_sensitivity(void* hp, const float* inv_proj, const float* inv_view, const void* env,
                            const void* settings, int W, int H, int sample0, int nsamples, int rng_order,
                            int row0, int nrows, float eps, float eps_pos, int ncopies, float* radiance,
                            float* response, int nthreads) {
    Frame F;
    F.s = &((orc_handle*)hp)->s;
    std::memcpy(&F.env, env, sizeof(Env));
    std::memcpy(&F.set, settings, sizeof(Settings));
    F.inv_proj = m4_from(inv_proj);
    F.inv_view = m4_from(inv_view);
    F.cam_pos = xyz(F.inv_view.c[3]);
    F.sun_dir = sun_direction(F.env);
    F.atm = make_atmosphere(F.env, F.sun_dir);
    F.rng_order = rng_order;
    if (nrows <= 0) nrows = H - row0;
    std::vector<Counters> cs(std::max(nthreads, 1));
    parallel_rows(nrows, nthreads, [&](int ry, int tid) {
        int y = row0 + ry;
        for (int x = 0; x < W; ++x) {
            for (int k = 0; k < nsamples; ++k) {
                PathResult pr = megakernel_sample(F, x, y, W, H, sample0 + k, cs[tid]);
                float scale = fmaxf(fmaxf(fabsf(pr.L.x), fmaxf(fabsf(pr.L.y), fabsf(pr.L.z))), 1e-3f);
                float worst = 0.0f;
                for (int q = 0; q < ncopies; ++q) {
                    Perturb P{pcg_hash((uint32_t)(y * W + x) * 7919u + (uint32_t)(sample0 + k) * 104729u +
                                       (uint32_t)q * 15485863u), eps, eps_pos};
                    PathResult pp = megakernel_sample(F, x, y, W, H, sample0 + k, cs[tid], &P);
                    float d = fmaxf(fabsf(pp.L.x - pr.L.x), fmaxf(fabsf(pp.L.y - pr.L.y), fabsf(pp.L.z - pr.L.z)));
                    worst = fmaxf(worst, d / scale);
                }
                size_t o = ((size_t)k * nrows + ry) * W + x;
                if (radiance) { radiance[3 * o] = pr.L.x; radiance[3 * o + 1] = pr.L.y; radiance[3 * o + 2] = pr.L.z; }
                response[o] = worst;
            }
        }
    });
}

// Nishita radiance seen from 1 m above the ground for n directions.
void orc_sky(const void* env, int n, const float* dirs, float* out) {
    Env e;
    std::memcpy(&e, env, sizeof e);
    Atmosphere A = make_atmosphere(e, sun_direction(e));
    f3 obs = {0.0f, A.Re + 1.0f, 0.0f};
    for (int i = 0; i < n; ++i) {
        f3 L = sky(A, make_ray(obs, F3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2])));
        out[3 * i] = L.x; out[3 * i + 1] = L.y; out[3 * i + 2] = L.z;
    }
}

// UnifiedBSDF for unit tests: per case (tangent-frame normal n, albedo,
// metallic, roughness, transmission, ior, backface, regularize) evaluate
// f(wo, wi), pdf(wo, wi) and sampleF(wo, u, X).  params: [n][12]
// (nx ny nz ar ag ab metal rough trans ior backface regularize);
// dirs: [n][6] (wo, wi); u: [n][4]; out: [n][12] (f rgb, pdf, sample f rgb,
// sample wi xyz, sample pdf, scatter).
void orc_bsdf_eval(int n, const float* params, const float* dirs, const float* u, float* out) {
    for (int i = 0; i < n; ++i) {
        const float* p = params + 12 * i;
        BSDF b;
        b.basis = onb_frisvad(F3(p[0], p[1], p[2]));
        b.albedo = {p[3], p[4], p[5]};
        b.metallic = p[6]; b.roughness = p[7]; b.transmission = p[8]; b.ior = p[9];
        b.backface = p[10] != 0.0f;
        b.ggx.alpha = Sqr(p[7]);
        if (p[11] != 0.0f) b.regularize();
        f3 wo = {dirs[6 * i], dirs[6 * i + 1], dirs[6 * i + 2]};
        f3 wi = {dirs[6 * i + 3], dirs[6 * i + 4], dirs[6 * i + 5]};
        f3 fv = b.f(wo, wi);
        float pd = b.pdf(wo, wi);
        BSDFSample bs = b.sample(wo, F2(u[4 * i], u[4 * i + 1]), F2(u[4 * i + 2], u[4 * i + 3]));
        float* o = out + 12 * i;
        o[0] = fv.x; o[1] = fv.y; o[2] = fv.z; o[3] = pd;
        o[4] = bs.f.x; o[5] = bs.f.y; o[6] = bs.f.z;
        o[7] = bs.wi.x; o[8] = bs.wi.y; o[9] = bs.wi.z; o[10] = bs.pdf; o[11] = (float)bs.scatter;
    }
}

// Histogram bin thresholds and bins for a list of luminances.
void orc_hist_thresholds(float black_ev, float white_ev, float* thr) { bin_thresholds(black_ev, white_ev, thr); }
void orc_lum_bins(int n, const float* Y, float black_ev, float white_ev, int* bins) {
    float thr[255];
    bin_thresholds(black_ev, white_ev, thr);
    for (int i = 0; i < n; ++i) bins[i] = bin_of(Y[i], thr);
}

// modulate (integrator.cuh:406-415, kernels.cu:453-472): render = (sum / n)
// times the 8-bit quantised visible-surface albedo, alpha 1.
void orc_modulate(int W, int H, const float* acc_sum, int nsamples, const float* albedo, float* render_out) {
    auto q = [](float v) { uint32_t b = (uint32_t)(saturate(v) * 255.0f) & 0xFFu; return (float)(b & 0xFFu) / 255.0f; };
    for (size_t p = 0; p < (size_t)W * H; ++p) {
        f3 est = F3(acc_sum[3 * p], acc_sum[3 * p + 1], acc_sum[3 * p + 2]) / (float)nsamples;
        f3 m = {q(albedo[3 * p]), q(albedo[3 * p + 1]), q(albedo[3 * p + 2])};
        f3 r = est * m;
        render_out[4 * p] = r.x; render_out[4 * p + 1] = r.y; render_out[4 * p + 2] = r.z; render_out[4 * p + 3] = 1.0f;
    }
}

// Bloom mip chain on a [H][W][4] image; writes mip 0 after the up passes.
void orc_bloom(int W, int H, const float* render, int karis, float internal_blend, float* bloom_out) {
    int levels = std::min((int)std::log2((double)W), (int)std::log2((double)H));
    levels = std::min(levels, 6);
    std::vector<Image> mips(levels + 1);
    for (int l = 0; l <= levels; ++l) {
        mips[l].w = W >> l; mips[l].h = H >> l;
        mips[l].px.assign((size_t)mips[l].w * mips[l].h, F4(0, 0, 0, 0));
    }
    std::memcpy(mips[0].px.data(), render, sizeof(f4) * (size_t)W * H);
    for (int l = 0; l < levels; ++l) bloom_down(mips[l], mips[l + 1], karis != 0 && l == 0);
    for (int l = levels; l > 0; --l) bloom_up(mips[l], mips[l - 1], internal_blend);
    std::memcpy(bloom_out, mips[0].px.data(), sizeof(f4) * (size_t)W * H);
}

// Display image from render and bloom (computePostProcess, kernels.cu:475-504).
void orc_post_image(int W, int H, const float* render, const float* bloom, int use_bloom, float final_blend,
                    float expo, float white_ev, float black_ev, float* image_out) {
    Image r, b;
    r.w = b.w = W; r.h = b.h = H;
    r.px.resize((size_t)W * H);
    std::memcpy(r.px.data(), render, sizeof(f4) * r.px.size());
    if (use_bloom) { b.px.resize((size_t)W * H); std::memcpy(b.px.data(), bloom, sizeof(f4) * b.px.size()); }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            f2 uv = {((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H};
            int sx = (int)(uv.x * (float)W), sy = (int)(uv.y * (float)H);
            f3 c = xyz(r.at(sx, sy));
            f3 bl = use_bloom ? xyz(b.at(sx, sy)) : F3(0.0f);
            f3 o = post_pixel(c, bl, use_bloom != 0, final_blend, expo, white_ev, black_ev);
            size_t p = (size_t)y * W + x;
            image_out[4 * p] = o.x; image_out[4 * p + 1] = o.y; image_out[4 * p + 2] = o.z; image_out[4 * p + 3] = 1.0f;
        }
}

void orc_metering_weights(int W, int H, float* out) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) out[(size_t)y * W + x] = metering_weight(W, H, x, y);
}

// Fixed-point (2^24) histogram of a [H][W][4] render with the reference's
// dropped bins at the image edge.
void orc_histogram(int W, int H, const float* render, float black_ev, float white_ev, unsigned long long* hist) {
    float thr[255];
    bin_thresholds(black_ev, white_ev, thr);
    for (int b = 0; b < 256; ++b) hist[b] = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float* c = render + 4 * ((size_t)y * W + x);
            int b = bin_of(luminance(F3(c[0], c[1], c[2])), thr);
            if (!bin_flushed(W, H, x, y, b)) continue;
            float w = (b > 0) ? metering_weight(W, H, x, y) : 1.0f;
            hist[b] += (uint64_t)nearbyint((double)w * HIST_ONE);
        }
}

// Exposure record from a fixed-point histogram: avg bin, avg lum, adapted
// lum, exposure scalar, iso, shutter.
void orc_exposure(const unsigned long long* hist, const void* exposure, float last_lum, float delta_ms, float* out) {
    Exposure ex;
    std::memcpy(&ex, exposure, sizeof ex);
    std::vector<uint64_t> h(hist, hist + 256);
    ExposureOut eo = exposure_from_hist(h.data(), ex, last_lum, delta_ms);
    float v[6] = {eo.avg_bin, eo.avg_lum, eo.adapted, eo.exposure_scalar, eo.iso, eo.shutter};
    std::memcpy(out, v, sizeof v);
}

// Post chain of one frame.  Inputs: sample sum per pixel (accumulated in
// sample order) and sample count, the visible-surface albedo, settings,
// exposure state and the adapted luminance of the previous frame.
// Outputs: render (after modulate) [H][W][4], bloom mip 0 [H][W][4] (if
// enabled), display image [H][W][4], the fixed-point histogram [256] and
// the exposure record [6] (avg bin, avg lum, adapted lum, exposure scalar,
// iso, shutter).
void orc_post_frame(int W, int H, const float* acc_sum, int nsamples, const float* albedo,
                    const void* settings, const void* exposure, float last_lum,
                    float* render_out, float* bloom_out, float* image_out,
                    unsigned long long* hist_out, float* expo_out) {
    Settings set;
    Exposure ex;
    std::memcpy(&set, settings, sizeof set);
    std::memcpy(&ex, exposure, sizeof ex);
    Image render;
    render.w = W; render.h = H;
    render.px.resize((size_t)W * H);
    for (size_t p = 0; p < (size_t)W * H; ++p) {
        // addSample (integrator.cuh:406-415) then modulateSamples (kernels.cu:453-472)
        f3 est = F3(acc_sum[3 * p], acc_sum[3 * p + 1], acc_sum[3 * p + 2]) / (float)nsamples;
        f3 a = {albedo[3 * p], albedo[3 * p + 1], albedo[3 * p + 2]};
        auto q = [](float v) { uint32_t b = (uint32_t)(saturate(v) * 255.0f) & 0xFFu; return (float)(b & 0xFFu) / 255.0f; };
        f3 m = {q(a.x), q(a.y), q(a.z)};
        render.px[p] = F4(est * m, 1.0f);
    }
    if (render_out) std::memcpy(render_out, render.px.data(), sizeof(f4) * render.px.size());
    // exposure: histogram of the modulated render, then the exposure program
    float expo = 1.0f;
    {
        // the film's exposure scalar as last set (renderer.cu:312-329)
        double N = ex.aperture;
        double lavg = (10.0 / 0.65) * ((N * N) / ((double)ex.iso * (double)ex.shutter));
        expo = (float)(0.18 / lavg);
    }
    if (set.auto_exposure) {
        float thr[255];
        bin_thresholds(ex.black_ev, ex.white_ev, thr);
        std::vector<uint64_t> hist(256, 0);
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                f4 c = render.px[(size_t)y * W + x];
                float Yl = luminance(xyz(c));
                int b = bin_of(Yl, thr);
                if (!bin_flushed(W, H, x, y, b)) continue;
                float w = (b > 0) ? metering_weight(W, H, x, y) : 1.0f;
                hist[b] += (uint64_t)nearbyint((double)w * HIST_ONE);
            }
        ExposureOut eo = exposure_from_hist(hist.data(), ex, last_lum, set.frame_delta_ms);
        expo = eo.exposure_scalar;
        if (hist_out) for (int b = 0; b < 256; ++b) hist_out[b] = hist[b];
        if (expo_out) {
            float v[6] = {eo.avg_bin, eo.avg_lum, eo.adapted, eo.exposure_scalar, eo.iso, eo.shutter};
            std::memcpy(expo_out, v, sizeof v);
        }
    }
    // bloom (renderer.cu:438-475, mipchain.cuh:17-59)
    std::vector<Image> mips;
    if (set.bloom) {
        int levels = std::min((int)std::log2((double)W), (int)std::log2((double)H));
        levels = std::min(levels, 6);
        mips.resize(levels + 1);
        mips[0] = render;
        for (int l = 1; l <= levels; ++l) {
            mips[l].w = W >> l; mips[l].h = H >> l;
            mips[l].px.assign((size_t)mips[l].w * mips[l].h, F4(0, 0, 0, 0));
        }
        for (int l = 0; l < levels; ++l) bloom_down(mips[l], mips[l + 1], set.karis && l == 0);
        for (int l = levels; l > 0; --l) bloom_up(mips[l], mips[l - 1], set.bloom_internal_blend);
        if (bloom_out) std::memcpy(bloom_out, mips[0].px.data(), sizeof(f4) * mips[0].px.size());
    }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            // textureReadNearestUV of the pixel centre
            f2 uv = {((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H};
            int sx = (int)(uv.x * (float)W), sy = (int)(uv.y * (float)H);
            f3 c = xyz(render.at(sx, sy));
            f3 bl = set.bloom ? xyz(mips[0].at(sx, sy)) : F3(0.0f);
            f3 o = post_pixel(c, bl, set.bloom != 0, set.bloom_final_blend, expo, ex.white_ev, ex.black_ev);
            size_t p = (size_t)y * W + x;
            image_out[4 * p] = o.x; image_out[4 * p + 1] = o.y; image_out[4 * p + 2] = o.z; image_out[4 * p + 3] = 1.0f;
        }
}

// Temporal accumulation of one reference frame over every pixel: the
// megakernel's temporal branch (kernels.cu:422-428) with computeVelocity
// (:164-192), testReprojection (:206-223) and reprojectAccumulate without
// SUPER_SAMPLE (:299-327).  Inputs: the previous and current inverse camera
// matrices, every instance's current and previous model matrix
// (column-major, 16 floats each), per pixel the first hit's instance (-1:
// miss) and distance, this frame's clamped sample, the previous frame's
// distances and history image (color, frames); writes the new history.
static M4 mul44(const M4& a, const M4& b) {   // matrix_maths.cuh:269-283: rows of a dotted with columns of b
    M4 r;
    for (int c = 0; c < 4; ++c) {
        const f4 bc = b.c[c];
        r.c[c] = {a.c[0].x * bc.x + a.c[1].x * bc.y + a.c[2].x * bc.z + a.c[3].x * bc.w,
                  a.c[0].y * bc.x + a.c[1].y * bc.y + a.c[2].y * bc.z + a.c[3].y * bc.w,
                  a.c[0].z * bc.x + a.c[1].z * bc.y + a.c[2].z * bc.z + a.c[3].z * bc.w,
                  a.c[0].w * bc.x + a.c[1].w * bc.y + a.c[2].w * bc.z + a.c[3].w * bc.w};
    }
    return r;
}

void orc_temporal_frame(int W, int H, const float* prev_ip, const float* prev_iv, const float* curr_ip,
                        const float* curr_iv, int ninst, const float* curr_models, const float* prev_models,
                        const int32_t* vis_inst, const float* vis_t, const float* sample, const float* prev_depth,
                        const float* hist_in, float* hist_out) {
    const M4 cip = m4_from(curr_ip), civ = m4_from(curr_iv), pip = m4_from(prev_ip), piv = m4_from(prev_iv);
    const M4 curr_vp = mul44(inverse(cip), inverse(civ));
    const M4 prev_vp = mul44(inverse(pip), inverse(piv));
    std::vector<M4> inv_m(ninst), prev_m(ninst), pm(ninst);
    for (int i = 0; i < ninst; ++i) {
        inv_m[i] = inverse(m4_from(curr_models + 16 * i));           // mesh.curr_inv_model_matrix
        prev_m[i] = inverse(inverse(m4_from(prev_models + 16 * i)));  // mesh.prev_inv_model_matrix.inverse()
        pm[i] = mul44(prev_vp, prev_m[i]);
    }
    Frame F{};
    F.inv_proj = cip;
    F.inv_view = civ;
    F.cam_pos = xyz(civ.c[3]);
    const f3 prev_origin = xyz(piv.c[3]);
    auto tex = [&](const float* t, int x, int y) {   // cudaBoundaryModeClamp
        x = std::min(std::max(x, 0), W - 1);
        y = std::min(std::max(y, 0), H - 1);
        const float* q = t + 4 * ((size_t)y * W + x);
        return F4(q[0], q[1], q[2], q[3]);
    };
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t p = (size_t)y * W + x;
            const f4 curr = F4(sample[4 * p], sample[4 * p + 1], sample[4 * p + 2], 0.0f);
            f4 out = curr;
            const int inst = vis_inst[p];
            if (inst >= 0) {
                f2 uv = {((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H};
                f2 ndc = {2.0f * uv.x - 1.0f, 2.0f * uv.y - 1.0f};
                const f3 pos = point_at(camera_ray(F, ndc), vis_t[p]);
                const f3 local = xyz(mul(inv_m[inst], F4(pos, 1.0f)));
                const f4 cc = mul(curr_vp, F4(pos, 1.0f));
                const f4 pc = mul(pm[inst], F4(local, 1.0f));
                const f3 cn = xyz(cc) / cc.w, pn = xyz(pc) / pc.w;
                const float vx = (cn.x + 1.0f) / 2.0f - (pn.x + 1.0f) / 2.0f;
                const float vy = (cn.y + 1.0f) / 2.0f - (pn.y + 1.0f) / 2.0f;
                const float qx = (float)x - vx * (float)W, qy = (float)y - vy * (float)H;
                if (!(qx < 0 || qx >= (float)W || qy < 0 || qy >= (float)H)) {
                    const int ix = (int)qx, iy = (int)qy;
                    const float d2 = prev_depth[(size_t)std::min(std::max(iy, 0), H - 1) * W + std::min(std::max(ix, 0), W - 1)];
                    const f3 pw = xyz(mul(prev_m[inst], F4(local, 1.0f)));
                    const float d1 = length(prev_origin - pw);
                    if (fabsf(d1 - d2) < (d2 * 0.045f)) {
                        const float ws = qx - (float)ix, wt = qy - (float)iy;
                        const f4 c0 = tex(hist_in, ix, iy), c1 = tex(hist_in, ix + 1, iy);
                        const f4 c2 = tex(hist_in, ix, iy + 1), c3 = tex(hist_in, ix + 1, iy + 1);
                        f4 prev = lerp4(lerp4(c0, c1, ws), lerp4(c2, c3, ws), wt);
                        prev.w = c0.w;
                        const float alpha = 1.0f / fminf(prev.w + 1, 16.0f);
                        out = F4(prev.x + alpha * (curr.x - prev.x), prev.y + alpha * (curr.y - prev.y),
                                 prev.z + alpha * (curr.z - prev.z), prev.w + 1);
                    }
                }
            }
            hist_out[4 * p] = out.x;
            hist_out[4 * p + 1] = out.y;
            hist_out[4 * p + 2] = out.z;
            hist_out[4 * p + 3] = out.w;
        }
}

// computeEffects with getFishEyeUV (kernels.cu:340-374, 506-527) on the
// tonemapped image src [H][W][4]: fisheye position (power 1.65, bound to the
// corners), red and blue read at +- the chromatic offset, texels by
// textureReadNearestUV (clamped).
void orc_effects(int W, int H, const float* src, float* dst) {
    auto nearest_uv = [&](float u, float v, int ch) {
        int x = (int)(u * (float)W), y = (int)(v * (float)H);
        x = std::min(std::max(x, 0), W - 1);
        y = std::min(std::max(y, 0), H - 1);
        return src[4 * ((size_t)y * W + x) + ch];
    };
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const f2 res = {(float)W, (float)H};
            const f2 p = {(float)x / res.x, (float)y / res.x};
            const float prop = res.x / res.y;
            const f2 m = {0.5f, 0.5f / prop};
            const f2 d = {p.x - m.x, p.y - m.y};
            const float r = sqrtf(d.x * d.x + d.y * d.y);
            const float power = 1.65f;
            const float bind = sqrtf(m.x * m.x + m.y * m.y);
            const float inv = rsqrt_(d.x * d.x + d.y * d.y);
            const float t1 = tanf(r * power), t2 = tanf(bind * power);
            f2 uv = {m.x + (d.x * inv) * t1 * bind / t2, m.y + (d.y * inv) * t1 * bind / t2};
            uv.y *= prop;
            const f2 uc = {((float)x + 0.5f) / res.x, ((float)y + 0.5f) / res.y};
            const f2 off = {powf(fabsf(uc.x - 0.5f) * 2.0f, 2.0f) * 0.01f, powf(fabsf(uc.y - 0.5f) * 2.0f, 2.0f) * 0.01f};
            float* o = dst + 4 * ((size_t)y * W + x);
            o[0] = nearest_uv(uv.x + off.x, uv.y + off.y, 0);
            o[1] = nearest_uv(uv.x, uv.y, 1);
            o[2] = nearest_uv(uv.x - off.x, uv.y - off.y, 2);
            o[3] = 1.0f;
        }
}

// upscale without FSR (upscale.cuh:260-291): every output pixel reads the
// render [sh][sw][4] bilinearly (textureReadBilinear, all channels) at
// (x / dw * sw, y / dh * sh).
void orc_upscale(int sw, int sh, const float* src, int dw, int dh, float* dst) {
    auto tex = [&](int x, int y) {
        x = std::min(std::max(x, 0), sw - 1);
        y = std::min(std::max(y, 0), sh - 1);
        const float* q = src + 4 * ((size_t)y * sw + x);
        return F4(q[0], q[1], q[2], q[3]);
    };
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            const float px = (float)x / (float)dw * (float)sw, py = (float)y / (float)dh * (float)sh;
            const int ix = (int)px, iy = (int)py;
            const float ws = px - (float)ix, wt = py - (float)iy;
            const f4 c = lerp4(lerp4(tex(ix, iy), tex(ix + 1, iy), ws), lerp4(tex(ix, iy + 1), tex(ix + 1, iy + 1), ws), wt);
            float* o = dst + 4 * ((size_t)y * dw + x);
            o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = c.w;
        }
}

// FSR 1.0 as the reference compiles it when USE_FSR is defined
// (kernels.cuh:3; launchUpscaleComputeKernel, kernels.cu:84-104).
// EASU (upscale.cuh:13-258) reads the render [sh][sw][4] with 12 taps, each a
// textureReadBilinearUV (device_texture_buffer.cuh:42-86: truncated pixel
// position, clamped texels, lerps with the remainder, even when it is
// negative) at a position of the FsrEasuCon constants; RCAS (upscale.cuh:
// 300-433, sharpness 0, FSR_RCAS_DENOISE undefined) sharpens the EASU image
// from its plus-shaped neighbourhood, read the same way at (p / size) * size.
// The reference's double-precision literals (0.5, .4, 1.5625, .29, 1. / lob,
// 4. * lobe + 1., the RCAS limit) keep their double arithmetic here.  The
// EASU image goes to easu_out, the sharpened one to dst ([dh][dw][4], alpha 1).
void orc_fsr(int sw, int sh, const float* src, int dw, int dh, float* easu_out, float* dst) {
    auto bilinear = [](const float* img, int w, int h, float px, float py) {
        auto tex = [&](int x, int y) {
            x = std::min(std::max(x, 0), w - 1);
            y = std::min(std::max(y, 0), h - 1);
            const float* q = img + 4 * ((size_t)y * w + x);
            return F4(q[0], q[1], q[2], q[3]);
        };
        const int ix = (int)px, iy = (int)py;
        const float ws = px - (float)ix, wt = py - (float)iy;
        return lerp4(lerp4(tex(ix, iy), tex(ix + 1, iy), ws), lerp4(tex(ix, iy + 1), tex(ix + 1, iy + 1), ws), wt);
    };
    // FsrEasuCon (upscale.cuh:18-62) with the render size as viewport and input
    const float inw = (float)sw, inh = (float)sh, ow = (float)dw, oh = (float)dh;
    const f4 con0 = F4(inw / ow, inh / oh, (float)(0.5 * (double)inw / (double)ow - 0.5),
                       (float)(0.5 * (double)inh / (double)oh - 0.5));
    const f4 con1 = F4(1.0f / inw, 1.0f / inh, 1.0f / inw, -1.0f / inh);
    const f4 con2 = F4(-1.0f / inw, 2.0f / inh, 1.0f / inw, 2.0f / inh);
    const f2 con3 = F2(0.0f / inw, 4.0f / inh);
    const f4 off = F4(-0.5f * con1.x, 0.5f * con1.x, -0.5f * con1.y, 0.5f * con1.y);
    // FsrEasuSetF (upscale.cuh:101-130): direction and edge length of one
    // bilinear corner from its '+' of lumas
    auto setf = [](f2& dir, float& len, float w, float lA, float lB, float lC, float lD, float lE) {
        float lenX = fmaxf(fabsf(lD - lC), fabsf(lC - lB));
        const float dirX = lD - lB;
        dir.x += dirX * w;
        lenX = clampf(fabsf(dirX) / lenX, 0.0f, 1.0f);
        lenX *= lenX;
        len += lenX * w;
        float lenY = fmaxf(fabsf(lE - lC), fabsf(lC - lA));
        const float dirY = lE - lA;
        dir.y += dirY * w;
        lenY = clampf(fabsf(dirY) / lenY, 0.0f, 1.0f);
        lenY *= lenY;
        len += lenY * w;
    };
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            // FsrEasuF (upscale.cuh:133-254)
            float ppx = (float)x * con0.x + con0.z, ppy = (float)y * con0.y + con0.w;
            const float fpx = floorf(ppx), fpy = floorf(ppy);
            ppx -= fpx;
            ppy -= fpy;
            const f2 p0 = F2(fpx * con1.x + con1.z, fpy * con1.y + con1.w);
            const f2 p1 = p0 + F2(con2.x, con2.y), p2 = p0 + F2(con2.z, con2.w), p3 = p0 + F2(con3.x, con3.y);
            auto tap = [&](f2 p, float ox, float oy) {
                const f2 q = p + F2(ox, oy);
                return xyz(bilinear(src, sw, sh, q.x * (float)sw, q.y * (float)sh));
            };
            auto luma = [](f3 c) { return (float)((double)c.y + 0.5 * (double)(c.x + c.z)); };
            const f3 bC = tap(p0, off.x, off.w), cC = tap(p0, off.y, off.w);
            const f3 iC = tap(p1, off.x, off.w), jC = tap(p1, off.y, off.w);
            const f3 fC = tap(p1, off.y, off.z), eC = tap(p1, off.x, off.z);
            const f3 kC = tap(p2, off.x, off.w), lC = tap(p2, off.y, off.w);
            const f3 hC = tap(p2, off.y, off.z), gC = tap(p2, off.x, off.z);
            const f3 oC = tap(p3, off.y, off.z), nC = tap(p3, off.x, off.z);
            const float bL = luma(bC), cL = luma(cC), iL = luma(iC), jL = luma(jC), fL = luma(fC), eL = luma(eC);
            const float kL = luma(kC), lL = luma(lC), hL = luma(hC), gL = luma(gC), oL = luma(oC), nL = luma(nC);
            f2 dir = F2(0.0f, 0.0f);
            float len = 0.0f;
            setf(dir, len, (float)((1.0 - (double)ppx) * (1.0 - (double)ppy)), bL, eL, fL, gL, jL);
            setf(dir, len, (float)((double)ppx * (1.0 - (double)ppy)), cL, fL, gL, hL, kL);
            setf(dir, len, (float)((1.0 - (double)ppx) * (double)ppy), fL, iL, jL, kL, nL);
            setf(dir, len, ppx * ppy, gL, jL, kL, lL, oL);
            // normalise the direction, shape the length (upscale.cuh:203-225)
            const float d2x = dir.x * dir.x, d2y = dir.y * dir.y;
            float dirR = d2x + d2y;
            const bool zro = dirR < 1.0f / 32768.0f;
            dirR = 1.0f / sqrtf(dirR);
            dirR = zro ? 1.0f : dirR;
            dir.x = zro ? 1.0f : dir.x;
            dir.x *= dirR;
            dir.y *= dirR;
            len = (float)((double)len * 0.5);
            len *= len;
            const float stretch = (dir.x * dir.x + dir.y * dir.y) / fmaxf(fabsf(dir.x), fabsf(dir.y));
            const f2 len2 = F2((float)(1.0 + ((double)stretch - 1.0) * (double)len), (float)(1.0 - 0.5 * (double)len));
            const float lob = (float)(0.5 - 0.29 * (double)len);
            const float clp = (float)(1.0 / (double)lob);
            const f3 min4 = fmin3(fmin3(fC, gC), fmin3(jC, kC));
            const f3 max4 = fmax3(fmax3(fC, gC), fmax3(jC, kC));
            f3 aC = F3(0.0f);
            float aW = 0.0f;
            // FsrEasuTapF (upscale.cuh:65-98): windowed Lanczos-2 approximation
            // along the rotated, stretched offset
            auto tapf = [&](float tx, float ty, f3 c) {
                const float ox = tx - ppx, oy = ty - ppy;
                float vx = ox * dir.x + oy * dir.y;
                float vy = ox * -dir.y + oy * dir.x;
                vx *= len2.x;
                vy *= len2.y;
                const float d2 = fminf(vx * vx + vy * vy, clp);
                float wB = (float)(0.4 * (double)d2 - 1.0);
                float wA = (float)((double)(lob * d2) - 1.0);
                wB *= wB;
                wA *= wA;
                wB = (float)(1.5625 * (double)wB - 0.5625);
                const float w = wB * wA;
                aC = aC + c * w;
                aW += w;
            };
            tapf(0, -1, bC); tapf(1, -1, cC); tapf(-1, 1, iC); tapf(0, 1, jC);
            tapf(0, 0, fC); tapf(-1, 0, eC); tapf(1, 1, kC); tapf(2, 1, lC);
            tapf(2, 0, hC); tapf(1, 0, gC); tapf(1, 2, oC); tapf(0, 2, nC);
            const f3 pix = fmin3(max4, fmax3(min4, aC / aW));
            float* o = easu_out + 4 * ((size_t)y * dw + x);
            o[0] = pix.x; o[1] = pix.y; o[2] = pix.z; o[3] = 1.0f;
        }
    // sharpen / FsrRcasF (upscale.cuh:316-375, 415-433)
    const float fw = (float)dw, fh = (float)dh;
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            auto load = [&](float px, float py) {
                return xyz(bilinear(easu_out, dw, dh, (px / fw) * fw, (py / fh) * fh));
            };
            const float sx = (float)x, sy = (float)y;
            const f3 b = load(sx + 0.0f, sy + -1.0f), d = load(sx + -1.0f, sy + 0.0f), e = load(sx, sy);
            const f3 f = load(sx + 1.0f, sy + 0.0f), h = load(sx + 0.0f, sy + 1.0f);
            const f3 mn4 = fmin3(b, fmin3(f, h)), mx4 = fmax3(b, fmax3(f, h));
            const f3 hitMin = mn4 / (4.0f * mx4);
            const f3 hitMax = (F3(1.0f) - mx4) / (4.0f * mn4 + -4.0f);
            const f3 lobeRGB = fmax3(-hitMin, hitMax);
            const float con = 1.0f;   // FsrRcasCon: exp2(-sharpness), sharpness 0
            const float lobe = (float)(fmax(-(0.25 - (1.0 / 16.0)),
                                            fmin((double)fmaxf(lobeRGB.x, fmaxf(lobeRGB.y, lobeRGB.z)), 0.0)) *
                                       (double)con);
            const f3 col = (lobe * (((b + d) + h) + f) + e) / (float)(4.0 * (double)lobe + 1.0);
            float* o = dst + 4 * ((size_t)y * dw + x);
            o[0] = col.x; o[1] = col.y; o[2] = col.z; o[3] = 1.0f;
        }
}

}  // extern "C"
