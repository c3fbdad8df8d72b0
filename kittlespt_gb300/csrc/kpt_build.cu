// kpt_build.cu -- the reference's binned SAH BLAS build (as_builder.cuh:110-261)
// on the GPU, producing the tree of the host build (kpt_scene.cpp) exactly:
// the same splits, node boxes and triangle order inside every leaf.
//
// The host build recurses node by node; here the nodes of one depth are
// split together, one block per node (1024 threads for a node of more than
// SMALL_MAX triangles, one warp otherwise).  A split is the reference's:
//   * centroids (v0 + v1 + v2) * 0.3333f; per axis the centroid bounds, 8
//     bins by (int)((c - min) * (8 / (max - min))), per bin the triangle
//     count and box; the left/right sweep with the reference's box growth
//     (an empty bin's box grows a side to +-FLT_MAX), cost nl * Al + nr * Ar,
//     first strict minimum over axes x, y, z and split planes 1..7;
//   * the in-place partition `i = first, j = last: c[i] < split ? i++ :
//     swap(i, j--)`.  It is sequential in the reference; its outcome has a
//     closed form that each thread evaluates for its own element.  Reading
//     the left end forwards (stream x) and the right end backwards (stream
//     y), the scan examines a run of x up to and including the next element
//     that goes right, then a run of y up to and including the next element
//     that goes left, and so on until the ends meet at `a`.  With XR(m) the
//     position of the m-th right-going element from the left and YL(m)
//     (YL(0) = 0) the index, counted from the right end, of the m-th
//     left-going element from the right, an element at p < a stays if it
//     goes left and moves to n-1-YL(m-1) if it is the m-th going right; at
//     p >= a it moves to XR(m) if it is the m-th going left (from the right)
//     and to p-1 if it goes right.  `a` follows from the first run that
//     cannot complete (x-run m: XR(m) >= n - YL(m-1); y-run m:
//     n - YL(m) <= XR(m)), found by a block-wide minimum;
//   * a partition with an empty side leaves the node a leaf (permuted, as in
//     the reference); otherwise the children's boxes are their triangles'.
// All arithmetic is IEEE single precision with explicit rounding intrinsics
// (no contraction), so every comparison sees the host build's values.
// Boxes are reduced with fminf/fmaxf in a different order than the host's
// loops: equal in value, a zero may differ in sign.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <vector>

#include "kpt_scene.h"

namespace kpt {
namespace {

constexpr int LEAF_MAX = 8;      // a node of at most 8 triangles is a leaf (as_builder.cuh:186)
constexpr int BINS = 8;
constexpr int BIG = 1024;        // threads per block for a large node
constexpr int SMALL_MAX = 2048;  // larger nodes get a BIG block, smaller ones a warp
constexpr int WIDE_MIN = 65536;  // larger nodes are split by WG blocks of WT threads each
constexpr int WG = 256;
constexpr int WT = 256;
constexpr int TINY_MAX = 128;    // a node of at most this many triangles is finished by one thread

struct Split {                   // outcome of one node's split
    int nl;                      // triangles going left, 0: the node stays a leaf
    float llo[3], lhi[3], rlo[3], rhi[3];
};

struct Counters {                // written by k_assign, read by the host after each depth
    int next_id, nlevel, nbig, nsmall, nwide, ntiny;
    int bad;                     // partition destinations outside the node (none when the closed form holds)
};

// Accumulators of one wide node, combined across its WG blocks by atomics
// (boxes as order-preserving keys).
struct WideAcc {
    unsigned cmin[3], cmax[3];            // centroid bounds
    int bn[3][BINS];                      // per axis and bin: triangles
    unsigned blo[3][BINS][3], bhi[3][BINS][3];
    int axis;
    float split;
    int nl, ev;                           // left-going count; first run that cannot complete
    unsigned llo[3], lhi[3], rlo[3], rhi[3];
    int boff[WG];                         // per block: left-going count, then the count before the block
};

__device__ __forceinline__ float comp(float4 c, int a) { return a == 0 ? c.x : (a == 1 ? c.y : c.z); }

// Block-wide reductions and scans for blocks of T threads (T a multiple of 32,
// <= 1024).  `sh` holds at least 32 words; every thread of the block calls.
template <int T>
__device__ __forceinline__ float block_min(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (T == 32) return v;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    v = (threadIdx.x & 31) < T / 32 ? sh[threadIdx.x & 31] : v;
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int T>
__device__ __forceinline__ float block_max(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (T == 32) return v;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    v = (threadIdx.x & 31) < T / 32 ? sh[threadIdx.x & 31] : v;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int T>
__device__ __forceinline__ int block_sum(int v, int* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (T == 32) return v;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    v = (threadIdx.x & 31) < T / 32 ? sh[threadIdx.x & 31] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int T>
__device__ __forceinline__ int block_min_int(int v, int* sh) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (T == 32) return v;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    v = (threadIdx.x & 31) < T / 32 ? sh[threadIdx.x & 31] : INT_MAX;
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// exclusive prefix sum over the block; *total receives the block's sum
template <int T>
__device__ __forceinline__ int block_scan(int v, int* sh, int* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (T == 32) {
        *total = __shfl_sync(0xffffffffu, x, 31);
        return x - v;
    }
    __syncthreads();
    if (lane == 31) sh[w] = x;
    __syncthreads();
    int wsum = lane < T / 32 ? sh[lane] : 0;
    int ws = wsum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += y;
    }
    const int before = __shfl_sync(0xffffffffu, ws - wsum, w);
    *total = __shfl_sync(0xffffffffu, ws, 31);
    return before + x - v;
}

// Box of the triangles order[first .. first+n) over their vertices.
template <int T>
__device__ __forceinline__ void block_bounds(const float* pos, const int* order, int first, int n, float* lo,
                                             float* hi, float* sh) {
    float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int p = threadIdx.x; p < n; p += T) {
        const float* v = pos + 9 * (size_t)order[first + p];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            l[k % 3] = fminf(l[k % 3], v[k]);
            h[k % 3] = fmaxf(h[k % 3], v[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = block_min<T>(l[k], sh);
        hi[k] = block_max<T>(h[k], sh);
    }
}

__device__ __forceinline__ float area(const float* lo, const float* hi) {   // Bounds3f::area, no contraction
    const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]), dz = __fsub_rn(hi[2], lo[2]);
    return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}
// Bounds3f::grow(Bounds3f): the other box's max corner, then its min corner
__device__ __forceinline__ void grow_box(float* lo, float* hi, const float* olo, const float* ohi) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = fminf(lo[k], ohi[k]);
        hi[k] = fmaxf(hi[k], ohi[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = fminf(lo[k], olo[k]);
        hi[k] = fmaxf(hi[k], olo[k]);
    }
}

// The sweep of BLASBuilder::findBestSplitPlane over one axis's bins, in its
// order of operations: left and right counts and grown boxes, cost
// nl * Al + nr * Ar, first strict minimum (over the axes in order).
__device__ __forceinline__ void sweep(const int* bn, const float (*blo)[3], const float (*bhi)[3], float mn,
                                      float mx, int a, float& best, int& axis, float& split) {
    constexpr int P = BINS - 1;
    float la[P], ra[P];
    int lc[P], rc[P];
    float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int ls = 0, rs = 0;
    for (int i = 0; i < P; ++i) {
        ls += bn[i];
        lc[i] = ls;
        grow_box(llo, lhi, blo[i], bhi[i]);
        la[i] = area(llo, lhi);
        rs += bn[P - i];
        rc[P - 1 - i] = rs;
        grow_box(rlo, rhi, blo[P - i], bhi[P - i]);
        ra[P - 1 - i] = area(rlo, rhi);
    }
    const float step = __fdiv_rn(__fsub_rn(mx, mn), (float)BINS);
    for (int i = 0; i < P; ++i) {
        const float cost = __fadd_rn(__fmul_rn((float)lc[i], la[i]), __fmul_rn((float)rc[i], ra[i]));
        if (cost < best) {
            axis = a;
            split = __fadd_rn(mn, __fmul_rn(step, (float)(i + 1)));
            best = cost;
        }
    }
}

// Order-preserving keys of floats for atomicMin / atomicMax on unsigned
// (-0 below +0).
__device__ __forceinline__ unsigned fkey(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float kfloat(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void k_centroids(const float* pos, int n, float4* cen, int* order) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float* v = pos + 9 * (size_t)t;
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = __fmul_rn(__fadd_rn(__fadd_rn(v[k], v[3 + k]), v[6 + k]), 0.3333f);
    cen[t] = make_float4(c[0], c[1], c[2], 0.0f);
    order[t] = t;
}

__global__ void __launch_bounds__(BIG) k_root(const float* pos, const int* order, int n, BlasNode* nodes) {
    __shared__ float sh[32];
    float lo[3], hi[3];
    block_bounds<BIG>(pos, order, 0, n, lo, hi, sh);
    if (threadIdx.x == 0) {
        BlasNode r;
        r.left_first = 0;
        r.count = n;
        for (int k = 0; k < 3; ++k) {
            r.lo[k] = lo[k];
            r.hi[k] = hi[k];
        }
        nodes[0] = r;
    }
}

// One node per block: the split (BLASBuilder::findBestSplitPlane), the
// partition and the children's boxes.  which[blockIdx.x] indexes the depth's
// node list; the outcome goes to out[that index].
template <int T>
__global__ void __launch_bounds__(T) k_split(const float* pos, const float4* cen, int* order, int* tmp, int* xr,
                                             int* yl, int* rank, const BlasNode* nodes, const int* level,
                                             const int* which, Split* out, Counters* cnt) {
    __shared__ float shf[32];
    __shared__ int shi[32];
    __shared__ int s_axis;
    __shared__ float s_pos;
    const int k = which[blockIdx.x];
    const BlasNode nd = nodes[level[k]];
    const int f = nd.left_first, n = nd.count;

    // --- best split: 8 bins per axis over the centroid bounds
    float best = INFINITY;
    int axis = -1;
    float split = 0.0f;
    for (int a = 0; a < 3; ++a) {
        float mn = INFINITY, mx = -INFINITY;
        for (int p = threadIdx.x; p < n; p += T) {
            const float c = comp(cen[order[f + p]], a);
            mn = fminf(mn, c);
            mx = fmaxf(mx, c);
        }
        mn = block_min<T>(mn, shf);
        mx = block_max<T>(mx, shf);
        if (mn == mx) continue;   // uniform in the block
        const float scale = __fdiv_rn((float)BINS, __fsub_rn(mx, mn));
        int bn[BINS];
        float blo[BINS][3], bhi[BINS][3];
#pragma unroll
        for (int b = 0; b < BINS; ++b) {
            bn[b] = 0;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                blo[b][q] = FLT_MAX;
                bhi[b][q] = -FLT_MAX;
            }
        }
        for (int p = threadIdx.x; p < n; p += T) {
            const int t = order[f + p];
            const int bi = min(BINS - 1, __float2int_rz(__fmul_rn(__fsub_rn(comp(cen[t], a), mn), scale)));
            const float* v = pos + 9 * (size_t)t;
            float tl[3], th[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                tl[q] = fminf(fminf(v[q], v[3 + q]), v[6 + q]);
                th[q] = fmaxf(fmaxf(v[q], v[3 + q]), v[6 + q]);
            }
#pragma unroll
            for (int b = 0; b < BINS; ++b) {
                if (bi == b) {
                    bn[b]++;
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        blo[b][q] = fminf(blo[b][q], tl[q]);
                        bhi[b][q] = fmaxf(bhi[b][q], th[q]);
                    }
                }
            }
        }
#pragma unroll
        for (int b = 0; b < BINS; ++b) {
            bn[b] = block_sum<T>(bn[b], shi);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                blo[b][q] = block_min<T>(blo[b][q], shf);
                bhi[b][q] = block_max<T>(bhi[b][q], shf);
            }
        }
        if (threadIdx.x == 0) sweep(bn, blo, bhi, mn, mx, a, best, axis, split);
    }
    if (threadIdx.x == 0) {
        s_axis = axis;   // -1 when no axis had distinct centroids: the reference then splits z at 0
        s_pos = split;
    }
    __syncthreads();
    axis = s_axis;
    split = s_pos;

    // --- the partition: left-going count, ranks, run ends, destinations
    int nl = 0;
    for (int p = threadIdx.x; p < n; p += T) nl += comp(cen[order[f + p]], axis) < split ? 1 : 0;
    nl = block_sum<T>(nl, shi);
    const int nr = n - nl;
    int carry_l = 0;
    for (int base = 0; base < n; base += T) {
        const int p = base + threadIdx.x;
        const bool in = p < n;
        const bool left = in && comp(cen[order[f + p]], axis) < split;
        int tot;
        const int lb = carry_l + block_scan<T>(left ? 1 : 0, shi, &tot);   // left-going before p
        if (in) {
            if (left) {
                const int m = nl - lb;            // rank from the right end
                yl[f + m - 1] = n - p;            // YL(m)
                rank[f + p] = m;
            } else {
                const int m = p - lb + 1;         // rank from the left end
                xr[f + m - 1] = p;                // XR(m)
                rank[f + p] = m;
            }
        }
        carry_l += tot;
    }
    __syncthreads();
    int ev = INT_MAX;
    const int mmax = min(nr, nl) + 1;
    for (int m = 1 + threadIdx.x; m <= mmax; m += T) {
        const int ylp = m > 1 ? yl[f + m - 2] : 0;
        const bool xfail = m > nr || xr[f + m - 1] >= n - ylp;
        if (xfail) {
            ev = min(ev, 2 * m - 1);
        } else if (m > nl || n - yl[f + m - 1] <= xr[f + m - 1]) {
            ev = min(ev, 2 * m);
        }
    }
    ev = block_min_int<T>(ev, shi);
    const int me = (ev + 1) >> 1;
    const int a = (ev & 1) ? n - (me > 1 ? yl[f + me - 2] : 0) : xr[f + me - 1] + 1;
    for (int p = threadIdx.x; p < n; p += T) {
        const bool left = comp(cen[order[f + p]], axis) < split;
        const int m = rank[f + p];
        int dst;
        if (p < a) dst = left ? p : n - 1 - (m > 1 ? yl[f + m - 2] : 0);
        else dst = left ? xr[f + m - 1] : p - 1;
        if (dst < 0 || dst >= n) {   // cannot happen; guards the write
            atomicAdd(&cnt->bad, 1);
            continue;
        }
        tmp[f + dst] = order[f + p];
    }
    __syncthreads();
    for (int p = threadIdx.x; p < n; p += T) order[f + p] = tmp[f + p];
    __syncthreads();

    // --- children's boxes (BLASBuilder::updateNodeBounds)
    Split s;
    s.nl = (nl == 0 || nl == n) ? 0 : nl;
    if (s.nl) {
        block_bounds<T>(pos, order, f, nl, s.llo, s.lhi, shf);
        block_bounds<T>(pos, order, f + nl, n - nl, s.rlo, s.rhi, shf);
    }
    if (threadIdx.x == 0) out[k] = s;
}

// Children of the depth's split nodes: ids next_id + 2j for the j-th split
// node (left, then right); the next depth's list (children of more than
// TINY_MAX triangles, in order) with its wide / large / small node lists
// (positions in that list), and the tiny children (LEAF_MAX < count <=
// TINY_MAX, node ids) that k_subtree finishes.
__device__ __forceinline__ void classify(int o, int id, int count, int* wide, int* big, int* small, int* tiny,
                                         int* nwide, int* nbig, int* nsmall, int* ntiny) {
    if (count > WIDE_MIN) wide[atomicAdd(nwide, 1)] = o;
    else if (count > SMALL_MAX) big[atomicAdd(nbig, 1)] = o;
    else if (count > TINY_MAX) small[atomicAdd(nsmall, 1)] = o;
    else if (count > LEAF_MAX) tiny[atomicAdd(ntiny, 1)] = id;
}

__global__ void __launch_bounds__(1024) k_assign(BlasNode* nodes, const int* level, int nlevel, const Split* sp,
                                                 int* next_level, int* wide, int* big, int* small, int* tiny,
                                                 Counters* cnt) {
    __shared__ int shi[32];
    __shared__ int s_next_id, s_nnext, s_nwide, s_nbig, s_nsmall, s_ntiny;
    if (threadIdx.x == 0) {
        s_next_id = cnt->next_id;
        s_nnext = s_nwide = s_nbig = s_nsmall = s_ntiny = 0;
    }
    __syncthreads();
    for (int base = 0; base < nlevel; base += 1024) {
        const int k = base + threadIdx.x;
        const bool in = k < nlevel;
        const Split s = in ? sp[k] : Split{};
        const bool split = in && s.nl > 0;
        int nsplit;
        const int j = block_scan<1024>(split ? 1 : 0, shi, &nsplit);
        int na = 0;
        bool la = false, ra = false;
        BlasNode p{};
        if (split) {
            p = nodes[level[k]];
            la = s.nl > TINY_MAX;
            ra = p.count - s.nl > TINY_MAX;
            na = (la ? 1 : 0) + (ra ? 1 : 0);
        }
        int nact;
        const int q = block_scan<1024>(na, shi, &nact);
        if (split) {
            const int lid = s_next_id + 2 * j;
            BlasNode l, r;
            l.left_first = p.left_first;
            l.count = s.nl;
            r.left_first = p.left_first + s.nl;
            r.count = p.count - s.nl;
            for (int c = 0; c < 3; ++c) {
                l.lo[c] = s.llo[c];
                l.hi[c] = s.lhi[c];
                r.lo[c] = s.rlo[c];
                r.hi[c] = s.rhi[c];
            }
            nodes[lid] = l;
            nodes[lid + 1] = r;
            nodes[level[k]].left_first = lid;
            nodes[level[k]].count = 0;
            int o = s_nnext + q;
            if (la) next_level[o] = lid;
            classify(o, lid, l.count, wide, big, small, tiny, &s_nwide, &s_nbig, &s_nsmall, &s_ntiny);
            if (la) ++o;
            if (ra) next_level[o] = lid + 1;
            classify(o, lid + 1, r.count, wide, big, small, tiny, &s_nwide, &s_nbig, &s_nsmall, &s_ntiny);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_next_id += 2 * nsplit;
            s_nnext += nact;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        cnt->next_id = s_next_id;
        cnt->nlevel = s_nnext;
        cnt->nwide = s_nwide;
        cnt->nbig = s_nbig;
        cnt->nsmall = s_nsmall;
        cnt->ntiny = s_ntiny;   // cnt->bad accumulates
    }
}

// --- wide nodes: WG blocks per node, each over a contiguous chunk ----------

__device__ __forceinline__ void wide_chunk(const BlasNode& nd, int sub, int* b, int* e) {
    const int c = (nd.count + WG - 1) / WG;
    *b = min(nd.count, sub * c);
    *e = min(nd.count, *b + c);
}

__global__ void kw_init(WideAcc* acc) {
    WideAcc& A = acc[blockIdx.x];
    const int t = threadIdx.x;
    if (t < 3) {
        A.cmin[t] = fkey(INFINITY);
        A.cmax[t] = fkey(-INFINITY);
        A.llo[t] = A.rlo[t] = fkey(FLT_MAX);
        A.lhi[t] = A.rhi[t] = fkey(-FLT_MAX);
    }
    if (t < 3 * BINS) {
        (&A.bn[0][0])[t] = 0;
        for (int q = 0; q < 3; ++q) {
            (&A.blo[0][0][0])[3 * t + q] = fkey(FLT_MAX);
            (&A.bhi[0][0][0])[3 * t + q] = fkey(-FLT_MAX);
        }
    }
    if (t == 0) {
        A.nl = 0;
        A.ev = INT_MAX;
    }
}

__global__ void __launch_bounds__(WT) kw_cbounds(const float4* cen, const int* order, const BlasNode* nodes,
                                                 const int* level, const int* wide, WideAcc* acc) {
    __shared__ float sh[32];
    const int w = blockIdx.x / WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, blockIdx.x % WG, &b, &e);
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int p = b + threadIdx.x; p < e; p += WT) {
        const float4 c = cen[order[nd.left_first + p]];
        mn[0] = fminf(mn[0], c.x); mn[1] = fminf(mn[1], c.y); mn[2] = fminf(mn[2], c.z);
        mx[0] = fmaxf(mx[0], c.x); mx[1] = fmaxf(mx[1], c.y); mx[2] = fmaxf(mx[2], c.z);
    }
    for (int a = 0; a < 3; ++a) {
        const float lo = block_min<WT>(mn[a], sh), hi = block_max<WT>(mx[a], sh);
        if (threadIdx.x == 0 && b < e) {
            atomicMin(&acc[w].cmin[a], fkey(lo));
            atomicMax(&acc[w].cmax[a], fkey(hi));
        }
    }
}

__global__ void __launch_bounds__(WT) kw_bins(const float* pos, const float4* cen, const int* order,
                                              const BlasNode* nodes, const int* level, const int* wide, WideAcc* acc) {
    __shared__ float shf[32];
    __shared__ int shi[32];
    const int w = blockIdx.x / WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, blockIdx.x % WG, &b, &e);
    WideAcc& A = acc[w];
    for (int a = 0; a < 3; ++a) {
        const float mn = kfloat(A.cmin[a]), mx = kfloat(A.cmax[a]);
        if (mn == mx) continue;
        const float scale = __fdiv_rn((float)BINS, __fsub_rn(mx, mn));
        int bn[BINS];
        float blo[BINS][3], bhi[BINS][3];
#pragma unroll
        for (int k = 0; k < BINS; ++k) {
            bn[k] = 0;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                blo[k][q] = FLT_MAX;
                bhi[k][q] = -FLT_MAX;
            }
        }
        for (int p = b + threadIdx.x; p < e; p += WT) {
            const int t = order[nd.left_first + p];
            const int bi = min(BINS - 1, __float2int_rz(__fmul_rn(__fsub_rn(comp(cen[t], a), mn), scale)));
            const float* v = pos + 9 * (size_t)t;
            float tl[3], th[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                tl[q] = fminf(fminf(v[q], v[3 + q]), v[6 + q]);
                th[q] = fmaxf(fmaxf(v[q], v[3 + q]), v[6 + q]);
            }
#pragma unroll
            for (int k = 0; k < BINS; ++k) {
                if (bi == k) {
                    bn[k]++;
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        blo[k][q] = fminf(blo[k][q], tl[q]);
                        bhi[k][q] = fmaxf(bhi[k][q], th[q]);
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < BINS; ++k) {
            const int c = block_sum<WT>(bn[k], shi);
            float lo[3], hi[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                lo[q] = block_min<WT>(blo[k][q], shf);
                hi[q] = block_max<WT>(bhi[k][q], shf);
            }
            if (threadIdx.x == 0 && c) {
                atomicAdd(&A.bn[a][k], c);
                for (int q = 0; q < 3; ++q) {
                    atomicMin(&A.blo[a][k][q], fkey(lo[q]));
                    atomicMax(&A.bhi[a][k][q], fkey(hi[q]));
                }
            }
        }
    }
}

__global__ void kw_decide(WideAcc* acc, int nw) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    WideAcc& A = acc[w];
    float best = INFINITY, split = 0.0f;
    int axis = -1;
    for (int a = 0; a < 3; ++a) {
        const float mn = kfloat(A.cmin[a]), mx = kfloat(A.cmax[a]);
        if (mn == mx) continue;
        float blo[BINS][3], bhi[BINS][3];
        for (int k = 0; k < BINS; ++k)
            for (int q = 0; q < 3; ++q) {
                blo[k][q] = kfloat(A.blo[a][k][q]);
                bhi[k][q] = kfloat(A.bhi[a][k][q]);
            }
        sweep(A.bn[a], blo, bhi, mn, mx, a, best, axis, split);
    }
    A.axis = axis;
    A.split = split;
}

__global__ void __launch_bounds__(WT) kw_count(const float4* cen, const int* order, const BlasNode* nodes,
                                               const int* level, const int* wide, WideAcc* acc) {
    __shared__ int shi[32];
    const int w = blockIdx.x / WG, sub = blockIdx.x % WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, sub, &b, &e);
    WideAcc& A = acc[w];
    const int axis = A.axis;
    const float split = A.split;
    int c = 0;
    for (int p = b + threadIdx.x; p < e; p += WT) c += comp(cen[order[nd.left_first + p]], axis) < split ? 1 : 0;
    c = block_sum<WT>(c, shi);
    if (threadIdx.x == 0) {
        A.boff[sub] = c;
        atomicAdd(&A.nl, c);
    }
}

// one warp per node: the per-block counts become the counts before each block
__global__ void kw_offsets(WideAcc* acc) {
    WideAcc& A = acc[blockIdx.x];
    int carry = 0;
    for (int base = 0; base < WG; base += 32) {
        const int v = A.boff[base + threadIdx.x];
        int tot;
        const int x = block_scan<32>(v, nullptr, &tot);
        A.boff[base + threadIdx.x] = carry + x;
        carry += tot;
    }
}

__global__ void __launch_bounds__(WT) kw_rank(const float4* cen, const int* order, int* xr, int* yl, int* rank,
                                              const BlasNode* nodes, const int* level, const int* wide,
                                              const WideAcc* acc) {
    __shared__ int shi[32];
    const int w = blockIdx.x / WG, sub = blockIdx.x % WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, sub, &b, &e);
    const WideAcc& A = acc[w];
    const int f = nd.left_first, n = nd.count, nl = A.nl, axis = A.axis;
    const float split = A.split;
    int carry_l = A.boff[sub];
    for (int base = b; base < e; base += WT) {
        const int p = base + threadIdx.x;
        const bool in = p < e;
        const bool left = in && comp(cen[order[f + p]], axis) < split;
        int tot;
        const int lb = carry_l + block_scan<WT>(left ? 1 : 0, shi, &tot);
        if (in) {
            if (left) {
                const int m = nl - lb;
                yl[f + m - 1] = n - p;
                rank[f + p] = m;
            } else {
                const int m = p - lb + 1;
                xr[f + m - 1] = p;
                rank[f + p] = m;
            }
        }
        carry_l += tot;
    }
}

__global__ void __launch_bounds__(WT) kw_meet(const int* xr, const int* yl, const BlasNode* nodes, const int* level,
                                              const int* wide, WideAcc* acc) {
    __shared__ int shi[32];
    const int w = blockIdx.x / WG, sub = blockIdx.x % WG;
    const BlasNode nd = nodes[level[wide[w]]];
    WideAcc& A = acc[w];
    const int f = nd.left_first, n = nd.count, nl = A.nl, nr = n - nl;
    const int mmax = min(nr, nl) + 1;
    int ev = INT_MAX;
    for (int m = 1 + sub * WT + threadIdx.x; m <= mmax; m += WG * WT) {
        const int ylp = m > 1 ? yl[f + m - 2] : 0;
        if (m > nr || xr[f + m - 1] >= n - ylp) ev = min(ev, 2 * m - 1);
        else if (m > nl || n - yl[f + m - 1] <= xr[f + m - 1]) ev = min(ev, 2 * m);
    }
    ev = block_min_int<WT>(ev, shi);
    if (threadIdx.x == 0 && ev != INT_MAX) atomicMin(&A.ev, ev);
}

__global__ void __launch_bounds__(WT) kw_scatter(const float4* cen, const int* order, int* tmp, const int* xr,
                                                 const int* yl, const int* rank, const BlasNode* nodes,
                                                 const int* level, const int* wide, const WideAcc* acc,
                                                 Counters* cnt) {
    const int w = blockIdx.x / WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, blockIdx.x % WG, &b, &e);
    const WideAcc& A = acc[w];
    const int f = nd.left_first, n = nd.count, axis = A.axis, ev = A.ev;
    const float split = A.split;
    const int me = (ev + 1) >> 1;
    const int a = (ev & 1) ? n - (me > 1 ? yl[f + me - 2] : 0) : xr[f + me - 1] + 1;
    for (int p = b + threadIdx.x; p < e; p += WT) {
        const bool left = comp(cen[order[f + p]], axis) < split;
        const int m = rank[f + p];
        int dst;
        if (p < a) dst = left ? p : n - 1 - (m > 1 ? yl[f + m - 2] : 0);
        else dst = left ? xr[f + m - 1] : p - 1;
        if (dst < 0 || dst >= n) {   // cannot happen; guards the write
            atomicAdd(&cnt->bad, 1);
            continue;
        }
        tmp[f + dst] = order[f + p];
    }
}

__global__ void __launch_bounds__(WT) kw_copy(int* order, const int* tmp, const BlasNode* nodes, const int* level,
                                              const int* wide) {
    const int w = blockIdx.x / WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, blockIdx.x % WG, &b, &e);
    for (int p = b + threadIdx.x; p < e; p += WT) order[nd.left_first + p] = tmp[nd.left_first + p];
}

__global__ void __launch_bounds__(WT) kw_cbox(const float* pos, const int* order, const BlasNode* nodes,
                                              const int* level, const int* wide, WideAcc* acc) {
    __shared__ float sh[32];
    const int w = blockIdx.x / WG;
    const BlasNode nd = nodes[level[wide[w]]];
    int b, e;
    wide_chunk(nd, blockIdx.x % WG, &b, &e);
    WideAcc& A = acc[w];
    const int nl = A.nl;
    if (nl == 0 || nl == nd.count) return;   // uniform in the block
    float l[2][3], h[2][3];
    for (int s = 0; s < 2; ++s)
        for (int q = 0; q < 3; ++q) {
            l[s][q] = FLT_MAX;
            h[s][q] = -FLT_MAX;
        }
    for (int p = b + threadIdx.x; p < e; p += WT) {
        const float* v = pos + 9 * (size_t)order[nd.left_first + p];
        const int s = p < nl ? 0 : 1;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            if (s == 0) {
                l[0][k % 3] = fminf(l[0][k % 3], v[k]);
                h[0][k % 3] = fmaxf(h[0][k % 3], v[k]);
            } else {
                l[1][k % 3] = fminf(l[1][k % 3], v[k]);
                h[1][k % 3] = fmaxf(h[1][k % 3], v[k]);
            }
        }
    }
    for (int s = 0; s < 2; ++s)
        for (int q = 0; q < 3; ++q) {
            const float lo = block_min<WT>(l[s][q], sh), hi = block_max<WT>(h[s][q], sh);
            if (threadIdx.x == 0 && lo <= hi) {   // the chunk holds triangles of side s
                atomicMin(s ? &A.rlo[q] : &A.llo[q], fkey(lo));
                atomicMax(s ? &A.rhi[q] : &A.lhi[q], fkey(hi));
            }
        }
}

__global__ void kw_finish(const WideAcc* acc, const BlasNode* nodes, const int* level, const int* wide, int nw,
                          Split* out) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const WideAcc& A = acc[w];
    const int n = nodes[level[wide[w]]].count;
    Split s;
    s.nl = (A.nl == 0 || A.nl == n) ? 0 : A.nl;
    for (int q = 0; q < 3; ++q) {
        s.llo[q] = kfloat(A.llo[q]);
        s.lhi[q] = kfloat(A.lhi[q]);
        s.rlo[q] = kfloat(A.rlo[q]);
        s.rhi[q] = kfloat(A.rhi[q]);
    }
    out[wide[w]] = s;
}

// --- tiny nodes: one warp finishes the node's subtree ----------------------
// BLASBuilder::subdivide as the host runs it (as_builder.cuh:181-233) over
// the node's triangles held in shared memory: per split the lanes find the
// centroid bounds, 24 lanes build one (axis, bin) each, lane 0 sweeps and
// runs the in-place partition itself, the lanes reduce the children's
// boxes; children are numbered from the shared counter.  One block (one
// warp) per tiny node; all control flow below is uniform in the block.
__global__ void __launch_bounds__(32) k_subtree(const float* pos, const float4* cen, int* order, BlasNode* nodes,
                                                const int* tiny, Counters* cnt) {
    __shared__ float s_c[TINY_MAX][3], s_lo[TINY_MAX][3], s_hi[TINY_MAX][3];
    __shared__ int s_id[TINY_MAX], s_perm[TINY_MAX], s_stack[TINY_MAX];
    __shared__ int s_bn[3][BINS];
    __shared__ float s_blo[3][BINS][3], s_bhi[3][BINS][3];
    __shared__ int s_nl, s_lid;
    const int lane = threadIdx.x;
    const int root = tiny[blockIdx.x];
    const BlasNode r0 = nodes[root];
    const int f0 = r0.left_first, n0 = r0.count;
    for (int p = lane; p < n0; p += 32) {
        const int t = order[f0 + p];
        const float4 c = cen[t];
        const float* v = pos + 9 * (size_t)t;
        s_c[p][0] = c.x;
        s_c[p][1] = c.y;
        s_c[p][2] = c.z;
        for (int q = 0; q < 3; ++q) {
            s_lo[p][q] = fminf(fminf(v[q], v[3 + q]), v[6 + q]);
            s_hi[p][q] = fmaxf(fmaxf(v[q], v[3 + q]), v[6 + q]);
        }
        s_id[p] = t;
        s_perm[p] = p;
    }
    if (lane == 0) s_stack[0] = root;
    int sp = 1;
    __syncthreads();
    while (sp > 0) {
        const int ni = s_stack[--sp];
        const BlasNode nd = nodes[ni];
        const int lf = nd.left_first - f0, n = nd.count;
        // centroid bounds per axis
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a) {
            mn[a] = INFINITY;
            mx[a] = -INFINITY;
        }
        for (int p = lane; p < n; p += 32) {
            const int el = s_perm[lf + p];
            for (int a = 0; a < 3; ++a) {
                mn[a] = fminf(mn[a], s_c[el][a]);
                mx[a] = fmaxf(mx[a], s_c[el][a]);
            }
        }
        for (int a = 0; a < 3; ++a) {
            mn[a] = block_min<32>(mn[a], nullptr);
            mx[a] = block_max<32>(mx[a], nullptr);
        }
        // lane 8a + k: bin k of axis a
        if (lane < 3 * BINS) {
            const int a = lane / BINS, k = lane % BINS;
            int c = 0;
            float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            if (mn[a] != mx[a]) {
                const float scale = __fdiv_rn((float)BINS, __fsub_rn(mx[a], mn[a]));
                for (int p = 0; p < n; ++p) {
                    const int el = s_perm[lf + p];
                    const int bi = min(BINS - 1, __float2int_rz(__fmul_rn(__fsub_rn(s_c[el][a], mn[a]), scale)));
                    if (bi == k) {
                        c++;
                        for (int q = 0; q < 3; ++q) {
                            lo[q] = fminf(lo[q], s_lo[el][q]);
                            hi[q] = fmaxf(hi[q], s_hi[el][q]);
                        }
                    }
                }
            }
            s_bn[a][k] = c;
            for (int q = 0; q < 3; ++q) {
                s_blo[a][k][q] = lo[q];
                s_bhi[a][k][q] = hi[q];
            }
        }
        __syncthreads();
        if (lane == 0) {
            float best = INFINITY, split = 0.0f;
            int axis = -1;
            for (int a = 0; a < 3; ++a)
                if (mn[a] != mx[a]) sweep(s_bn[a], s_blo[a], s_bhi[a], mn[a], mx[a], a, best, axis, split);
            const int ax = axis < 0 ? 2 : axis;   // comp() reads z for axis -1
            int l = lf, r = lf + n - 1;
            while (l <= r) {
                if (s_c[s_perm[l]][ax] < split) {
                    l++;
                } else {
                    const int x = s_perm[l];
                    s_perm[l] = s_perm[r];
                    s_perm[r--] = x;
                }
            }
            s_nl = l - lf;
            s_lid = (s_nl == 0 || s_nl == n) ? -1 : atomicAdd(&cnt->next_id, 2);
        }
        __syncthreads();
        const int nl = s_nl, lid = s_lid;
        if (lid < 0) continue;   // a leaf: uniform in the block
        float lo[2][3], hi[2][3];
        for (int s2 = 0; s2 < 2; ++s2)
            for (int q = 0; q < 3; ++q) {
                lo[s2][q] = FLT_MAX;
                hi[s2][q] = -FLT_MAX;
            }
        for (int p = lane; p < n; p += 32) {
            const int el = s_perm[lf + p];
            const int s2 = p < nl ? 0 : 1;
            for (int q = 0; q < 3; ++q) {
                lo[s2][q] = fminf(lo[s2][q], s_lo[el][q]);
                hi[s2][q] = fmaxf(hi[s2][q], s_hi[el][q]);
            }
        }
        for (int s2 = 0; s2 < 2; ++s2)
            for (int q = 0; q < 3; ++q) {
                lo[s2][q] = block_min<32>(lo[s2][q], nullptr);
                hi[s2][q] = block_max<32>(hi[s2][q], nullptr);
            }
        if (lane == 0) {
            BlasNode c[2];
            c[0].left_first = nd.left_first;
            c[0].count = nl;
            c[1].left_first = nd.left_first + nl;
            c[1].count = n - nl;
            for (int s2 = 0; s2 < 2; ++s2)
                for (int q = 0; q < 3; ++q) {
                    c[s2].lo[q] = lo[s2][q];
                    c[s2].hi[q] = hi[s2][q];
                }
            nodes[lid] = c[0];
            nodes[lid + 1] = c[1];
            nodes[ni].left_first = lid;
            nodes[ni].count = 0;
        }
        // children with more than LEAF_MAX triangles: right pushed first, so left is taken next
        if (n - nl > LEAF_MAX) {
            if (lane == 0) s_stack[sp] = lid + 1;
            ++sp;
        }
        if (nl > LEAF_MAX) {
            if (lane == 0) s_stack[sp] = lid;
            ++sp;
        }
        __syncthreads();
    }
    for (int p = lane; p < n0; p += 32) order[f0 + p] = s_id[s_perm[p]];
}

// --- packing into the device format (pack_blas of kpt_scene.cpp) ------------
// Interior nodes are numbered depth first, left child first: the left child
// of v is dfs(v) + 1, the right one dfs(v) + 1 + (interior nodes under the
// left child).  Children always have larger ids than their parent.

__global__ void k_parents(const BlasNode* nodes, int nn, int* parent, int* need) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    if (v == 0) parent[0] = -1;
    const BlasNode nd = nodes[v];
    need[v] = 0;
    if (nd.count != 0) return;
    parent[nd.left_first] = v;
    parent[nd.left_first + 1] = v;
    need[v] = (nodes[nd.left_first].count == 0 ? 1 : 0) + (nodes[nd.left_first + 1].count == 0 ? 1 : 0);
}

// interior nodes under and including each interior node, bottom up: a node
// is finished by the thread of the last of its interior children to finish
__global__ void k_sizes(const BlasNode* nodes, int nn, const int* parent, const int* need, int* size, int* arrive) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn || nodes[v].count != 0 || need[v] != 0) return;
    int c = v;
    size[c] = 1;
    for (;;) {
        const int p = parent[c];
        if (p < 0) break;
        __threadfence();
        if (atomicAdd(&arrive[p], 1) + 1 != need[p]) break;   // the other interior child finishes p
        __threadfence();
        const int l = nodes[p].left_first;
        const int sl = nodes[l].count == 0 ? ((volatile int*)size)[l] : 0;
        const int sr = nodes[l + 1].count == 0 ? ((volatile int*)size)[l + 1] : 0;
        size[p] = 1 + sl + sr;
        c = p;
    }
}

__device__ __forceinline__ int dfs_index(const BlasNode* nodes, const int* parent, const int* size, int v,
                                         int* depth) {
    int d = 0, k = 1;
    for (int c = v, p = parent[v]; p >= 0; c = p, p = parent[p]) {
        const int l = nodes[p].left_first;
        d += c == l ? 1 : 1 + (nodes[l].count == 0 ? size[l] : 0);
        ++k;
    }
    *depth = k;
    return d;
}

__global__ void k_pack(const BlasNode* nodes, int nn, const int* parent, const int* size, BvhNode* out,
                       int* max_depth) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    const BlasNode nd = nodes[v];
    if (nd.count != 0) return;
    int dep, dl, dr;
    const int dv = dfs_index(nodes, parent, size, v, &dep);
    atomicMax(max_depth, dep);
    const BlasNode l = nodes[nd.left_first], r = nodes[nd.left_first + 1];
    dl = dv + 1;
    dr = dv + 1 + (l.count == 0 ? size[nd.left_first] : 0);
    BvhNode o;
    o.a = make_float4(l.lo[0], l.lo[1], l.lo[2], l.hi[0]);
    o.b = make_float4(l.hi[1], l.hi[2], r.lo[0], r.lo[1]);
    o.c = make_float4(r.lo[2], r.hi[0], r.hi[1], r.hi[2]);
    o.d = make_int4(l.count ? l.left_first : dl, l.count, r.count ? r.left_first : dr, r.count);
    out[dv] = o;
}

template <class X>
struct DevArray {
    X* p = nullptr;
    ~DevArray() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(X)); }
};

}  // namespace

int build_blas_device(HostMesh& m, cudaStream_t st) {
    const int N = m.ntris();
    if (N <= 0) return (int)cudaErrorInvalidValue;
    const size_t lcap = (size_t)N / (LEAF_MAX + 1) + 2;   // nodes of one depth with more than LEAF_MAX triangles
    const size_t wcap = (size_t)N / WIDE_MIN + 2;
    DevArray<float> pos;
    DevArray<float4> cen;
    DevArray<int> order, tmp, xr, yl, rank, level, next_level, wide, big, small, tiny;
    DevArray<BlasNode> nodes;
    DevArray<Split> sp;
    DevArray<WideAcc> acc;
    DevArray<Counters> cnt;
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {pos.alloc(9 * (size_t)N), cen.alloc(N), order.alloc(N), tmp.alloc(N), xr.alloc(N),
                          yl.alloc(N), rank.alloc(N), nodes.alloc(2 * (size_t)N), level.alloc(lcap),
                          next_level.alloc(lcap), wide.alloc(wcap), big.alloc(lcap), small.alloc(lcap),
                          tiny.alloc(lcap), sp.alloc(lcap), acc.alloc(wcap), cnt.alloc(1)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyAsync(pos.p, m.pos.data(), 9 * (size_t)N * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return (int)e;
    k_centroids<<<(N + 255) / 256, 256, 0, st>>>(pos.p, N, cen.p, order.p);
    k_root<<<1, BIG, 0, st>>>(pos.p, order.p, N, nodes.p);
    int nodes_used = 1;
    if (N > LEAF_MAX) {
        // depth 0: the root alone, in the list its size picks
        const int zero = 0;
        Counters c{1, N > TINY_MAX ? 1 : 0, 0, 0, 0, 0, 0};
        int* first_list = N > WIDE_MIN ? wide.p : N > SMALL_MAX ? big.p : N > TINY_MAX ? small.p : tiny.p;
        (N > WIDE_MIN ? c.nwide : N > SMALL_MAX ? c.nbig : N > TINY_MAX ? c.nsmall : c.ntiny) = 1;
        e = cudaMemcpyAsync(level.p, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(first_list, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.p, &c, sizeof c, cudaMemcpyHostToDevice, st);
        int* cur = level.p;
        int* nxt = next_level.p;
        while (e == cudaSuccess && (c.nlevel > 0 || c.ntiny > 0)) {
            if (c.ntiny) k_subtree<<<c.ntiny, 32, 0, st>>>(pos.p, cen.p, order.p, nodes.p, tiny.p, cnt.p);
            if (c.nlevel == 0) {
                e = cudaMemcpyAsync(&c, cnt.p, sizeof c, cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                break;
            }
            if (c.nwide) {
                const int g = c.nwide * WG;
                kw_init<<<c.nwide, 32, 0, st>>>(acc.p);
                kw_cbounds<<<g, WT, 0, st>>>(cen.p, order.p, nodes.p, cur, wide.p, acc.p);
                kw_bins<<<g, WT, 0, st>>>(pos.p, cen.p, order.p, nodes.p, cur, wide.p, acc.p);
                kw_decide<<<(c.nwide + 31) / 32, 32, 0, st>>>(acc.p, c.nwide);
                kw_count<<<g, WT, 0, st>>>(cen.p, order.p, nodes.p, cur, wide.p, acc.p);
                kw_offsets<<<c.nwide, 32, 0, st>>>(acc.p);
                kw_rank<<<g, WT, 0, st>>>(cen.p, order.p, xr.p, yl.p, rank.p, nodes.p, cur, wide.p, acc.p);
                kw_meet<<<g, WT, 0, st>>>(xr.p, yl.p, nodes.p, cur, wide.p, acc.p);
                kw_scatter<<<g, WT, 0, st>>>(cen.p, order.p, tmp.p, xr.p, yl.p, rank.p, nodes.p, cur, wide.p, acc.p,
                                             cnt.p);
                kw_copy<<<g, WT, 0, st>>>(order.p, tmp.p, nodes.p, cur, wide.p);
                kw_cbox<<<g, WT, 0, st>>>(pos.p, order.p, nodes.p, cur, wide.p, acc.p);
                kw_finish<<<(c.nwide + 31) / 32, 32, 0, st>>>(acc.p, nodes.p, cur, wide.p, c.nwide, sp.p);
            }
            if (c.nbig)
                k_split<BIG><<<c.nbig, BIG, 0, st>>>(pos.p, cen.p, order.p, tmp.p, xr.p, yl.p, rank.p, nodes.p, cur,
                                                   big.p, sp.p, cnt.p);
            if (c.nsmall)
                k_split<32><<<c.nsmall, 32, 0, st>>>(pos.p, cen.p, order.p, tmp.p, xr.p, yl.p, rank.p, nodes.p, cur,
                                                   small.p, sp.p, cnt.p);
            k_assign<<<1, 1024, 0, st>>>(nodes.p, cur, c.nlevel, sp.p, nxt, wide.p, big.p, small.p, tiny.p, cnt.p);
            e = cudaMemcpyAsync(&c, cnt.p, sizeof c, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            std::swap(cur, nxt);
        }
        nodes_used = c.next_id;
        if (e == cudaSuccess && c.bad) e = cudaErrorUnknown;
    }
    if (e != cudaSuccess) return (int)e;
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    // the device format, as pack_blas writes it
    BlasNode root;
    e = cudaMemcpyAsync(&root, nodes.p, sizeof root, cudaMemcpyDeviceToHost, st);
    const int ninterior = (nodes_used - 1) / 2;
    DevArray<int> parent, need, size, arrive, depth;
    DevArray<BvhNode> packed;
    for (cudaError_t r : {parent.alloc(nodes_used), need.alloc(nodes_used), size.alloc(nodes_used),
                          arrive.alloc(nodes_used), depth.alloc(1), packed.alloc(ninterior)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    if (e == cudaSuccess) e = cudaMemsetAsync(arrive.p, 0, nodes_used * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(depth.p, 0, sizeof(int), st);
    if (e != cudaSuccess) return (int)e;
    const int gb = (nodes_used + 255) / 256;
    k_parents<<<gb, 256, 0, st>>>(nodes.p, nodes_used, parent.p, need.p);
    k_sizes<<<gb, 256, 0, st>>>(nodes.p, nodes_used, parent.p, need.p, size.p, arrive.p);
    k_pack<<<gb, 256, 0, st>>>(nodes.p, nodes_used, parent.p, size.p, packed.p, depth.p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    m.nodes.resize(ninterior);
    m.order.resize(N);
    if (ninterior) e = cudaMemcpyAsync(m.nodes.data(), packed.p, ninterior * sizeof(BvhNode), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m.order.data(), order.p, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&m.max_depth, depth.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return (int)e;
    for (int k = 0; k < 3; ++k) {
        m.lo[k] = root.lo[k];
        m.hi[k] = root.hi[k];
    }
    if (root.count != 0) {   // the root is a leaf
        m.root = -1;
        m.leaf_first = 0;
        m.leaf_count = root.count;
        m.max_depth = 0;
    } else {
        m.root = 0;
    }
    return 0;
}

// --- refit: new positions, same tree -------------------------------------
// Every node's child boxes are recomputed bottom up from the triangles below
// them (min / max, so each box equals the one a build of the same tree would
// give); triangle records in leaf order are rewritten.  Nodes are the
// device-format nodes of one mesh at node_base in the scene's node array
// (child references global: nodes node_base + local, triangles tri_base +
// leaf position).

namespace {

__global__ void k_refit_tris(const float* pos, const int* order, int n, int tri_base, float4* tris) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = order[k];
    const float* p = pos + 9 * (size_t)t;
    float4* o = tris + 3 * ((size_t)tri_base + k);
    o[0] = make_float4(p[0], p[1], p[2], __int_as_float(t));
    o[1] = make_float4(__fsub_rn(p[3], p[0]), __fsub_rn(p[4], p[1]), __fsub_rn(p[5], p[2]), 0.0f);
    o[2] = make_float4(__fsub_rn(p[6], p[0]), __fsub_rn(p[7], p[1]), __fsub_rn(p[8], p[2]), 0.0f);
}

// tri_normal_area (kpt_scene.cpp) on the device, the same IEEE operations:
// the geometric normal facing the mean vertex normal (Triangle constructor,
// triangle.cuh:51-64)
__global__ void k_refit_shade(const float* pos, const float* nrm, int n, TriShade* shade) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float* p = pos + 9 * (size_t)t;
    const float* q = nrm + 9 * (size_t)t;
    const float e0x = __fsub_rn(p[3], p[0]), e0y = __fsub_rn(p[4], p[1]), e0z = __fsub_rn(p[5], p[2]);
    const float e1x = __fsub_rn(p[6], p[0]), e1y = __fsub_rn(p[7], p[1]), e1z = __fsub_rn(p[8], p[2]);
    const float gx = __fsub_rn(__fmul_rn(e0y, e1z), __fmul_rn(e0z, e1y));
    const float gy = __fsub_rn(__fmul_rn(e0z, e1x), __fmul_rn(e0x, e1z));
    const float gz = __fsub_rn(__fmul_rn(e0x, e1y), __fmul_rn(e0y, e1x));
    const float ax = __fdiv_rn(__fadd_rn(__fadd_rn(q[0], q[3]), q[6]), 3.0f);
    const float ay = __fdiv_rn(__fadd_rn(__fadd_rn(q[1], q[4]), q[7]), 3.0f);
    const float az = __fdiv_rn(__fadd_rn(__fadd_rn(q[2], q[5]), q[8]), 3.0f);
    const float d = __fadd_rn(__fadd_rn(__fmul_rn(gx, ax), __fmul_rn(gy, ay)), __fmul_rn(gz, az));
    const float ox = d < 0.0f ? -gx : gx, oy = d < 0.0f ? -gy : gy, oz = d < 0.0f ? -gz : gz;
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ox, ox), __fmul_rn(oy, oy)), __fmul_rn(oz, oz))));
    shade[t].gnx = __fmul_rn(ox, inv);
    shade[t].gny = __fmul_rn(oy, inv);
    shade[t].gnz = __fmul_rn(oz, inv);
}

__device__ __forceinline__ void leaf_box(const float* pos, const int* order, int tri_base, int first, int count,
                                         float* lo, float* hi) {
    for (int q = 0; q < 3; ++q) {
        lo[q] = FLT_MAX;
        hi[q] = -FLT_MAX;
    }
    for (int k = first; k < first + count; ++k) {
        const float* v = pos + 9 * (size_t)order[k - tri_base];
        for (int j = 0; j < 9; ++j) {
            lo[j % 3] = fminf(lo[j % 3], v[j]);
            hi[j % 3] = fmaxf(hi[j % 3], v[j]);
        }
    }
}
__device__ __forceinline__ void set_child(BvhNode& n, int slot, const float* lo, const float* hi) {
    if (slot == 0) {
        n.a = make_float4(lo[0], lo[1], lo[2], hi[0]);
        n.b.x = hi[1];
        n.b.y = hi[2];
    } else {
        n.b.z = lo[0];
        n.b.w = lo[1];
        n.c = make_float4(lo[2], hi[0], hi[1], hi[2]);
    }
}

// parents (local), interior children to wait for, and the leaf children's boxes
__global__ void k_refit_leaves(BvhNode* nodes, int node_base, int nn, int tri_base, const float* pos,
                               const int* order, int* parent, int* need, int* arrive) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    BvhNode n = nodes[node_base + v];
    int nd = 0;
    for (int slot = 0; slot < 2; ++slot) {
        const int ref = slot ? n.d.z : n.d.x, cnt = slot ? n.d.w : n.d.y;
        if (cnt == 0) {
            parent[ref - node_base] = v;
            ++nd;
        } else {
            float lo[3], hi[3];
            leaf_box(pos, order, tri_base, ref, cnt, lo, hi);
            set_child(n, slot, lo, hi);
        }
    }
    nodes[node_base + v] = n;
    need[v] = nd;
    arrive[v] = 0;
    if (v == 0) parent[0] = -1;
}

// a node whose children's boxes are final passes their union to its parent;
// the last of a parent's interior children to arrive carries on upwards
__global__ void k_refit_up(BvhNode* nodes, int node_base, int nn, const int* parent, const int* need, int* arrive) {
    const int v0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (v0 >= nn || need[v0] != 0) return;
    int v = v0;
    for (;;) {
        const int p = parent[v];
        if (p < 0) break;
        // this node's child boxes, written by other threads before their arrival
        volatile const float* f = reinterpret_cast<volatile const float*>(nodes + node_base + v);
        const float lo[3] = {fminf(f[0], f[6]), fminf(f[1], f[7]), fminf(f[2], f[8])};
        const float hi[3] = {fmaxf(f[3], f[9]), fmaxf(f[4], f[10]), fmaxf(f[5], f[11])};
        BvhNode* pn = nodes + node_base + p;
        const int slot = (pn->d.y == 0 && pn->d.x == node_base + v) ? 0 : 1;
        if (slot == 0) {
            pn->a = make_float4(lo[0], lo[1], lo[2], hi[0]);
            pn->b.x = hi[1];
            pn->b.y = hi[2];
        } else {
            pn->b.z = lo[0];
            pn->b.w = lo[1];
            pn->c = make_float4(lo[2], hi[0], hi[1], hi[2]);
        }
        __threadfence();
        if (atomicAdd(&arrive[p], 1) + 1 != need[p]) break;
        __threadfence();
        v = p;
    }
}

}  // namespace

int refit_blas_device(HostMesh& m, BvhNode* d_nodes, int node_base, float4* d_tris, int tri_base, TriShade* d_shade,
                      cudaStream_t st) {
    const int N = m.ntris(), nn = (int)m.nodes.size();
    DevArray<float> pos, nrm;
    DevArray<int> order, parent, need, arrive;
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {pos.alloc(9 * (size_t)N), nrm.alloc(9 * (size_t)N), order.alloc(N), parent.alloc(nn),
                          need.alloc(nn), arrive.alloc(nn)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(pos.p, m.pos.data(), 9 * (size_t)N * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(nrm.p, m.nrm.data(), 9 * (size_t)N * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(order.p, m.order.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return (int)e;
    k_refit_tris<<<(N + 255) / 256, 256, 0, st>>>(pos.p, order.p, N, tri_base, d_tris);
    k_refit_shade<<<(N + 255) / 256, 256, 0, st>>>(pos.p, nrm.p, N, d_shade + tri_base);
    if (nn > 0) {
        k_refit_leaves<<<(nn + 255) / 256, 256, 0, st>>>(d_nodes, node_base, nn, tri_base, pos.p, order.p, parent.p,
                                                         need.p, arrive.p);
        k_refit_up<<<(nn + 255) / 256, 256, 0, st>>>(d_nodes, node_base, nn, parent.p, need.p, arrive.p);
        // the host copy of the nodes: boxes from the device, references local as built
        std::vector<BvhNode> h(nn);
        e = cudaMemcpyAsync(h.data(), d_nodes + node_base, nn * sizeof(BvhNode), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return (int)e;
        for (int k = 0; k < nn; ++k) {
            m.nodes[k].a = h[k].a;
            m.nodes[k].b = h[k].b;
            m.nodes[k].c = h[k].c;
        }
        const BvhNode& r = m.nodes[0];
        m.lo[0] = fminf(r.a.x, r.b.z); m.lo[1] = fminf(r.a.y, r.b.w); m.lo[2] = fminf(r.a.z, r.c.x);
        m.hi[0] = fmaxf(r.a.w, r.c.y); m.hi[1] = fmaxf(r.b.x, r.c.z); m.hi[2] = fmaxf(r.b.y, r.c.w);
    } else {   // the root is a leaf: the mesh's box
        for (int q = 0; q < 3; ++q) {
            m.lo[q] = FLT_MAX;
            m.hi[q] = -FLT_MAX;
        }
        for (size_t j = 0; j < m.pos.size(); ++j) {
            m.lo[j % 3] = fminf(m.lo[j % 3], m.pos[j]);
            m.hi[j % 3] = fmaxf(m.hi[j % 3], m.pos[j]);
        }
        e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return (int)e;
}

}  // namespace kpt
