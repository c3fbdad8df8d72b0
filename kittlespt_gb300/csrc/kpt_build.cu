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

struct Split {                   // outcome of one node's split
    int nl;                      // triangles going left, 0: the node stays a leaf
    float llo[3], lhi[3], rlo[3], rhi[3];
};

struct Counters {                // written by k_assign, read by the host after each depth
    int next_id, nlevel, nbig, nsmall;
    int bad;                     // partition destinations outside the node (none when the closed form holds)
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
        if (threadIdx.x == 0) {
            // the sweep of findBestSplitPlane, in its order of operations
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
// node (left, then right), the next depth's list (children of more than
// LEAF_MAX triangles, in order) and its large / small node lists.
__global__ void __launch_bounds__(1024) k_assign(BlasNode* nodes, const int* level, int nlevel, const Split* sp,
                                                 int* next_level, int* big, int* small, Counters* cnt) {
    __shared__ int shi[32];
    __shared__ int s_next_id, s_nnext, s_nbig, s_nsmall;
    if (threadIdx.x == 0) {
        s_next_id = cnt->next_id;
        s_nnext = s_nbig = s_nsmall = 0;
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
            la = s.nl > LEAF_MAX;
            ra = p.count - s.nl > LEAF_MAX;
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
            if (la) {
                next_level[o] = lid;
                if (l.count > SMALL_MAX) big[atomicAdd(&s_nbig, 1)] = o;
                else small[atomicAdd(&s_nsmall, 1)] = o;
                ++o;
            }
            if (ra) {
                next_level[o] = lid + 1;
                if (r.count > SMALL_MAX) big[atomicAdd(&s_nbig, 1)] = o;
                else small[atomicAdd(&s_nsmall, 1)] = o;
            }
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
        cnt->nbig = s_nbig;
        cnt->nsmall = s_nsmall;   // cnt->bad accumulates
    }
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
    DevArray<float> pos;
    DevArray<float4> cen;
    DevArray<int> order, tmp, xr, yl, rank, level, next_level, big, small;
    DevArray<BlasNode> nodes;
    DevArray<Split> sp;
    DevArray<Counters> cnt;
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {pos.alloc(9 * (size_t)N), cen.alloc(N), order.alloc(N), tmp.alloc(N), xr.alloc(N),
                          yl.alloc(N), rank.alloc(N), nodes.alloc(2 * (size_t)N), level.alloc(lcap),
                          next_level.alloc(lcap), big.alloc(lcap), small.alloc(lcap), sp.alloc(lcap), cnt.alloc(1)})
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyAsync(pos.p, m.pos.data(), 9 * (size_t)N * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return (int)e;
    k_centroids<<<(N + 255) / 256, 256, 0, st>>>(pos.p, N, cen.p, order.p);
    k_root<<<1, BIG, 0, st>>>(pos.p, order.p, N, nodes.p);
    int nodes_used = 1;
    if (N > LEAF_MAX) {
        // depth 0: the root alone
        const int zero = 0;
        Counters c{1, 1, N > SMALL_MAX ? 1 : 0, N > SMALL_MAX ? 0 : 1, 0};
        e = cudaMemcpyAsync(level.p, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(N > SMALL_MAX ? big.p : small.p, &zero, sizeof(int),
                                                  cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.p, &c, sizeof c, cudaMemcpyHostToDevice, st);
        int* cur = level.p;
        int* nxt = next_level.p;
        while (e == cudaSuccess && c.nlevel > 0) {
            if (c.nbig)
                k_split<BIG><<<c.nbig, BIG, 0, st>>>(pos.p, cen.p, order.p, tmp.p, xr.p, yl.p, rank.p, nodes.p, cur,
                                                   big.p, sp.p, cnt.p);
            if (c.nsmall)
                k_split<32><<<c.nsmall, 32, 0, st>>>(pos.p, cen.p, order.p, tmp.p, xr.p, yl.p, rank.p, nodes.p, cur,
                                                   small.p, sp.p, cnt.p);
            k_assign<<<1, 1024, 0, st>>>(nodes.p, cur, c.nlevel, sp.p, nxt, big.p, small.p, cnt.p);
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
    std::vector<BlasNode> h_nodes(nodes_used);
    std::vector<int> h_order(N);
    e = cudaMemcpyAsync(h_nodes.data(), nodes.p, nodes_used * sizeof(BlasNode), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_order.data(), order.p, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return (int)e;
    pack_blas(m, h_nodes, std::move(h_order));
    return 0;
}

}  // namespace kpt
