// GPU BVH construction for a scene (replaces SweepSahBuilder + ParallelReinsertionOptimizer +
// NodeLayoutOptimizer of the reference, lib/bvh/sweep_sah_builder.hpp:43-111,
// parallel_reinsertion_optimizer.hpp:140-211, node_layout_optimizer.hpp:30-92).
//
// Pipeline, one stream, no host round trips except one frontier count per collapse level:
//   k_transform      entity transform in FP64 (transform.hpp:43-85), FP32 triangle records
//                    (p0, p1, p2, n), exact FP32 boxes, centroids, normals
//   k_bounds         scene and centroid bounds (order-preserving integer atomics)
//   k_morton         30-bit Morton codes of centroids in the centroid bounds
//   radix_sort       stable LSD radix sort, 8-bit digits, 4 passes (histogram / scan / scatter)
//   k_karras         binary radix tree (Karras, "Maximizing parallelism in the construction of
//                    BVHs, octrees, and k-d trees", HPG 2012); ties broken by index
//   k_refit          bottom-up boxes and collapse costs, second arrival at each node does the
//                    union
//   k_collapse       top-down, level-synchronous collapse into 8-wide nodes by a surface-area
//                    cost dynamic program over the binary tree (costs computed in the refit:
//                    each wide node spreads its 8 slots over subtrees where that is cheaper than
//                    keeping them whole); children with <= 3 triangles become leaves, slots ordered by octant, child boxes quantised to 8 bits
//                    (Ylitie, Karras, Laine, "Efficient incoherent ray traversal on GPUs through
//                    compressed wide BVHs", HPG 2017); leaf triangles written contiguously.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int BLOCK = 256;

struct EntXform {
    double scale;
    double pos[3];
    double rot[9];
    uint32_t first;      // first scene primitive of this entity
    uint32_t has_vn;
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return {ds(a.x, b.x), ds(a.y, b.y), ds(a.z, b.z)}; }
__device__ __forceinline__ D3 d3add(D3 a, D3 b) { return {da(a.x, b.x), da(a.y, b.y), da(a.z, b.z)}; }
__device__ __forceinline__ D3 d3scl(D3 a, double s) { return {dm(a.x, s), dm(a.y, s), dm(a.z, s)}; }
// transform.hpp:22-28 rotate(): rows of R, left-to-right sums, no fused multiply-add
__device__ __forceinline__ D3 d3rot(D3 v, const double* R) {
    return {da(da(dm(R[0], v.x), dm(R[1], v.y)), dm(R[2], v.z)), da(da(dm(R[3], v.x), dm(R[4], v.y)), dm(R[5], v.z)),
            da(da(dm(R[6], v.x), dm(R[7], v.y)), dm(R[8], v.z))};
}
// bvh::cross (vector.hpp:161-169)
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) {
    return {ds(dm(a.y, b.z), dm(a.z, b.y)), ds(dm(a.z, b.x), dm(a.x, b.z)), ds(dm(a.x, b.y), dm(a.y, b.x))};
}

// Order-preserving float <-> uint32 key for atomic min/max.
__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float fkey_inv(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// ---------------------------------------------------------------- K0 transform
__global__ void k_transform(const float* __restrict__ xyz, const float* __restrict__ vn, const EntXform* __restrict__ xf,
                            uint32_t n_ents, uint32_t n, float4* __restrict__ geo, float4* __restrict__ vn_out,
                            uint32_t* __restrict__ prim_ent, float4* __restrict__ box, float4* __restrict__ cen) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // entity of primitive i: last entity whose first <= i (few entities; linear search is fine)
    uint32_t e = 0;
    for (uint32_t k = 1; k < n_ents; ++k)
        if (xf[k].first <= i) e = k;
    const EntXform& X = xf[e];
    const float* q = xyz + 9ull * i;
    const D3 p0 = {q[0], q[1], q[2]}, p1 = {q[3], q[4], q[5]}, p2 = {q[6], q[7], q[8]};
    // resize_triangles, rotate_triangles, translate_triangles (p' = R (s p) + t), applied to each vertex
    // directly so that a vertex shared by several triangles gets one FP32 value in all of them (the
    // watertight test relies on it).  The reference carries each triangle as p0, e1 = p0 - p1,
    // e2 = p2 - p0 through the three steps (triangle.hpp:31-33, 81-82); the results differ by FP64
    // rounding only.
    const D3 t = {X.pos[0], X.pos[1], X.pos[2]};
    const D3 a = d3add(d3rot(d3scl(p0, X.scale), X.rot), t);
    const D3 b = d3add(d3rot(d3scl(p1, X.scale), X.rot), t);
    const D3 c = d3add(d3rot(d3scl(p2, X.scale), X.rot), t);
    const D3 nn = d3cross(d3sub(a, b), d3sub(c, a));   // n = e1 x e2
    const float P[3][3] = {{(float)a.x, (float)a.y, (float)a.z}, {(float)b.x, (float)b.y, (float)b.z},
                           {(float)c.x, (float)c.y, (float)c.z}};
    geo[3ull * i + 0] = make_float4(P[0][0], P[0][1], P[0][2], P[1][0]);
    geo[3ull * i + 1] = make_float4(P[1][1], P[1][2], P[2][0], P[2][1]);
    geo[3ull * i + 2] = make_float4(P[2][2], (float)nn.x, (float)nn.y, (float)nn.z);
    // box of the FP32 triangle (exact), centroid of its vertices
    float lo[3], hi[3], cc[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = fminf(P[0][k], fminf(P[1][k], P[2][k]));
        hi[k] = fmaxf(P[0][k], fmaxf(P[1][k], P[2][k]));
        cc[k] = (float)(((double)P[0][k] + (double)P[1][k] + (double)P[2][k]) * (1.0 / 3.0));
    }
    box[2ull * i] = make_float4(lo[0], lo[1], lo[2], 0.f);
    box[2ull * i + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    cen[i] = make_float4(cc[0], cc[1], cc[2], 0.f);
    prim_ent[i] = e;
    if (vn_out) {
        if (X.has_vn && vn) {
            const float* w = vn + 9ull * i;
            for (int k = 0; k < 3; ++k) {
                D3 v = d3rot(D3{w[3 * k], w[3 * k + 1], w[3 * k + 2]}, X.rot);
                vn_out[3ull * i + k] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
            }
        } else {
            for (int k = 0; k < 3; ++k) vn_out[3ull * i + k] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// ---------------------------------------------------------------- K1 bounds
// keys[0..5] = scene box min xyz (as fkey, atomicMin) / max xyz (atomicMax); keys[6..11] centroid box
__global__ void k_bounds(const float4* __restrict__ box, const float4* __restrict__ cen, uint32_t n,
                         uint32_t* __restrict__ keys) {
    __shared__ uint32_t s[12];
    if (threadIdx.x < 12) s[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    uint32_t lo[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t hi[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = box[2ull * i], b = box[2ull * i + 1], c = cen[i];
        float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z}, cv[3] = {c.x, c.y, c.z};
        for (int k = 0; k < 3; ++k) {
            lo[k] = min(lo[k], fkey(av[k]));
            hi[k] = max(hi[k], fkey(bv[k]));
            lo[3 + k] = min(lo[3 + k], fkey(cv[k]));
            hi[3 + k] = max(hi[3 + k], fkey(cv[k]));
        }
    }
    for (int k = 0; k < 6; ++k) {
        for (int o = 16; o; o >>= 1) {
            lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(&s[k], lo[k]);
            atomicMax(&s[3 + k], hi[k]);
            atomicMin(&s[6 + k], lo[3 + k]);
            atomicMax(&s[9 + k], hi[3 + k]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        if ((threadIdx.x % 6) < 3) atomicMin(&keys[threadIdx.x], s[threadIdx.x]);
        else atomicMax(&keys[threadIdx.x], s[threadIdx.x]);
    }
}

// ---------------------------------------------------------------- K2 Morton codes
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__global__ void k_morton(const float4* __restrict__ cen, uint32_t n, const uint32_t* __restrict__ keys,
                         uint32_t* __restrict__ code, uint32_t* __restrict__ idx) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3], ext[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = fkey_inv(keys[6 + k]);
        float h = fkey_inv(keys[9 + k]);
        ext[k] = h - lo[k];
    }
    float4 c = cen[i];
    float cv[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        float t = ext[k] > 0.f ? (cv[k] - lo[k]) / ext[k] : 0.5f;
        q[k] = (uint32_t)fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
    }
    code[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    idx[i] = i;
}

// ---------------------------------------------------------------- K3 stable LSD radix sort
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

__global__ void __launch_bounds__(SORT_THREADS) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                               int shift, uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; ++r) {
        uint32_t i = base + r * SORT_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of m values with one block of 1024 threads
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ a, uint32_t m) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += a[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
}

// Stable scatter: items of a tile are ranked in tile order (round, warp, lane); within a warp,
// equal digits are ranked with __match_any_sync, across warps with per-round digit counts.
__global__ void __launch_bounds__(SORT_THREADS) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                                  const uint32_t* __restrict__ vin,
                                                                  uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                  uint32_t n, int shift,
                                                                  const uint32_t* __restrict__ offs) {
    constexpr int WARPS = SORT_THREADS / 32;
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[WARPS][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offs[tid * gridDim.x + blockIdx.x];
    const uint32_t tile = blockIdx.x * SORT_TILE;
    const uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < SORT_ITEMS; ++r) {
        for (int w = 0; w < WARPS; ++w) wcnt[w][tid] = 0;
        __syncthreads();
        const uint32_t i = tile + r * SORT_THREADS + tid;
        const bool valid = i < n;
        uint32_t k = 0, v = 0, d = 256 + lane;
        if (valid) {
            k = kin[i];
            v = vin[i];
            d = (k >> shift) & 0xFF;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = base[d] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < WARPS; ++w) add += wcnt[w][tid];
        base[tid] += add;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- K4 Karras radix tree
__device__ __forceinline__ int delta(const uint32_t* __restrict__ code, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}
// children: >= 0 internal index, < 0 leaf ~j (sorted position j)
__global__ void k_karras(const uint32_t* __restrict__ code, int n, int2* __restrict__ child, int2* __restrict__ range,
                         int* __restrict__ parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(code, n, i, i + 1) - delta(code, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(code, n, i, i - d);
    int lmax = 2;
    while (delta(code, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(code, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(code, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(code, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = (lo == gamma) ? ~gamma : gamma;
    const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(lo, hi);
    parent[left >= 0 ? left : (n - 1) + ~left] = i;
    parent[right >= 0 ? right : (n - 1) + ~right] = i;
}

// ---------------------------------------------------------------- refit + collapse costs
// Surface-area costs for the 8-wide collapse (a dynamic program over the binary tree): for an
// internal node b, dp[8 b] = cost of b as one root of a wide node's slot (a leaf when it holds at
// most 3 triangles, else an 8-wide node: COST_NODE area + the best spread of 8 slots over its
// children), dp[8 b + j - 1] = cost of spreading j = 2..8 slots over its two children.  The ratio
// triangle-test cost `cost_tri` is relative to an 8-wide node test (COST_NODE = 1): the default
// 0.15 is the trace kernel's instruction ratio (~40 : ~280), best for coherent rays; incoherent
// multi-bounce workloads prefer smaller leaves (a larger cost, crt_tuning.collapse_tri_cost).
constexpr float COST_NODE = 1.0f;

__device__ __forceinline__ float box_area(const float4& lo, const float4& hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// cost of child `ref` given i slots (1..8): out[i]
__device__ __forceinline__ void dp_child(const float* __restrict__ dp, int ref, float leaf_area, float cost_tri,
                                         float out[9]) {
    if (ref < 0) {
        const float v = cost_tri * leaf_area;
        for (int i = 1; i <= 8; ++i) out[i] = v;
        return;
    }
    const float* d = dp + 8ull * ref;
    const float single = __ldcg(d);
    out[1] = single;
    for (int i = 2; i <= 8; ++i) out[i] = fminf(single, __ldcg(d + i - 1));
}

// node boxes: 2 float4 per node; internal nodes [0, n-1), leaves [n-1, 2n-1)
__global__ void k_refit(const uint32_t* __restrict__ sorted, const float4* __restrict__ tbox, int n,
                        const int2* __restrict__ child, const int* __restrict__ parent, float4* nbox,
                        uint32_t* __restrict__ flags, const int2* __restrict__ range, float* __restrict__ dp,
                        float cost_tri, uint32_t* __restrict__ err) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t p = sorted[j];
    float4 lo = tbox[2ull * p], hi = tbox[2ull * p + 1];
    nbox[2ull * (n - 1 + j)] = lo;
    nbox[2ull * (n - 1 + j) + 1] = hi;
    int node = parent[n - 1 + j];
    for (int steps = 0; node >= 0; ++steps) {
        if (steps >= 1024) {   // deeper than any tree built here, or damaged links: report, do not loop
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0) return;   // first arrival: the sibling finishes the union
        const int2 c = child[node];
        const size_t a = c.x >= 0 ? (size_t)c.x : (size_t)(n - 1 + ~c.x);
        const size_t b = c.y >= 0 ? (size_t)c.y : (size_t)(n - 1 + ~c.y);
        const float4 alo = __ldcg(&nbox[2 * a]), ahi = __ldcg(&nbox[2 * a + 1]);
        const float4 blo = __ldcg(&nbox[2 * b]), bhi = __ldcg(&nbox[2 * b + 1]);
        lo = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f);
        hi = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f);
        __stcg(&nbox[2ull * node], lo);
        __stcg(&nbox[2ull * node + 1], hi);
        if (dp) {
            float cl[9], cr[9];
            dp_child(dp, c.x, box_area(alo, ahi), cost_tri, cl);
            dp_child(dp, c.y, box_area(blo, bhi), cost_tri, cr);
            float* out = dp + 8ull * node;
            float dist8 = 3.0e38f;
            for (int j = 2; j <= 8; ++j) {
                float best = 3.0e38f;
                for (int k = 1; k < j; ++k) best = fminf(best, cl[k] + cr[j - k]);
                __stcg(out + j - 1, best);
                dist8 = best;
            }
            const int2 r = range[node];
            const float a = box_area(lo, hi);
            const float c_int = COST_NODE * a + dist8;
            const float c_leaf = r.y - r.x + 1 <= 3 ? cost_tri * (float)(r.y - r.x + 1) * a : 3.0e38f;
            __stcg(out, fminf(c_int, c_leaf));
        }
        node = parent[node];
    }
}

// ---------------------------------------------------------------- treelet restructuring
// Tree optimisation after the topology build, in place of the reference's parallel reinsertion
// (ParallelReinsertionOptimizer::optimize, parallel_reinsertion_optimizer.hpp:140-211): treelet
// restructuring after Karras and Aila, "Fast parallel construction of high-quality bounding volume
// hierarchies" (HPG 2013).  A treelet is a node R with up to TL_LEAVES descendants as leaves, grown
// from R's two children by repeatedly opening the leaf of largest surface area; its internal nodes
// are rebuilt into the topology of least summed surface area (the surface-area cost with the leaf
// subtrees fixed: their costs are the same in every topology), found by a dynamic program over the
// 2^7 - 1 subsets of leaves, one warp per treelet.  Node indices, boxes of R and everything outside
// the treelet stay; only child / parent links of its internal nodes and their boxes change.
// Treelets of one launch must not share nodes: a launch takes the roots whose depth is = r (mod 7),
// and a treelet from depth d holds internal nodes at depths d .. d + 5 and leaves at depths up to
// d + 6, so two roots 7 or more levels apart, or in disjoint subtrees, touch disjoint nodes.  Depths
// are recomputed before every launch.  Afterwards k_tl_count / k_tl_position / k_tl_relayout renumber
// the leaves in depth-first order, so every subtree is again a contiguous range of sorted positions
// (what the refit and the 8-wide collapse read).
constexpr int TL_LEAVES = 7;
constexpr int TL_WARPS = 4;

__device__ __forceinline__ size_t tl_index(int n, int ref) { return ref >= 0 ? (size_t)ref : (size_t)(n - 1 + ~ref); }

// depth of every internal node (root 0), by walking up the parent links
__global__ void k_tl_depth(const int* __restrict__ parent, int n, uint8_t* __restrict__ depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = 0, node = i;
    while (true) {
        const int p = parent[node];
        if (p < 0 || d >= 255) break;
        node = p;
        ++d;
    }
    depth[i] = (uint8_t)d;
}

__global__ void __launch_bounds__(32 * TL_WARPS) k_treelet(int2* __restrict__ child, int* __restrict__ parent,
                                                          float4* __restrict__ nbox,
                                                          const uint8_t* __restrict__ depth, int n, int cls,
                                                          uint32_t* __restrict__ stats) {
    __shared__ float s_area[TL_WARPS][128];
    __shared__ float s_cost[TL_WARPS][128];
    __shared__ uint8_t s_part[TL_WARPS][128];
    __shared__ float s_box[TL_WARPS][TL_LEAVES][6];
    __shared__ int s_leaf[TL_WARPS][TL_LEAVES];
    __shared__ int s_int[TL_WARPS][TL_LEAVES - 1];
    __shared__ int s_nl[TL_WARPS];
    __shared__ float s_old[TL_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int warps = gridDim.x * TL_WARPS;
    uint32_t improved = 0;
    for (int R = blockIdx.x * TL_WARPS + w; R < n - 1; R += warps) {
        if (depth[R] == 255 || (int)depth[R] % 7 != cls) continue;   // warp-uniform; 255: deeper than tracked
        if (lane == 0) {
            // grow the treelet: open the leaf of largest area that is an internal node
            int leaf[TL_LEAVES], nl = 2, ni = 1;
            float area[TL_LEAVES];
            const int2 c = child[R];
            leaf[0] = c.x;
            leaf[1] = c.y;
            s_int[w][0] = R;
            float old = box_area(nbox[2 * (size_t)R], nbox[2 * (size_t)R + 1]);
            for (int k = 0; k < 2; ++k) area[k] = leaf[k] >= 0 ? box_area(nbox[2 * tl_index(n, leaf[k])], nbox[2 * tl_index(n, leaf[k]) + 1]) : -1.f;
            while (nl < TL_LEAVES) {
                int best = -1;
                float ba = -1.f;
                for (int k = 0; k < nl; ++k)
                    if (leaf[k] >= 0 && area[k] > ba) { ba = area[k]; best = k; }
                if (best < 0) break;
                const int L = leaf[best];
                s_int[w][ni++] = L;
                old += ba;
                const int2 cc = child[L];
                leaf[best] = cc.x;
                leaf[nl] = cc.y;
                area[best] = cc.x >= 0 ? box_area(nbox[2 * tl_index(n, cc.x)], nbox[2 * tl_index(n, cc.x) + 1]) : -1.f;
                area[nl] = cc.y >= 0 ? box_area(nbox[2 * tl_index(n, cc.y)], nbox[2 * tl_index(n, cc.y) + 1]) : -1.f;
                ++nl;
            }
            for (int k = 0; k < nl; ++k) {
                s_leaf[w][k] = leaf[k];
                const size_t bi = tl_index(n, leaf[k]);
                const float4 lo = nbox[2 * bi], hi = nbox[2 * bi + 1];
                s_box[w][k][0] = lo.x; s_box[w][k][1] = lo.y; s_box[w][k][2] = lo.z;
                s_box[w][k][3] = hi.x; s_box[w][k][4] = hi.y; s_box[w][k][5] = hi.z;
            }
            s_nl[w] = nl;
            s_old[w] = old;
        }
        __syncwarp();
        const int nl = s_nl[w];
        if (nl < 3) {
            __syncwarp();
            continue;
        }
        const uint32_t full = (1u << nl) - 1u;
        // surface area of the union of each subset's boxes
        for (uint32_t S = lane + 1; S <= full; S += 32) {
            float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
            for (int k = 0; k < nl; ++k)
                if ((S >> k) & 1u)
                    for (int a = 0; a < 3; ++a) {
                        lo[a] = fminf(lo[a], s_box[w][k][a]);
                        hi[a] = fmaxf(hi[a], s_box[w][k][3 + a]);
                    }
            const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
            s_area[w][S] = dx * dy + dy * dz + dz * dx;
            s_cost[w][S] = 0.f;
        }
        __syncwarp();
        // cost of the best subtree over each subset, by subset size
        for (int size = 2; size <= nl; ++size) {
            for (uint32_t S = lane + 1; S <= full; S += 32) {
                if (__popc(S) != size) continue;
                const uint32_t low = S & (0u - S);
                float best = 3.0e38f;
                uint32_t bp = low;
                for (uint32_t P = (S - 1) & S; P; P = (P - 1) & S) {
                    if (!(P & low)) continue;
                    const float c = s_cost[w][P] + s_cost[w][S ^ P];
                    if (c < best) { best = c; bp = P; }
                }
                s_cost[w][S] = s_area[w][S] + best;
                s_part[w][S] = (uint8_t)bp;
            }
            __syncwarp();
        }
        if (lane == 0 && s_cost[w][full] < s_old[w] * (1.0f - 1e-5f)) {
            // rebuild: internal nodes reuse the treelet's indices (R stays the root)
            uint32_t stk_s[TL_LEAVES], ord_s[TL_LEAVES];
            int stk_n[TL_LEAVES], ord_n[TL_LEAVES];
            int sp = 0, no = 0, next = 1;
            stk_s[sp] = full;
            stk_n[sp++] = R;
            while (sp) {
                --sp;
                const uint32_t S = stk_s[sp];
                const int node = stk_n[sp];
                ord_s[no] = S;
                ord_n[no++] = node;
                const uint32_t P = s_part[w][S], Q = S ^ P;
                int ch[2];
                const uint32_t part[2] = {P, Q};
                for (int k = 0; k < 2; ++k) {
                    if (__popc(part[k]) == 1) {
                        ch[k] = s_leaf[w][__ffs(part[k]) - 1];
                    } else {
                        ch[k] = s_int[w][next++];
                        stk_s[sp] = part[k];
                        stk_n[sp++] = ch[k];
                    }
                    parent[tl_index(n, ch[k])] = node;
                }
                child[node] = make_int2(ch[0], ch[1]);
            }
            // boxes of the rebuilt internal nodes (R's box is unchanged)
            for (int k = 1; k < no; ++k) {
                float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
                for (int j = 0; j < nl; ++j)
                    if ((ord_s[k] >> j) & 1u)
                        for (int a = 0; a < 3; ++a) {
                            lo[a] = fminf(lo[a], s_box[w][j][a]);
                            hi[a] = fmaxf(hi[a], s_box[w][j][3 + a]);
                        }
                nbox[2 * (size_t)ord_n[k]] = make_float4(lo[0], lo[1], lo[2], 0.f);
                nbox[2 * (size_t)ord_n[k] + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
            }
            ++improved;
        }
        __syncwarp();
    }
    if (stats && lane == 0 && improved) atomicAdd(stats, improved);
}

// boxes only (the treelet pass reads node areas): second arrival at each node does the union
// Every walk up the parent links below stops after TL_MAX_WALK steps with DEVERR_BUILD_OVERFLOW (a
// binary tree this deep, or a damaged one, is reported instead of looping).
constexpr int TL_MAX_WALK = 1024;

__global__ void k_tl_boxes(const uint32_t* __restrict__ sorted, const float4* __restrict__ tbox, int n,
                           const int2* __restrict__ child, const int* __restrict__ parent, float4* nbox,
                           uint32_t* __restrict__ flags, uint32_t* __restrict__ err) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t p = sorted[j];
    nbox[2ull * (n - 1 + j)] = tbox[2ull * p];
    nbox[2ull * (n - 1 + j) + 1] = tbox[2ull * p + 1];
    int node = parent[n - 1 + j];
    for (int steps = 0; node >= 0; ++steps) {
        if (steps >= TL_MAX_WALK) {
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0) return;
        const int2 c = child[node];
        const size_t a = tl_index(n, c.x), b = tl_index(n, c.y);
        const float4 alo = __ldcg(&nbox[2 * a]), ahi = __ldcg(&nbox[2 * a + 1]);
        const float4 blo = __ldcg(&nbox[2 * b]), bhi = __ldcg(&nbox[2 * b + 1]);
        __stcg(&nbox[2ull * node], make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f));
        __stcg(&nbox[2ull * node + 1], make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f));
        node = parent[node];
    }
}

// triangles under every internal node: second arrival at each node adds its children's counts
__global__ void k_tl_count(int n, const int2* __restrict__ child, const int* __restrict__ parent,
                           int* __restrict__ cnt, uint32_t* __restrict__ flags, uint32_t* __restrict__ err) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int node = parent[n - 1 + j];
    for (int steps = 0; node >= 0; ++steps) {
        if (steps >= TL_MAX_WALK) {
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0) return;
        const int2 c = child[node];
        const int a = c.x >= 0 ? __ldcg(&cnt[c.x]) : 1, b = c.y >= 0 ? __ldcg(&cnt[c.y]) : 1;
        __stcg(&cnt[node], a + b);
        node = parent[node];
    }
}

// depth-first position of every node (internal: of its first leaf): the triangles of the left
// siblings along the path to the root
__global__ void k_tl_position(int n, const int2* __restrict__ child, const int* __restrict__ parent,
                              const int* __restrict__ cnt, int* __restrict__ pos, uint32_t* __restrict__ err) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 2 * n - 1) return;
    int node = x, p = 0;
    int ref = x < n - 1 ? x : ~(x - (n - 1));
    for (int steps = 0;; ++steps) {
        const int par = parent[node];
        if (par < 0) break;
        if (steps >= TL_MAX_WALK) {
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
            p = 0;
            break;
        }
        const int2 c = child[par];
        if (c.y == ref) p += c.x >= 0 ? cnt[c.x] : 1;
        node = par;
        ref = par;
    }
    pos[x] = p;
}

// renumber leaves by their depth-first position: sorted order, leaf references, leaf parents, ranges
__global__ void k_tl_relayout(int n, const int* __restrict__ pos, const int* __restrict__ cnt,
                              const uint32_t* __restrict__ sorted_in, uint32_t* __restrict__ sorted_out,
                              int2* __restrict__ child, int2* __restrict__ range, const int* __restrict__ parent_in,
                              int* __restrict__ leaf_parent_out, uint32_t* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {   // leaf at sorted position i moves to pos[n - 1 + i]
        const int q = pos[n - 1 + i];
        if (q < 0 || q >= n) {
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
        } else {
            sorted_out[q] = sorted_in[i];
            leaf_parent_out[q] = parent_in[n - 1 + i];
        }
    }
    if (i < n - 1) {
        int2 c = child[i];
        const bool ok = (c.x >= 0 ? c.x < n - 1 : ~c.x < n) && (c.y >= 0 ? c.y < n - 1 : ~c.y < n) && cnt[i] >= 2 &&
                        pos[i] >= 0 && pos[i] + cnt[i] <= n;
        if (!ok) {
            atomicOr(err, (uint32_t)DEVERR_BUILD_OVERFLOW);
            return;
        }
        if (c.x < 0) c.x = ~pos[n - 1 + ~c.x];
        if (c.y < 0) c.y = ~pos[n - 1 + ~c.y];
        child[i] = c;
        range[i] = make_int2(pos[i], pos[i] + cnt[i] - 1);
    }
}

// ---------------------------------------------------------------- K5 collapse to 8-wide nodes
struct CollapseArgs {
    int n;                        // triangles
    const int2* child;            // binary children
    const int2* range;            // binary ranges
    const float4* nbox;           // binary node boxes
    const uint32_t* sorted;       // sorted position -> scene primitive
    const float4* geo;            // triangle records, scene order
    const float4* vn;             // vertex normals, scene order (may be null)
    const uint32_t* prim_ent;     // entity per scene primitive
    WideNode* nodes;
    float4* tris;                 // leaf-order triangle records
    uint32_t* leaf_prim;
    float4* leaf_vn;
    uint32_t* leaf_entity;
    uint32_t* counters;           // [0] wide nodes used, [1] triangles placed, [2] next frontier size
    uint32_t node_cap;
    uint32_t* err;
    const float* dp;              // collapse costs from k_refit
    float cost_tri;               // triangle-test cost relative to a node test
};

__device__ __forceinline__ size_t box_index(int n, int ref) { return ref >= 0 ? (size_t)ref : (size_t)(n - 1 + ~ref); }
__device__ __forceinline__ int ref_count(const CollapseArgs& A, int ref) {
    if (ref < 0) return 1;
    int2 r = A.range[ref];
    return r.y - r.x + 1;
}
__device__ __forceinline__ int ref_first(const CollapseArgs& A, int ref) { return ref < 0 ? ~ref : A.range[ref].x; }

// Quantisation grid for a node: p = lo - q, q = 2^e with (hi - lo) / q <= 252 and q >= 4 ulps of the
// largest coordinate; every child box is widened by one quantum on each side, so the decoded FP32
// planes enclose the FP32 triangles with a margin of at least 4 ulps.
__device__ void node_grid(const float lo[3], const float hi[3], float p[3], int ex[3]) {
    for (int k = 0; k < 3; ++k) {
        const double ext = (double)hi[k] - (double)lo[k];
        int e = ext > 0 ? (int)ceil(log2(ext / 252.0)) : -126;
        const float m = fmaxf(fabsf(lo[k]), fabsf(hi[k]));
        int em = -126;
        if (m > 0.f) {
            int fe;
            frexpf(m, &fe);          // m in [2^(fe-1), 2^fe)
            em = fe - 1 - 23 + 2;    // 4 ulps
        }
        e = max(e, em);
        e = max(e, -126);
        e = min(e, 127);
        ex[k] = e;
        p[k] = __double2float_rd((double)lo[k] - ldexp(1.0, e));
    }
}

__global__ void k_collapse(CollapseArgs A, const int2* __restrict__ frontier, uint32_t fcount,
                           int2* __restrict__ next) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= fcount) return;
    const int bnode = frontier[t].x;       // binary internal node (or ~0 for the 1-leaf root)
    const uint32_t wnode = (uint32_t)frontier[t].y;
    const int n = A.n;

    int refs[8];
    int nc = 0;
    if (bnode == 0x7FFFFFFF) {
        // tiny scene: the root holds one leaf with all (<= 3) triangles
        nc = n > 0 ? 1 : 0;
        refs[0] = 0x7FFFFFFF;
    } else {
        // expand by the cost decisions: a child given k slots stays one root (a leaf or an 8-wide
        // node) unless spreading its k slots over its own children is cheaper
        int sr[8], sk[8], sp = 0;
        sr[sp] = bnode;
        sk[sp++] = 8;
        while (sp) {
            --sp;
            const int r = sr[sp], k = sk[sp];
            if (r != bnode && (r < 0 || k == 1 || !(__ldg(A.dp + 8ull * r + k - 1) < __ldg(A.dp + 8ull * r)))) {
                refs[nc++] = r;
                continue;
            }
            const int2 c = A.child[r];
            float cl[9], cr[9];
            dp_child(A.dp, c.x, c.x < 0 ? box_area(A.nbox[2 * box_index(n, c.x)], A.nbox[2 * box_index(n, c.x) + 1]) : 0.f,
                     A.cost_tri, cl);
            dp_child(A.dp, c.y, c.y < 0 ? box_area(A.nbox[2 * box_index(n, c.y)], A.nbox[2 * box_index(n, c.y) + 1]) : 0.f,
                     A.cost_tri, cr);
            int bk = 1;
            float best = 3.0e38f;
            for (int kk = 1; kk < k; ++kk) {
                const float v = cl[kk] + cr[k - kk];
                if (v < best) {
                    best = v;
                    bk = kk;
                }
            }
            sr[sp] = c.y;
            sk[sp++] = k - bk;
            sr[sp] = c.x;
            sk[sp++] = bk;
        }
    }

    // child boxes, counts, first sorted positions
    float clo[8][3], chi[8][3];
    int cnt[8], first[8];
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int k = 0; k < nc; ++k) {
        if (refs[k] == 0x7FFFFFFF) {   // all triangles
            cnt[k] = n;
            first[k] = 0;
            const size_t bi = n > 1 ? 0 : (size_t)(n - 1);   // root box (internal 0) or the single leaf
            const float4 a = A.nbox[2 * bi], b = A.nbox[2 * bi + 1];
            clo[k][0] = a.x; clo[k][1] = a.y; clo[k][2] = a.z;
            chi[k][0] = b.x; chi[k][1] = b.y; chi[k][2] = b.z;
        } else {
            cnt[k] = ref_count(A, refs[k]);
            first[k] = ref_first(A, refs[k]);
            if (cnt[k] < 1 || first[k] < 0 || first[k] + cnt[k] > n) {   // damaged ranges: report, read nothing
                atomicOr(A.err, (uint32_t)DEVERR_BUILD_OVERFLOW);
                return;
            }
            const size_t bi = box_index(n, refs[k]);
            const float4 a = A.nbox[2 * bi], b = A.nbox[2 * bi + 1];
            clo[k][0] = a.x; clo[k][1] = a.y; clo[k][2] = a.z;
            chi[k][0] = b.x; chi[k][1] = b.y; chi[k][2] = b.z;
        }
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], clo[k][a]);
            hi[a] = fmaxf(hi[a], chi[k][a]);
        }
    }
    if (nc == 0) {
        for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0.f;
    }

    // slot assignment: slot s takes the child whose centroid lies farthest along
    // D(s) = (s&1 ? -1 : 1, s&2 ? -1 : 1, s&4 ? -1 : 1) from the node centre (greedy)
    int slot_of[8];
    int child_in[8];
    for (int s = 0; s < 8; ++s) child_in[s] = -1;
    {
        float score[8][8];
        const float cxn = 0.5f * (lo[0] + hi[0]), cyn = 0.5f * (lo[1] + hi[1]), czn = 0.5f * (lo[2] + hi[2]);
        for (int k = 0; k < nc; ++k) {
            const float ox = 0.5f * (clo[k][0] + chi[k][0]) - cxn;
            const float oy = 0.5f * (clo[k][1] + chi[k][1]) - cyn;
            const float oz = 0.5f * (clo[k][2] + chi[k][2]) - czn;
            for (int s = 0; s < 8; ++s)
                score[k][s] = ((s & 1) ? -ox : ox) + ((s & 2) ? -oy : oy) + ((s & 4) ? -oz : oz);
            slot_of[k] = -1;
        }
        for (int it = 0; it < nc; ++it) {
            float best = -3.0e38f;
            int bk = -1, bs = -1;
            for (int k = 0; k < nc; ++k) {
                if (slot_of[k] >= 0) continue;
                for (int s = 0; s < 8; ++s) {
                    if (child_in[s] >= 0) continue;
                    if (score[k][s] > best) { best = score[k][s]; bk = k; bs = s; }
                }
            }
            slot_of[bk] = bs;
            child_in[bs] = bk;
        }
    }

    // leaves (<= 3 triangles) vs internal children; allocation
    uint32_t imask = 0, n_int = 0, n_tri = 0;
    int tri_off[8];
    for (int s = 0; s < 8; ++s) {
        tri_off[s] = 0;
        const int k = child_in[s];
        if (k < 0) continue;
        if (cnt[k] <= 3) {
            tri_off[s] = (int)n_tri;
            n_tri += cnt[k];
        } else {
            imask |= 1u << s;
            ++n_int;
        }
    }
    uint32_t child_base = 0, tri_base = 0;
    if (n_int) child_base = atomicAdd(&A.counters[0], n_int);
    if (n_tri) tri_base = atomicAdd(&A.counters[1], n_tri);
    if (child_base + n_int > A.node_cap || tri_base + n_tri > (uint32_t)n) {
        atomicOr(A.err, (uint32_t)DEVERR_BUILD_OVERFLOW);
        return;
    }

    float p[3];
    int ex[3];
    node_grid(lo, hi, p, ex);
    uint8_t meta[8], qlo[3][8], qhi[3][8];
    uint32_t rank = 0;
    for (int s = 0; s < 8; ++s) {
        const int k = child_in[s];
        if (k < 0) {
            meta[s] = 0;
            for (int a = 0; a < 3; ++a) { qlo[a][s] = 0xFF; qhi[a][s] = 0; }
            continue;
        }
        for (int a = 0; a < 3; ++a) {
            const double iq = ldexp(1.0, -ex[a]);   // 1 / 2^ex, exact: the products equal the quotients
            double l = floor(((double)clo[k][a] - (double)p[a]) * iq);
            double h = ceil(((double)chi[k][a] - (double)p[a]) * iq);
            l -= 1.0;
            h += 1.0;
            if (l < 0 || h > 255) atomicOr(A.err, (uint32_t)DEVERR_QUANT_RANGE);
            qlo[a][s] = (uint8_t)fmax(0.0, fmin(255.0, l));
            qhi[a][s] = (uint8_t)fmax(0.0, fmin(255.0, h));
        }
        if (imask & (1u << s)) {
            meta[s] = (uint8_t)((1u << 5) | (24u + s));
            next[atomicAdd(&A.counters[2], 1u)] = make_int2(refs[k], (int)(child_base + rank));
            ++rank;
        } else {
            const uint32_t unary = (1u << cnt[k]) - 1u;
            meta[s] = (uint8_t)((unary << 5) | (uint32_t)tri_off[s]);
            for (int m = 0; m < cnt[k]; ++m) {
                const uint32_t slot = tri_base + tri_off[s] + m;
                const uint32_t prim = A.sorted[first[k] + m];
                A.tris[3ull * slot + 0] = A.geo[3ull * prim + 0];
                A.tris[3ull * slot + 1] = A.geo[3ull * prim + 1];
                A.tris[3ull * slot + 2] = A.geo[3ull * prim + 2];
                A.leaf_prim[slot] = prim;
                A.leaf_entity[slot] = A.prim_ent[prim];
                if (A.vn) {
                    A.leaf_vn[3ull * slot + 0] = A.vn[3ull * prim + 0];
                    A.leaf_vn[3ull * slot + 1] = A.vn[3ull * prim + 1];
                    A.leaf_vn[3ull * slot + 2] = A.vn[3ull * prim + 2];
                }
            }
        }
    }
    auto pack4 = [](const uint8_t* b) {
        return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
    };
    WideNode w;
    const uint32_t eword = ((uint32_t)(uint8_t)(int8_t)ex[0]) | ((uint32_t)(uint8_t)(int8_t)ex[1] << 8) |
                           ((uint32_t)(uint8_t)(int8_t)ex[2] << 16) | (imask << 24);
    w.w[0] = make_float4(p[0], p[1], p[2], __uint_as_float(eword));
    w.w[1] = make_float4(__uint_as_float(child_base), __uint_as_float(tri_base), __uint_as_float(pack4(meta)),
                         __uint_as_float(pack4(meta + 4)));
    // planes: per axis 8 halves 0x5C00 | q (= 256 + q / 4), lo x/y/z then hi x/y/z
    auto pack_h = [](const uint8_t* b) {
        uint32_t v[4];
        for (int j = 0; j < 4; ++j) v[j] = (0x5C00u | b[2 * j]) | ((0x5C00u | b[2 * j + 1]) << 16);
        return make_float4(__uint_as_float(v[0]), __uint_as_float(v[1]), __uint_as_float(v[2]), __uint_as_float(v[3]));
    };
    for (int a = 0; a < 3; ++a) {
        w.w[2 + a] = pack_h(qlo[a]);
        w.w[5 + a] = pack_h(qhi[a]);
    }
    A.nodes[wnode] = w;
}

// ---------------------------------------------------------------- binned-SAH topology
// Top-down, level-synchronous binned SAH (16 bins on each axis over the centroid bounds) down to
// segments of at most SAH_T triangles, which Karras' construction then builds (its prefix function
// restricted to the segment).  Partitions are stable, so every segment keeps the Morton order of
// the global sort.  Node numbering follows the binary radix tree: a segment [f, l] uses internal
// indices f .. l - 1, and the split that puts [first, p) left and [p, last] right gets index p - 1,
// the last position of its left part, which no segment uses; together that is exactly n - 1 nodes,
// so the collapse consumes the tree unchanged (its root is passed explicitly).
constexpr int SAH_BINS = 16;
constexpr int SAH_T = 4;
constexpr int SAH_W = 13;                               // count, box lo/hi, centroid lo/hi (fkeys)
constexpr int SAH_TASK_WORDS = 3 * SAH_BINS * SAH_W;
constexpr int SAH_BLOCK_ITEMS = 2048;
constexpr int SAH_SMALL = 2048;                         // tasks of at most this many triangles: k_sah_bin_small

struct SahTask {
    int first, count;
    float clo[3], chi[3];    // centroid bounds
    int parent, side;        // parent split node (-1 for the root) and which child this is
};

struct SahSplit {
    int nl;                  // triangles of the left child
    int axis, bin;           // axis < 0: split by position (no usable centroid extent)
    float lclo[3], lchi[3], rclo[3], rchi[3];
};

struct SahSeg {
    int first, count, parent, side;
};

__device__ __forceinline__ int sah_bin(float c, float lo, float hi) {
    const float ext = hi - lo;
    if (!(ext > 0.f)) return 0;
    const int b = (int)((c - lo) * ((float)SAH_BINS / ext));
    return max(0, min(SAH_BINS - 1, b));
}

__global__ void k_sah_root(const uint32_t* __restrict__ keys, int n, SahTask* __restrict__ t) {
    SahTask r;
    r.first = 0;
    r.count = n;
    for (int k = 0; k < 3; ++k) {
        r.clo[k] = fkey_inv(keys[6 + k]);
        r.chi[k] = fkey_inv(keys[9 + k]);
    }
    r.parent = -1;
    r.side = 0;
    t[0] = r;
}

__global__ void k_sah_clear(uint32_t* __restrict__ bins, size_t words) {
    for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(w % SAH_W);
        bins[w] = k == 0 ? 0u : (((k - 1) % 6) < 3 ? 0xFFFFFFFFu : 0u);
    }
}

__device__ __forceinline__ void sah_add(uint32_t* b, const float4& lo, const float4& hi, const float4& c) {
    atomicAdd(&b[0], 1u);
    atomicMin(&b[1], fkey(lo.x)); atomicMin(&b[2], fkey(lo.y)); atomicMin(&b[3], fkey(lo.z));
    atomicMax(&b[4], fkey(hi.x)); atomicMax(&b[5], fkey(hi.y)); atomicMax(&b[6], fkey(hi.z));
    atomicMin(&b[7], fkey(c.x)); atomicMin(&b[8], fkey(c.y)); atomicMin(&b[9], fkey(c.z));
    atomicMax(&b[10], fkey(c.x)); atomicMax(&b[11], fkey(c.y)); atomicMax(&b[12], fkey(c.z));
}

// One warp per task of at most SAH_SMALL triangles: the warp bins its task's positions (a contiguous
// range) into warp-private shared memory, where only its own lanes contend, and stores the task's
// bins, which no other kernel writes (k_sah_bin skips these tasks).  Counts, minima and maxima do not
// depend on the order of the additions, so the bins equal those of k_sah_bin.
__global__ void __launch_bounds__(256) k_sah_bin_small(const uint32_t* __restrict__ perm,
                                                       const SahTask* __restrict__ tasks, int n_tasks,
                                                       const float4* __restrict__ tbox, const float4* __restrict__ cen,
                                                       uint32_t* __restrict__ bins) {
    __shared__ uint32_t sb[8][SAH_TASK_WORDS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * 8 + warp;
    if (t >= n_tasks) return;            // warp-uniform; the kernel has no block-wide barrier
    const SahTask T = tasks[t];
    if (T.count > SAH_SMALL) return;     // warp-uniform: binned by k_sah_bin
    uint32_t* b = sb[warp];
    for (int w = lane; w < SAH_TASK_WORDS; w += 32) {
        const int k = w % SAH_W;
        b[w] = k == 0 ? 0u : (((k - 1) % 6) < 3 ? 0xFFFFFFFFu : 0u);
    }
    __syncwarp();
    for (int i = T.first + lane; i < T.first + T.count; i += 32) {
        const uint32_t p = perm[i];
        const float4 lo = tbox[2ull * p], hi = tbox[2ull * p + 1], c = cen[p];
        const float cv[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; ++a) sah_add(b + (a * SAH_BINS + sah_bin(cv[a], T.clo[a], T.chi[a])) * SAH_W, lo, hi, c);
    }
    __syncwarp();
    uint32_t* g = bins + (size_t)t * SAH_TASK_WORDS;
    for (int w = lane; w < SAH_TASK_WORDS; w += 32) g[w] = b[w];
}

// One block per SAH_BLOCK_ITEMS positions; a block whose positions all belong to one task (tasks
// are contiguous ranges) bins into shared memory first.  Positions of tasks of at most SAH_SMALL
// triangles are left to k_sah_bin_small.
__global__ void __launch_bounds__(256) k_sah_bin(const uint32_t* __restrict__ perm, const int* __restrict__ task_of,
                                                 const SahTask* __restrict__ tasks, const float4* __restrict__ tbox,
                                                 const float4* __restrict__ cen, int n, uint32_t* __restrict__ bins) {
    __shared__ uint32_t sb[SAH_TASK_WORDS];
    const int b0 = blockIdx.x * SAH_BLOCK_ITEMS, b1 = min(n, b0 + SAH_BLOCK_ITEMS);
    if (b0 >= n) return;
    const int t0 = task_of[b0], t1 = task_of[b1 - 1];
    const bool priv = t0 >= 0 && t0 == t1;
    if (priv && tasks[t0].count <= SAH_SMALL) return;   // block-uniform, before any barrier
    if (priv) {
        for (int w = threadIdx.x; w < SAH_TASK_WORDS; w += blockDim.x) {
            const int k = w % SAH_W;
            sb[w] = k == 0 ? 0u : (((k - 1) % 6) < 3 ? 0xFFFFFFFFu : 0u);
        }
        __syncthreads();
    }
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const int t = task_of[i];
        if (t < 0) continue;
        const SahTask& T = tasks[t];
        if (T.count <= SAH_SMALL) continue;
        const uint32_t p = perm[i];
        const float4 lo = tbox[2ull * p], hi = tbox[2ull * p + 1], c = cen[p];
        const float cv[3] = {c.x, c.y, c.z};
        uint32_t* base = priv ? sb : bins + (size_t)t * SAH_TASK_WORDS;
        for (int a = 0; a < 3; ++a) sah_add(base + (a * SAH_BINS + sah_bin(cv[a], T.clo[a], T.chi[a])) * SAH_W, lo, hi, c);
    }
    if (priv) {
        __syncthreads();
        uint32_t* g = bins + (size_t)t0 * SAH_TASK_WORDS;
        for (int w = threadIdx.x; w < SAH_TASK_WORDS; w += blockDim.x) {
            const int k = w % SAH_W;
            const uint32_t v = sb[w];
            if (k == 0) {
                if (v) atomicAdd(&g[w], v);
            } else if (((k - 1) % 6) < 3) {
                if (v != 0xFFFFFFFFu) atomicMin(&g[w], v);
            } else if (v) {
                atomicMax(&g[w], v);
            }
        }
    }
}

__device__ __forceinline__ float sah_area(const float lo[3], const float hi[3]) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// One thread per task: the cheapest of the 3 x 15 bin boundaries by surface area x count.
__global__ void k_sah_split(const SahTask* __restrict__ tasks, int n_tasks, const uint32_t* __restrict__ bins,
                            SahSplit* __restrict__ splits) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    const SahTask T = tasks[t];
    const uint32_t* B = bins + (size_t)t * SAH_TASK_WORDS;
    float best = 3.0e38f;
    int ba = -1, bb = 0;
    for (int a = 0; a < 3; ++a) {
        if (!(T.chi[a] - T.clo[a] > 0.f)) continue;
        // right sweep: area x count of bins [s, SAH_BINS)
        float rcost[SAH_BINS];
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        uint32_t cnt = 0;
        for (int s = SAH_BINS - 1; s >= 1; --s) {
            const uint32_t* w = B + (a * SAH_BINS + s) * SAH_W;
            if (w[0]) {
                cnt += w[0];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = fminf(lo[k], fkey_inv(w[1 + k]));
                    hi[k] = fmaxf(hi[k], fkey_inv(w[4 + k]));
                }
            }
            rcost[s] = cnt ? sah_area(lo, hi) * (float)cnt : -1.f;
        }
        for (int k = 0; k < 3; ++k) { lo[k] = 3.0e38f; hi[k] = -3.0e38f; }
        cnt = 0;
        for (int s = 1; s < SAH_BINS; ++s) {
            const uint32_t* w = B + (a * SAH_BINS + s - 1) * SAH_W;
            if (w[0]) {
                cnt += w[0];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = fminf(lo[k], fkey_inv(w[1 + k]));
                    hi[k] = fmaxf(hi[k], fkey_inv(w[4 + k]));
                }
            }
            if (cnt == 0 || rcost[s] < 0.f) continue;
            const float c = sah_area(lo, hi) * (float)cnt + rcost[s];
            if (c < best) {
                best = c;
                ba = a;
                bb = s;
            }
        }
    }
    SahSplit S;
    if (ba < 0) {
        S.nl = T.count / 2;
        S.axis = -1;
        S.bin = 0;
        for (int k = 0; k < 3; ++k) {
            S.lclo[k] = S.rclo[k] = T.clo[k];
            S.lchi[k] = S.rchi[k] = T.chi[k];
        }
    } else {
        int nl = 0;
        float llo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, lhi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        float rlo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, rhi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        for (int s = 0; s < SAH_BINS; ++s) {
            const uint32_t* w = B + (ba * SAH_BINS + s) * SAH_W;
            if (!w[0]) continue;
            float* clo = s < bb ? llo : rlo;
            float* chi = s < bb ? lhi : rhi;
            if (s < bb) nl += (int)w[0];
            for (int k = 0; k < 3; ++k) {
                clo[k] = fminf(clo[k], fkey_inv(w[7 + k]));
                chi[k] = fmaxf(chi[k], fkey_inv(w[10 + k]));
            }
        }
        S.nl = nl;
        S.axis = ba;
        S.bin = bb;
        for (int k = 0; k < 3; ++k) {
            S.lclo[k] = llo[k];
            S.lchi[k] = lhi[k];
            S.rclo[k] = rlo[k];
            S.rchi[k] = rhi[k];
        }
    }
    splits[t] = S;
}

__device__ __forceinline__ bool sah_left(const SahTask& T, const SahSplit& S, int i, const float4& c) {
    if (S.axis < 0) return i - T.first < S.nl;
    const float cv[3] = {c.x, c.y, c.z};
    return sah_bin(cv[S.axis], T.clo[S.axis], T.chi[S.axis]) < S.bin;
}

__global__ void k_sah_flags(const uint32_t* __restrict__ perm, const int* __restrict__ task_of,
                            const SahTask* __restrict__ tasks, const SahSplit* __restrict__ splits,
                            const float4* __restrict__ cen, int n, uint32_t* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = task_of[i];
    flags[i] = t >= 0 && sah_left(tasks[t], splits[t], i, cen[perm[i]]) ? 1u : 0u;
}

// child-task and segment flags: [2t] left, [2t + 1] right
__global__ void k_sah_child_flags(const SahTask* __restrict__ tasks, const SahSplit* __restrict__ splits, int n_tasks,
                                  uint32_t* __restrict__ tflag, uint32_t* __restrict__ sflag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    const int cl = splits[t].nl, cr = tasks[t].count - cl;
    tflag[2 * t] = cl > SAH_T;
    tflag[2 * t + 1] = cr > SAH_T;
    sflag[2 * t] = cl <= SAH_T;
    sflag[2 * t + 1] = cr <= SAH_T;
}

// Split nodes and the next level's tasks / final segments.  tscan / sscan: exclusive scans of the
// child flags; seg_base: segments found by earlier levels.
__global__ void k_sah_emit(const SahTask* __restrict__ tasks, const SahSplit* __restrict__ splits, int n_tasks,
                           const uint32_t* __restrict__ tflag, const uint32_t* __restrict__ tscan,
                           const uint32_t* __restrict__ sflag, const uint32_t* __restrict__ sscan, uint32_t seg_base,
                           SahTask* __restrict__ next, SahSeg* __restrict__ segs, int2* __restrict__ child,
                           int2* __restrict__ range, int* __restrict__ parent) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    const SahTask T = tasks[t];
    const SahSplit S = splits[t];
    const int X = T.first + S.nl - 1;
    range[X] = make_int2(T.first, T.first + T.count - 1);
    parent[X] = T.parent;
    if (T.parent >= 0) {
        if (T.side == 0) child[T.parent].x = X;
        else child[T.parent].y = X;
    }
    for (int side = 0; side < 2; ++side) {
        const int f = side ? T.first + S.nl : T.first;
        const int c = side ? T.count - S.nl : S.nl;
        if (tflag[2 * t + side]) {
            SahTask C;
            C.first = f;
            C.count = c;
            for (int k = 0; k < 3; ++k) {
                C.clo[k] = side ? S.rclo[k] : S.lclo[k];
                C.chi[k] = side ? S.rchi[k] : S.lchi[k];
            }
            C.parent = X;
            C.side = side;
            next[tscan[2 * t + side]] = C;
        } else if (sflag[2 * t + side]) {
            segs[seg_base + sscan[2 * t + side]] = SahSeg{f, c, X, side};
        }
    }
}

__global__ void k_sah_scatter(const uint32_t* __restrict__ perm_in, uint32_t* __restrict__ perm_out,
                              const int* __restrict__ task_in, int* __restrict__ task_out,
                              const SahTask* __restrict__ tasks, const SahSplit* __restrict__ splits,
                              const uint32_t* __restrict__ flags, const uint32_t* __restrict__ scan,
                              const uint32_t* __restrict__ tflag, const uint32_t* __restrict__ tscan, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = task_in[i];
    if (t < 0) {
        perm_out[i] = perm_in[i];
        task_out[i] = -1;
        return;
    }
    const int f = tasks[t].first, nl = splits[t].nl;
    const int lr = (int)(scan[i] - scan[f]);   // left items before i in this task
    const bool left = flags[i] != 0;
    const int pos = left ? f + lr : f + nl + (i - f - lr);
    const int side = left ? 0 : 1;
    perm_out[pos] = perm_in[i];
    task_out[pos] = tflag[2 * t + side] ? (int)tscan[2 * t + side] : -1;
}

__global__ void k_sah_segments(const SahSeg* __restrict__ segs, int n_segs, int n, int* __restrict__ seg_lo,
                               int* __restrict__ seg_hi, int2* __restrict__ child, int* __restrict__ parent) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_segs) return;
    const SahSeg S = segs[s];
    for (int p = S.first; p < S.first + S.count; ++p) {
        seg_lo[p] = S.first;
        seg_hi[p] = S.first + S.count - 1;
    }
    const int root = S.count >= 2 ? S.first : ~S.first;
    if (S.parent >= 0) {
        if (S.side == 0) child[S.parent].x = root;
        else child[S.parent].y = root;
        parent[root >= 0 ? root : (n - 1) + ~root] = S.parent;
    }
}

__global__ void k_gather_codes(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ code_by_prim, int n,
                               uint32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = code_by_prim[perm[i]];
}

__device__ __forceinline__ int delta_seg(const uint32_t* __restrict__ code, int lo, int hi, int i, int j) {
    if (j < lo || j > hi) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

// Karras' construction inside each segment [seg_lo, seg_hi] (the last position of a segment is not
// an internal node of it)
__global__ void k_karras_seg(const uint32_t* __restrict__ code, int n, const int* __restrict__ seg_lo,
                             const int* __restrict__ seg_hi, int2* __restrict__ child, int2* __restrict__ range,
                             int* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int lo_s = seg_lo[i], hi_s = seg_hi[i];
    if (i >= hi_s) return;
    const int d = (delta_seg(code, lo_s, hi_s, i, i + 1) - delta_seg(code, lo_s, hi_s, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta_seg(code, lo_s, hi_s, i, i - d);
    int lmax = 2;
    while (delta_seg(code, lo_s, hi_s, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta_seg(code, lo_s, hi_s, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta_seg(code, lo_s, hi_s, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta_seg(code, lo_s, hi_s, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = (lo == gamma) ? ~gamma : gamma;
    const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(lo, hi);
    parent[left >= 0 ? left : (n - 1) + ~left] = i;
    parent[right >= 0 ? right : (n - 1) + ~right] = i;
}

// exclusive scan, multi-block: per-block totals, one-block scan of the totals, per-block scan
constexpr int SCAN_ITEMS = 2048;
__global__ void __launch_bounds__(256) k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                     uint32_t m, uint32_t* __restrict__ totals) {
    __shared__ uint32_t part[256];
    const uint32_t b0 = blockIdx.x * SCAN_ITEMS + threadIdx.x * 8;
    uint32_t v[8], s = 0;
    for (int k = 0; k < 8; ++k) {
        v[k] = b0 + k < m ? in[b0 + k] : 0u;
        s += v[k];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const uint32_t x = threadIdx.x >= (uint32_t)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (int k = 0; k < 8; ++k) {
        if (b0 + k < m) out[b0 + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 255) totals[blockIdx.x] = part[255];
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint32_t m, const uint32_t* __restrict__ totals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) out[i] += totals[i / SCAN_ITEMS];
}

void scan_exclusive(crt_context* ctx, const uint32_t* in, uint32_t* out, uint32_t m, uint32_t* totals) {
    if (!m) return;
    cudaStream_t st = ctx->stream;
    const uint32_t nb = (m + SCAN_ITEMS - 1) / SCAN_ITEMS;
    k_scan_blocks<<<nb, 256, 0, st>>>(in, out, m, totals);
    check_launch(ctx, "k_scan_blocks");
    k_scan<<<1, 1024, 0, st>>>(totals, nb);
    check_launch(ctx, "k_scan");
    k_scan_add<<<(m + 255) / 256, 256, 0, st>>>(out, m, totals);
    check_launch(ctx, "k_scan_add");
}

// Binned-SAH binary tree over the Morton-sorted triangles (n > SAH_T): fills child / range / parent
// like k_karras and writes the triangle order of the tree's leaves to `sorted` (in place of the
// Morton order).  Returns the root's internal index, or -1 (with nothing modified) when its
// temporaries (about 0.6 GB per million triangles) cannot be allocated.
int sah_topology(crt_context* ctx, int n, const float4* tbox, const float4* cen, const uint32_t* keys,
                 uint32_t* sorted, const uint32_t* code_by_prim, int2* child, int2* range, int* parent) {
    cudaStream_t st = ctx->stream;
    const size_t max_tasks = (size_t)n / (SAH_T + 1) + 2;
    const size_t max_segs = (size_t)n;
    char* mem = nullptr;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_perm = take(4ull * n), o_task0 = take(4ull * n), o_task1 = take(4ull * n), o_flags = take(4ull * n),
                 o_scan = take(4ull * n), o_tot = take(4ull * ((2 * max_tasks + n) / SCAN_ITEMS + 2)),
                 o_tasks0 = take(sizeof(SahTask) * max_tasks), o_tasks1 = take(sizeof(SahTask) * max_tasks),
                 o_split = take(sizeof(SahSplit) * max_tasks), o_bins = take(4ull * SAH_TASK_WORDS * max_tasks),
                 o_tf = take(8ull * max_tasks), o_ts = take(8ull * max_tasks), o_sf = take(8ull * max_tasks),
                 o_ss = take(8ull * max_tasks), o_segs = take(sizeof(SahSeg) * max_segs), o_lo = take(4ull * n),
                 o_hi = take(4ull * n), o_code = take(4ull * n);
    if (cudaMalloc(&mem, off) != cudaSuccess) {   // nothing modified yet: the caller builds a radix tree
        cudaGetLastError();
        return -1;
    }
    struct Free {
        char* p;
        ~Free() { cudaFree(p); }
    } guard{mem};
    uint32_t* perm[2] = {sorted, (uint32_t*)(mem + o_perm)};
    int* task_of[2] = {(int*)(mem + o_task0), (int*)(mem + o_task1)};
    uint32_t* flags = (uint32_t*)(mem + o_flags);
    uint32_t* scan = (uint32_t*)(mem + o_scan);
    uint32_t* totals = (uint32_t*)(mem + o_tot);
    SahTask* tasks[2] = {(SahTask*)(mem + o_tasks0), (SahTask*)(mem + o_tasks1)};
    SahSplit* splits = (SahSplit*)(mem + o_split);
    uint32_t* bins = (uint32_t*)(mem + o_bins);
    uint32_t *tflag = (uint32_t*)(mem + o_tf), *tscan = (uint32_t*)(mem + o_ts);
    uint32_t *sflag = (uint32_t*)(mem + o_sf), *sscan = (uint32_t*)(mem + o_ss);
    SahSeg* segs = (SahSeg*)(mem + o_segs);
    int *seg_lo = (int*)(mem + o_lo), *seg_hi = (int*)(mem + o_hi);
    uint32_t* code = (uint32_t*)(mem + o_code);

    CRT_CUDA(cudaMemsetAsync(task_of[0], 0, 4ull * n, st));   // every position in task 0 (the root)
    k_sah_root<<<1, 1, 0, st>>>(keys, n, tasks[0]);
    check_launch(ctx, "k_sah_root");
    int cur = 0, n_tasks = 1, root = -1;
    uint32_t n_segs = 0;
    for (int level = 0; n_tasks > 0; ++level) {
        CRT_CHECK(level < 256 && (size_t)n_tasks <= max_tasks, CRT_ERR_DEVICE, "SAH build did not converge");
        const size_t words = (size_t)n_tasks * SAH_TASK_WORDS;
        k_sah_clear<<<(uint32_t)std::min<size_t>((words + 255) / 256, 4096), 256, 0, st>>>(bins, words);
        check_launch(ctx, "k_sah_clear");
        k_sah_bin<<<(n + SAH_BLOCK_ITEMS - 1) / SAH_BLOCK_ITEMS, 256, 0, st>>>(perm[cur], task_of[cur], tasks[cur],
                                                                              tbox, cen, n, bins);
        check_launch(ctx, "k_sah_bin");
        k_sah_bin_small<<<(n_tasks + 7) / 8, 256, 0, st>>>(perm[cur], tasks[cur], n_tasks, tbox, cen, bins);
        check_launch(ctx, "k_sah_bin_small");
        k_sah_split<<<(n_tasks + 127) / 128, 128, 0, st>>>(tasks[cur], n_tasks, bins, splits);
        check_launch(ctx, "k_sah_split");
        k_sah_flags<<<(n + 255) / 256, 256, 0, st>>>(perm[cur], task_of[cur], tasks[cur], splits, cen, n, flags);
        check_launch(ctx, "k_sah_flags");
        scan_exclusive(ctx, flags, scan, (uint32_t)n, totals);
        k_sah_child_flags<<<(n_tasks + 255) / 256, 256, 0, st>>>(tasks[cur], splits, n_tasks, tflag, sflag);
        check_launch(ctx, "k_sah_child_flags");
        scan_exclusive(ctx, tflag, tscan, 2u * n_tasks, totals);
        scan_exclusive(ctx, sflag, sscan, 2u * n_tasks, totals);
        k_sah_emit<<<(n_tasks + 255) / 256, 256, 0, st>>>(tasks[cur], splits, n_tasks, tflag, tscan, sflag, sscan, n_segs,
                                                          tasks[cur ^ 1], segs, child, range, parent);
        check_launch(ctx, "k_sah_emit");
        k_sah_scatter<<<(n + 255) / 256, 256, 0, st>>>(perm[cur], perm[cur ^ 1], task_of[cur], task_of[cur ^ 1],
                                                       tasks[cur], splits, flags, scan, tflag, tscan, n);
        check_launch(ctx, "k_sah_scatter");
        if (level == 0) {
            int nl = 0;
            CRT_CUDA(cudaMemcpyAsync(&nl, &splits[0].nl, sizeof(int), cudaMemcpyDeviceToHost, st));
            CRT_CUDA(cudaStreamSynchronize(st));
            root = nl - 1;
        }
        // next level's task count and the segment count: last exclusive-scan value + last flag
        uint32_t h[4];
        CRT_CUDA(cudaMemcpyAsync(&h[0], tscan + 2 * n_tasks - 1, 4, cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaMemcpyAsync(&h[1], tflag + 2 * n_tasks - 1, 4, cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaMemcpyAsync(&h[2], sscan + 2 * n_tasks - 1, 4, cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaMemcpyAsync(&h[3], sflag + 2 * n_tasks - 1, 4, cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaStreamSynchronize(st));
        n_tasks = (int)(h[0] + h[1]);
        n_segs += h[2] + h[3];
        CRT_CHECK(n_segs <= max_segs, CRT_ERR_DEVICE, "SAH build: too many segments");
        cur ^= 1;
    }
    if (perm[cur] != sorted)
        CRT_CUDA(cudaMemcpyAsync(sorted, perm[cur], 4ull * n, cudaMemcpyDeviceToDevice, st));
    k_sah_segments<<<(n_segs + 255) / 256, 256, 0, st>>>(segs, (int)n_segs, n, seg_lo, seg_hi, child, parent);
    check_launch(ctx, "k_sah_segments");
    k_gather_codes<<<(n + 255) / 256, 256, 0, st>>>(sorted, code_by_prim, n, code);
    check_launch(ctx, "k_gather_codes");
    k_karras_seg<<<(n + 254) / 256, 256, 0, st>>>(code, n, seg_lo, seg_hi, child, range, parent);
    check_launch(ctx, "k_karras_seg");
    CRT_CUDA(cudaStreamSynchronize(st));   // the temporaries are released on return
    return root;
}

inline uint32_t cdiv(size_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

// Builds every device array of the scene.  Throws CrtError on failure.
void scene_build(crt_scene* s, const crt_entity_desc* ents, uint32_t n_ents) {
    crt_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    size_t n64 = 0;
    for (uint32_t e = 0; e < n_ents; ++e) n64 += ents[e].n_tris;
    CRT_CHECK(n64 < 0x7FFFFFF0ull, CRT_ERR_INVALID, "scene too large (>= 2^31 triangles)");
    const uint32_t n = (uint32_t)n64;
    s->n_tris = n;
    s->n_entities = n_ents;
    bool any_vn = false;
    for (uint32_t e = 0; e < n_ents; ++e) {
        CRT_CHECK(ents[e].n_tris == 0 || ents[e].tri_xyz, CRT_ERR_INVALID, "entity without triangle data");
        if (ents[e].smooth_shading && ents[e].tri_vn) any_vn = true;
    }

    cudaEvent_t ev0, ev1;
    CRT_CUDA(cudaEventCreate(&ev0));
    CRT_CUDA(cudaEventCreate(&ev1));
    CRT_CUDA(cudaEventRecord(ev0, st));

    // entity table + transforms
    s->host_entities.resize(std::max<uint32_t>(n_ents, 1));
    std::vector<EntXform> xf(std::max<uint32_t>(n_ents, 1));
    uint32_t off = 0;
    for (uint32_t e = 0; e < n_ents; ++e) {
        EntityDev& d = s->host_entities[e];
        std::memcpy(d.color, ents[e].color, sizeof(d.color));
        d.smooth = ents[e].smooth_shading ? 1u : 0u;
        d.id = ents[e].id;
        d.rho_s = ents[e].rho_s;
        d.rho_d = ents[e].rho_d;
        d.pad = 0;
        xf[e].scale = ents[e].scale;
        std::memcpy(xf[e].pos, ents[e].position, sizeof(xf[e].pos));
        std::memcpy(xf[e].rot, ents[e].rotation, sizeof(xf[e].rot));
        xf[e].first = off;
        xf[e].has_vn = (ents[e].smooth_shading && ents[e].tri_vn) ? 1u : 0u;
        off += (uint32_t)ents[e].n_tris;
    }
    CRT_CUDA(cudaMalloc(&s->entities, sizeof(EntityDev) * s->host_entities.size()));
    CRT_CUDA(cudaMemcpyAsync(s->entities, s->host_entities.data(), sizeof(EntityDev) * s->host_entities.size(),
                             cudaMemcpyHostToDevice, st));
    EntXform* d_xf = (EntXform*)ctx_scratch(ctx, SCR_BUILD7, sizeof(EntXform) * xf.size());
    CRT_CUDA(cudaMemcpyAsync(d_xf, xf.data(), sizeof(EntXform) * xf.size(), cudaMemcpyHostToDevice, st));

    const size_t nn = std::max<uint32_t>(n, 1);
    // binned-SAH topology for scenes larger than one segment (the context's build setting), else
    // Karras' radix tree over the Morton order
    const bool sah = ctx->build_sah && n > (uint32_t)SAH_T;
    int root_index = 0;
    // scratch layout
    float* d_xyz = (float*)ctx_scratch(ctx, SCR_BUILD0, nn * 9 * sizeof(float));
    float* d_vnin = any_vn ? (float*)ctx_scratch(ctx, SCR_BUILD1, nn * 9 * sizeof(float)) : nullptr;
    for (uint32_t e = 0; e < n_ents; ++e) {
        if (!ents[e].n_tris) continue;
        const size_t b = (size_t)xf[e].first * 9 * sizeof(float), len = ents[e].n_tris * 9 * sizeof(float);
        CRT_CUDA(cudaMemcpyAsync((char*)d_xyz + b, ents[e].tri_xyz, len, cudaMemcpyDefault, st));
        if (d_vnin) {
            if (xf[e].has_vn) CRT_CUDA(cudaMemcpyAsync((char*)d_vnin + b, ents[e].tri_vn, len, cudaMemcpyDefault, st));
        }
    }
    // one scratch region carved into 256-byte aligned arrays (measured first, then assigned)
    float4 *geo = nullptr, *vn = nullptr, *tbox = nullptr, *cen = nullptr, *nbox = nullptr;
    uint32_t *prim_ent = nullptr, *code_a = nullptr, *idx_a = nullptr, *code_b = nullptr, *idx_b = nullptr;
    uint32_t* code_prim = nullptr;
    float* dpc = nullptr;
    uint32_t *hist = nullptr, *flags = nullptr, *keys = nullptr;
    int2 *child = nullptr, *range = nullptr, *front = nullptr, *front_b = nullptr;
    int* parent = nullptr;
    uint8_t* tl_depth = nullptr;
    int *tl_cnt = nullptr, *tl_pos = nullptr, *tl_par = nullptr;
    uint32_t* tl_sorted = nullptr;
    const size_t nb_sort = (nn + SORT_TILE - 1) / SORT_TILE;
    auto carve = [&](char* base) {
        size_t off = 0;
        auto take = [&](size_t bytes) {
            off = (off + 255) & ~size_t(255);
            char* p = base ? base + off : nullptr;
            off += bytes;
            return p;
        };
        geo = (float4*)take(nn * 48);
        vn = (float4*)take(any_vn ? nn * 48 : 16);
        prim_ent = (uint32_t*)take(nn * 4);
        tbox = (float4*)take(nn * 32);
        cen = (float4*)take(nn * 16);
        code_a = (uint32_t*)take(nn * 4);
        idx_a = (uint32_t*)take(nn * 4);
        code_prim = (uint32_t*)take(nn * 4);
        code_b = (uint32_t*)take(nn * 4);
        idx_b = (uint32_t*)take(nn * 4);
        hist = (uint32_t*)take(nb_sort * 256 * 4);
        child = (int2*)take(nn * 8);
        range = (int2*)take(nn * 8);
        parent = (int*)take(nn * 8);          // 2n - 1 entries: internal nodes then leaves
        flags = (uint32_t*)take(nn * 4);
        nbox = (float4*)take(nn * 64);        // 2n - 1 nodes x (lo, hi)
        dpc = (float*)take(nn * 32);          // collapse costs: 8 per internal node
        keys = (uint32_t*)take(64 * 4);
        front = (int2*)take(nn * 8 + 8);
        front_b = (int2*)take(nn * 8 + 8);
        tl_depth = (uint8_t*)take(nn);
        tl_cnt = (int*)take(nn * 4);
        tl_pos = (int*)take(nn * 8);          // 2n - 1 nodes
        tl_par = (int*)take(nn * 4);
        tl_sorted = (uint32_t*)take(nn * 4);
        return off;
    };
    const size_t total = carve(nullptr);
    carve((char*)ctx_scratch(ctx, SCR_BUILD2, total));

    CRT_CUDA(cudaMemsetAsync(parent, 0xFF, nn * 8, st));
    CRT_CUDA(cudaMemsetAsync(flags, 0, nn * 4, st));

    if (n) {
        k_transform<<<cdiv(n, BLOCK), BLOCK, 0, st>>>(d_xyz, d_vnin, d_xf, n_ents, n, geo, any_vn ? vn : nullptr,
                                                      prim_ent, tbox, cen);
        check_launch(ctx, "k_transform");
        uint32_t init[12];
        for (int k = 0; k < 12; ++k) init[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
        CRT_CUDA(cudaMemcpyAsync(keys, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_bounds<<<std::min<uint32_t>(cdiv(n, BLOCK), (uint32_t)ctx->sm_count * 4), BLOCK, 0, st>>>(tbox, cen, n, keys);
        check_launch(ctx, "k_bounds");
        k_morton<<<cdiv(n, BLOCK), BLOCK, 0, st>>>(cen, n, keys, code_a, idx_a);
        check_launch(ctx, "k_morton");
        if (sah) CRT_CUDA(cudaMemcpyAsync(code_prim, code_a, 4ull * n, cudaMemcpyDeviceToDevice, st));
        const uint32_t nb = cdiv(n, SORT_TILE);
        uint32_t *ka = code_a, *va = idx_a, *kb = code_b, *vb = idx_b;
        for (int shift = 0; shift < 32; shift += 8) {
            k_radix_hist<<<nb, SORT_THREADS, 0, st>>>(ka, n, shift, hist);
            check_launch(ctx, "k_radix_hist");
            k_scan<<<1, 1024, 0, st>>>(hist, nb * 256);
            check_launch(ctx, "k_scan");
            k_radix_scatter<<<nb, SORT_THREADS, 0, st>>>(ka, va, kb, vb, n, shift, hist);
            check_launch(ctx, "k_radix_scatter");
            std::swap(ka, kb);
            std::swap(va, vb);
        }
        // after 4 passes the sorted data is back in (code_a, idx_a)
        if (sah) root_index = sah_topology(ctx, (int)n, tbox, cen, keys, va, code_prim, child, range, parent);
        if ((!sah || root_index < 0) && n > 1) {   // radix tree (also when the SAH temporaries do not fit)
            root_index = 0;
            k_karras<<<cdiv(n - 1, BLOCK), BLOCK, 0, st>>>(ka, (int)n, child, range, parent);
            check_launch(ctx, "k_karras");
        }
        if (ctx->treelet_passes > 0 && n >= 8) {
            // treelet restructuring of the binary tree, then leaves renumbered depth-first
            k_tl_boxes<<<cdiv(n, BLOCK), BLOCK, 0, st>>>(va, tbox, (int)n, child, parent, nbox, flags, ctx->d_error);
            check_launch(ctx, "k_tl_boxes");
            const uint32_t tl_grid = std::min<uint32_t>(cdiv(n - 1, TL_WARPS), (uint32_t)ctx->sm_count * 16);
            for (uint32_t pass = 0; pass < ctx->treelet_passes; ++pass)
                for (int cls = 0; cls < 7; ++cls) {
                    k_tl_depth<<<cdiv(n - 1, BLOCK), BLOCK, 0, st>>>(parent, (int)n, tl_depth);
                    check_launch(ctx, "k_tl_depth");
                    k_treelet<<<tl_grid, 32 * TL_WARPS, 0, st>>>(child, parent, nbox, tl_depth, (int)n, cls, nullptr);
                    check_launch(ctx, "k_treelet");
                }
            CRT_CUDA(cudaMemsetAsync(flags, 0, nn * 4, st));
            k_tl_count<<<cdiv(n, BLOCK), BLOCK, 0, st>>>((int)n, child, parent, tl_cnt, flags, ctx->d_error);
            check_launch(ctx, "k_tl_count");
            k_tl_position<<<cdiv(2 * n - 1, BLOCK), BLOCK, 0, st>>>((int)n, child, parent, tl_cnt, tl_pos,
                                                                   ctx->d_error);
            check_launch(ctx, "k_tl_position");
            k_tl_relayout<<<cdiv(n, BLOCK), BLOCK, 0, st>>>((int)n, tl_pos, tl_cnt, va, tl_sorted, child, range, parent,
                                                           tl_par, ctx->d_error);
            check_launch(ctx, "k_tl_relayout");
            CRT_CUDA(cudaMemcpyAsync(va, tl_sorted, 4ull * n, cudaMemcpyDeviceToDevice, st));
            CRT_CUDA(cudaMemcpyAsync(parent + (n - 1), tl_par, 4ull * n, cudaMemcpyDeviceToDevice, st));
            CRT_CUDA(cudaMemsetAsync(flags, 0, nn * 4, st));
        }
        k_refit<<<cdiv(n, BLOCK), BLOCK, 0, st>>>(va, tbox, (int)n, child, parent, nbox, flags, range, dpc,
                                                  ctx->collapse_tri_cost, ctx->d_error);
        check_launch(ctx, "k_refit");
        idx_a = va;
    }

    // wide-node capacity: every wide node but the root is an internal child holding > 3 triangles
    const uint32_t cap = std::max<uint32_t>(1, n / 3 + 2);
    CRT_CUDA(cudaMalloc(&s->nodes, sizeof(WideNode) * cap));
    CRT_CUDA(cudaMalloc(&s->tris, sizeof(float4) * 3 * nn));
    CRT_CUDA(cudaMalloc(&s->leaf_prim, sizeof(uint32_t) * nn));
    CRT_CUDA(cudaMalloc(&s->leaf_entity, sizeof(uint32_t) * nn));
    if (any_vn) CRT_CUDA(cudaMalloc(&s->leaf_vn, sizeof(float4) * 3 * nn));
    uint32_t* counters = keys + 16;
    const uint32_t c0[3] = {1, 0, 0};
    CRT_CUDA(cudaMemcpyAsync(counters, c0, sizeof(c0), cudaMemcpyHostToDevice, st));
    int2 root = make_int2(n > 3 ? root_index : 0x7FFFFFFF, 0);
    CRT_CUDA(cudaMemcpyAsync(front, &root, sizeof(root), cudaMemcpyHostToDevice, st));

    CollapseArgs A;
    A.n = (int)n;
    A.child = child;
    A.range = range;
    A.nbox = nbox;
    A.sorted = idx_a;
    A.geo = geo;
    A.vn = any_vn ? vn : nullptr;
    A.prim_ent = prim_ent;
    A.nodes = s->nodes;
    A.tris = s->tris;
    A.leaf_prim = s->leaf_prim;
    A.leaf_vn = s->leaf_vn;
    A.leaf_entity = s->leaf_entity;
    A.counters = counters;
    A.node_cap = cap;
    A.err = ctx->d_error;
    A.dp = dpc;
    A.cost_tri = ctx->collapse_tri_cost;

    uint32_t fcount = 1, depth = 0;
    int2 *cur = front, *nxt = front_b;
    while (fcount) {
        CRT_CUDA(cudaMemsetAsync(counters + 2, 0, sizeof(uint32_t), st));
        k_collapse<<<cdiv(fcount, 128), 128, 0, st>>>(A, cur, fcount, nxt);
        check_launch(ctx, "k_collapse");
        ++depth;
        CRT_CUDA(cudaMemcpyAsync(&fcount, counters + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaStreamSynchronize(st));
        std::swap(cur, nxt);
        CRT_CHECK(depth < 200, CRT_ERR_DEVICE, "BVH collapse did not terminate");
    }
    uint32_t used[2];
    CRT_CUDA(cudaMemcpyAsync(used, counters, sizeof(used), cudaMemcpyDeviceToHost, st));
    uint32_t kb_h[6] = {0, 0, 0, 0, 0, 0};
    if (n) CRT_CUDA(cudaMemcpyAsync(kb_h, keys, sizeof(kb_h), cudaMemcpyDeviceToHost, st));
    CRT_CUDA(cudaEventRecord(ev1, st));
    CRT_CUDA(cudaStreamSynchronize(st));
    check_device_error(ctx, "BVH build");
    CRT_CHECK(used[1] == n, CRT_ERR_DEVICE, "BVH collapse placed " + std::to_string(used[1]) + " of " +
                                                std::to_string(n) + " triangles");
    float ms = 0;
    CRT_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    s->build_ms = ms;
    s->n_nodes = used[0];
    s->depth = depth;
    // the node array was sized for the worst case (n / 3 + 2 nodes); keep only the nodes used
    if (used[0] < cap) {
        WideNode* exact = nullptr;
        CRT_CUDA(cudaMalloc(&exact, sizeof(WideNode) * std::max<uint32_t>(used[0], 1)));
        CRT_CUDA(cudaMemcpyAsync(exact, s->nodes, sizeof(WideNode) * used[0], cudaMemcpyDeviceToDevice, st));
        CRT_CUDA(cudaStreamSynchronize(st));
        CRT_CUDA(cudaFree(s->nodes));
        s->nodes = exact;
    }
    for (int k = 0; k < 6; ++k) s->bounds[k] = n ? fkey_inv(kb_h[k]) : 0.f;
    s->device_bytes = sizeof(WideNode) * std::max<uint32_t>(used[0], 1) + nn * (48 + 4 + 4) + (any_vn ? nn * 48 : 0) +
                      sizeof(EntityDev) * s->host_entities.size();
}
