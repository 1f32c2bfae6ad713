// GPU BVH construction for a scene (replaces SweepSahBuilder + ParallelReinsertionOptimizer +
// NodeLayoutOptimizer of the reference, lib/bvh/sweep_sah_builder.hpp:43-111,
// parallel_reinsertion_optimizer.hpp:140-211, node_layout_optimizer.hpp:30-92).
//
// Pipeline, one stream, no host round trips except one frontier count per collapse level:
//   k_transform      entity transform chain in FP64 (transform.hpp:43-85), FP32 triangle
//                    records (p0, e1, e2, n), conservative FP32 boxes, centroids, normals
//   k_bounds         scene and centroid bounds (order-preserving integer atomics)
//   k_morton         30-bit Morton codes of centroids in the centroid bounds
//   radix_sort       stable LSD radix sort, 8-bit digits, 4 passes (histogram / scan / scatter)
//   k_karras         binary radix tree (Karras, "Maximizing parallelism in the construction of
//                    BVHs, octrees, and k-d trees", HPG 2012); ties broken by index
//   k_refit          bottom-up boxes, second arrival at each node does the union
//   k_collapse       top-down, level-synchronous collapse into 8-wide nodes: greedily open the
//                    largest-area child of more than 3 triangles until 8 slots are used (then
//                    split small leaves into free slots), children with <= 3 triangles become
//                    leaves, slots ordered by octant, child boxes quantised to 8 bits
//                    (Ylitie, Karras, Laine, "Efficient incoherent ray traversal on GPUs through
//                    compressed wide BVHs", HPG 2017); leaf triangles written contiguously.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int BLOCK = 256;
constexpr uint32_t NO_CHILD = 0xFFFFFFFFu;

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
    D3 p0 = {q[0], q[1], q[2]}, p1 = {q[3], q[4], q[5]}, p2 = {q[6], q[7], q[8]};
    // Triangle(p0, p1, p2): e1 = p0 - p1, e2 = p2 - p0 (triangle.hpp:31-33)
    D3 e1 = d3sub(p0, p1), e2 = d3sub(p2, p0);
    // resize_triangles: p0' = s p0, p1' = s p1(), p2' = s p2() with p1() = p0 - e1, p2() = p0 + e2
    {
        D3 a = d3scl(p0, X.scale), b = d3scl(d3sub(p0, e1), X.scale), c = d3scl(d3add(p0, e2), X.scale);
        p0 = a; e1 = d3sub(a, b); e2 = d3sub(c, a);
    }
    // rotate_triangles (also rotates vertex normals)
    {
        D3 a = d3rot(p0, X.rot), b = d3rot(d3sub(p0, e1), X.rot), c = d3rot(d3add(p0, e2), X.rot);
        p0 = a; e1 = d3sub(a, b); e2 = d3sub(c, a);
    }
    // translate_triangles
    {
        D3 t = {X.pos[0], X.pos[1], X.pos[2]};
        D3 a = d3add(p0, t), b = d3add(d3sub(p0, e1), t), c = d3add(d3add(p0, e2), t);
        p0 = a; e1 = d3sub(a, b); e2 = d3sub(c, a);
    }
    D3 nn = d3cross(e1, e2);
    geo[3ull * i + 0] = make_float4((float)p0.x, (float)p0.y, (float)p0.z, (float)e1.x);
    geo[3ull * i + 1] = make_float4((float)e1.y, (float)e1.z, (float)e2.x, (float)e2.y);
    geo[3ull * i + 2] = make_float4((float)e2.z, (float)nn.x, (float)nn.y, (float)nn.z);
    // Box of the FP32 triangle as the intersection test sees it (p0, p0 - e1, p0 + e2 evaluated
    // exactly in FP64 from the FP32 values), rounded outward.
    double P0[3] = {(float)p0.x, (float)p0.y, (float)p0.z};
    double E1[3] = {(float)e1.x, (float)e1.y, (float)e1.z};
    double E2[3] = {(float)e2.x, (float)e2.y, (float)e2.z};
    float lo[3], hi[3], cc[3];
    for (int k = 0; k < 3; ++k) {
        double a = P0[k], b = P0[k] - E1[k], c = P0[k] + E2[k];
        lo[k] = __double2float_rd(fmin(a, fmin(b, c)));
        hi[k] = __double2float_ru(fmax(a, fmax(b, c)));
        cc[k] = (float)((a + b + c) * (1.0 / 3.0));
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

// ---------------------------------------------------------------- refit
// node boxes: 2 float4 per node; internal nodes [0, n-1), leaves [n-1, 2n-1)
__global__ void k_refit(const uint32_t* __restrict__ sorted, const float4* __restrict__ tbox, int n,
                        const int2* __restrict__ child, const int* __restrict__ parent, float4* nbox,
                        uint32_t* __restrict__ flags) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t p = sorted[j];
    float4 lo = tbox[2ull * p], hi = tbox[2ull * p + 1];
    nbox[2ull * (n - 1 + j)] = lo;
    nbox[2ull * (n - 1 + j) + 1] = hi;
    int node = parent[n - 1 + j];
    while (node >= 0) {
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
        node = node == 0 ? -1 : parent[node];
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
        int2 c = A.child[bnode];
        refs[0] = c.x;
        refs[1] = c.y;
        nc = 2;
        // open the largest-area child that would otherwise become an internal node (> 3 triangles);
        // only when none is left, split small leaves to fill the remaining slots
        while (nc < 8) {
            int best = -1;
            bool best_big = false;
            float best_area = -1.f;
            for (int k = 0; k < nc; ++k) {
                if (refs[k] < 0) continue;     // leaf of the binary tree: cannot open
                const bool big = ref_count(A, refs[k]) > 3;
                const size_t bi = box_index(n, refs[k]);
                const float4 lo = A.nbox[2 * bi], hi = A.nbox[2 * bi + 1];
                const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
                const float area = dx * dy + dy * dz + dz * dx;
                if ((big && !best_big) || (big == best_big && area > best_area)) {
                    best_area = area;
                    best = k;
                    best_big = big;
                }
            }
            if (best < 0) break;
            const int2 c2 = A.child[refs[best]];
            refs[best] = c2.x;
            refs[nc++] = c2.y;
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
            const double q = ldexp(1.0, ex[a]);
            double l = floor(((double)clo[k][a] - (double)p[a]) / q);
            double h = ceil(((double)chi[k][a] - (double)p[a]) / q);
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
    w.w[2] = make_float4(__uint_as_float(pack4(qlo[0])), __uint_as_float(pack4(qlo[0] + 4)),
                         __uint_as_float(pack4(qlo[1])), __uint_as_float(pack4(qlo[1] + 4)));
    w.w[3] = make_float4(__uint_as_float(pack4(qlo[2])), __uint_as_float(pack4(qlo[2] + 4)),
                         __uint_as_float(pack4(qhi[0])), __uint_as_float(pack4(qhi[0] + 4)));
    w.w[4] = make_float4(__uint_as_float(pack4(qhi[1])), __uint_as_float(pack4(qhi[1] + 4)),
                         __uint_as_float(pack4(qhi[2])), __uint_as_float(pack4(qhi[2] + 4)));
    A.nodes[wnode] = w;
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
    uint32_t *hist = nullptr, *flags = nullptr, *keys = nullptr;
    int2 *child = nullptr, *range = nullptr, *front = nullptr, *front_b = nullptr;
    int* parent = nullptr;
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
        code_b = (uint32_t*)take(nn * 4);
        idx_b = (uint32_t*)take(nn * 4);
        hist = (uint32_t*)take(nb_sort * 256 * 4);
        child = (int2*)take(nn * 8);
        range = (int2*)take(nn * 8);
        parent = (int*)take(nn * 8);          // 2n - 1 entries: internal nodes then leaves
        flags = (uint32_t*)take(nn * 4);
        nbox = (float4*)take(nn * 64);        // 2n - 1 nodes x (lo, hi)
        keys = (uint32_t*)take(64 * 4);
        front = (int2*)take(nn * 8 + 8);
        front_b = (int2*)take(nn * 8 + 8);
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
        if (n > 1) {
            k_karras<<<cdiv(n - 1, BLOCK), BLOCK, 0, st>>>(ka, (int)n, child, range, parent);
            check_launch(ctx, "k_karras");
        }
        k_refit<<<cdiv(n, BLOCK), BLOCK, 0, st>>>(va, tbox, (int)n, child, parent, nbox, flags);
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
    int2 root = make_int2(n > 3 ? 0 : 0x7FFFFFFF, 0);
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
    for (int k = 0; k < 6; ++k) s->bounds[k] = n ? fkey_inv(kb_h[k]) : 0.f;
    s->device_bytes = sizeof(WideNode) * cap + nn * (48 + 4 + 4) + (any_vn ? nn * 48 : 0) +
                      sizeof(EntityDev) * s->host_entities.size();
}
