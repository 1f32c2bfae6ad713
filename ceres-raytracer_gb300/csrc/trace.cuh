// Persistent trace-kernel template shared by every query, plus surface reconstruction helpers.
#pragma once

#include "common.cuh"
#include "traverse.cuh"

#include <type_traits>

#ifndef CRT_TRACE_BLOCK
#define CRT_TRACE_BLOCK 128
#endif
// resident blocks per SM the trace kernel is compiled for (registers per thread: 65536 / (128 x 7),
// 72 after allocation granularity).  With the half-precision plane rows of the 8-wide node, 8 blocks
// (64 registers) spill in the traversal loop and lose more than the eighth block's warps bring.
#ifndef CRT_TRACE_MIN_BLOCKS
#define CRT_TRACE_MIN_BLOCKS 7
#endif

__host__ __device__ __forceinline__ SceneView scene_view(const crt_scene* s) {
    SceneView v;
    v.nodes = s->nodes;
    v.tris = s->tris;
    v.leaf_prim = s->leaf_prim;
    v.leaf_vn = s->leaf_vn;
    v.leaf_entity = s->leaf_entity;
    v.entities = s->entities;
    v.n_tris = (uint32_t)s->n_tris;
    return v;
}

// SimpleCamera::pixel_to_ray in FP32 from the FP64-derived basis: d = normalize(a + u b + v c).
__device__ __forceinline__ TRay camera_ray(const CamBasis& c, float u, float v) {
    TRay r;
    const float3 d = f3(fmaf(v, c.c[0], fmaf(u, c.b[0], c.a[0])), fmaf(v, c.c[1], fmaf(u, c.b[1], c.a[1])),
                        fmaf(v, c.c[2], fmaf(u, c.b[2], c.a[2])));
    r.d = normalize3(d);
    r.o = f3(c.o[0], c.o[1], c.o[2]);
    r.tmin = 0.f;
    r.tmax = 3.402823466e38f;
    return r;
}

struct SurfacePoint {
    float3 x;           // u p1 + v p2 + (1-u-v) p0  (passes.hpp:53)
    float3 flat_n;      // normalize(n), left-handed (inward) like the reference
    float3 shading_n;   // smooth ? normalize(u vn1 + v vn2 + w vn0) : flat_n  (passes.hpp:179)
    uint32_t entity;
    uint32_t id;
};

__device__ __forceinline__ SurfacePoint surface_point(const SceneView& sv, const THit& h) {
    SurfacePoint sp;
    const float4* tp = sv.tris + 3ull * h.slot;
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    const float3 p0 = f3(a.x, a.y, a.z), n = f3(c.y, c.z, c.w);
    // u p1 + v p2 + (1 - u - v) p0 = p0 + u (p1 - p0) + v (p2 - p0)
    sp.x = tri_point(a, b, c, h.u, h.v);
    sp.flat_n = normalize3(n);
    sp.entity = __ldg(sv.leaf_entity + h.slot);
    const EntityDev& E = sv.entities[sp.entity];
    sp.id = E.id;
    if (E.smooth && sv.leaf_vn) {
        const float4* vp = sv.leaf_vn + 3ull * h.slot;
        const float4 v0 = __ldg(vp), v1 = __ldg(vp + 1), v2 = __ldg(vp + 2);
        const float w = 1.0f - h.u - h.v;
        sp.shading_n = normalize3(f3(h.u * v1.x + h.v * v2.x + w * v0.x, h.u * v1.y + h.v * v2.y + w * v0.y,
                                     h.u * v1.z + h.v * v2.z + w * v0.z));
    } else {
        sp.shading_n = sp.flat_n;
    }
    return sp;
}

// Jobs: ray(i, r, item) builds the ray of work item i and returns 1 to trace it, 0 when the item has
// no ray (padding), or 2 when the ray is resolved without a traversal (a miss known from a bounding
// test; the job has nothing to store, and the counting build counts it among the resolved rays);
// bool results mean 1 / 0.  view(sv, item) names the scene to traverse (requests of one launch may
// use different resident scenes), and write(sv, i, r, hit, item) stores the result.  JobBase
// supplies the single-scene defaults.
struct JobBase {
    struct Item {};
    __device__ __forceinline__ const SceneView& view(const SceneView& sv, const Item&) const { return sv; }
};

// Persistent ray-queue kernel.  Each warp takes groups of 32 consecutive items per atomic grab: with
// chunk == 1 one group, otherwise a guided size of up to `chunk` groups, shrinking with the work
// left so that the last grabs stay small (few atomics on the queue counter while much work is left,
// balance at the end).
// Resident blocks per SM for one job type: CRT_TRACE_MIN_BLOCKS unless the job names its own
// (kMinBlocks).  crt_trace_closest's job runs 5 % faster at 6 blocks (80 registers); the any-hit,
// LiDAR, pass and render jobs measured the same or slower there.  launch_trace sizes the persistent
// grid from the occupancy the kernel gets.
template <class J, class = void>
struct trace_min_blocks {
    static constexpr int value = CRT_TRACE_MIN_BLOCKS;
};
template <class J>
struct trace_min_blocks<J, std::void_t<decltype(J::kMinBlocks)>> {
    static constexpr int value = J::kMinBlocks;
};

template <bool ANY, bool COUNT, class Job>
__global__ void __launch_bounds__(CRT_TRACE_BLOCK, trace_min_blocks<Job>::value) k_trace(SceneView sv, Job job, uint32_t n_items,
                                                            const uint32_t* __restrict__ n_dev,
                                                            uint32_t* __restrict__ queue, uint32_t* __restrict__ err,
                                                            unsigned long long* __restrict__ counters, uint32_t chunk) {
    extern __shared__ uint2 sstack[];
    if (n_dev) n_items = *n_dev;   // item count produced by an earlier kernel on the stream
    const int lane = threadIdx.x & 31;
    TravStats st{0u, 0u};
    uint32_t nrays = 0, nres = 0;
    const uint32_t warps_total = gridDim.x * (blockDim.x >> 5);
    while (true) {
        uint32_t base = 0, take = 1;
        if (lane == 0) {
            if (chunk > 1) {
                const uint32_t cur = *reinterpret_cast<volatile uint32_t*>(queue);
                const uint32_t left = cur < n_items ? (n_items - cur) >> 5 : 0u;
                take = min(chunk, max(1u, left / (4u * warps_total)));
            }
            base = atomicAdd(queue, 32u * take);
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        take = __shfl_sync(0xffffffffu, take, 0);
        if (base >= n_items) break;
        for (uint32_t c = 0; c < take; ++c) {
            const uint32_t i = base + 32u * c + lane;
            TRay r;
            typename Job::Item it;
            const int kind = i < n_items ? (int)job.ray(i, r, it) : 0;
            if (kind == 1) {
                const THit h = traverse<ANY, COUNT>(job.view(sv, it), r, sstack + threadIdx.x, CRT_TRACE_BLOCK, st, err);
                job.write(sv, i, r, h, it);
            }
            if (COUNT) {
                nrays += kind == 1;
                nres += kind == 2;
            }
        }
    }
    if (COUNT) {
        unsigned long long a = nrays, b = st.nodes, c = st.tris, d = nres;
        for (int o = 16; o; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
            d += __shfl_xor_sync(0xffffffffu, d, o);
        }
        if (lane == 0) {
            atomicAdd(counters + 0, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
            if (d) atomicAdd(counters + 3, d);
        }
    }
}

// Launches the persistent trace kernel over n_items work items (or over *n_dev items when n_dev is
// given: n_items is then the upper bound used to size the grid).
template <bool ANY, class Job>
void launch_trace(crt_context* ctx, const SceneView& sv, const Job& job, uint32_t n_items,
                  const uint32_t* n_dev = nullptr, uint32_t* queue = nullptr, uint32_t chunk_override = 0) {
    if (!queue) queue = (uint32_t*)ctx_scratch(ctx, SCR_QUEUE, 256);
    CRT_CUDA(cudaMemsetAsync(queue, 0, sizeof(uint32_t), ctx->stream));
    const size_t smem = (size_t)CRT_STACK_SMEM * CRT_TRACE_BLOCK * sizeof(uint2);
    const void* kfn = ctx->counting ? (const void*)k_trace<ANY, true, Job> : (const void*)k_trace<ANY, false, Job>;
    int grid = occupancy_grid(ctx, kfn, CRT_TRACE_BLOCK, smem);
    const uint32_t need = (n_items + CRT_TRACE_BLOCK - 1) / CRT_TRACE_BLOCK;
    if ((uint32_t)grid > need) grid = (int)std::max<uint32_t>(need, 1u);
    const uint32_t chunk = chunk_override ? chunk_override : (ctx->queue_chunk ? ctx->queue_chunk : 1u);
    if (ctx->counting)
        k_trace<ANY, true, Job><<<grid, CRT_TRACE_BLOCK, smem, ctx->stream>>>(sv, job, n_items, n_dev, queue,
                                                                             ctx->d_error, ctx->d_counters, chunk);
    else
        k_trace<ANY, false, Job><<<grid, CRT_TRACE_BLOCK, smem, ctx->stream>>>(sv, job, n_items, n_dev, queue,
                                                                              ctx->d_error, ctx->d_counters, chunk);
    check_launch(ctx, "k_trace");
}

template <bool ANY, class Job>
void launch_trace(crt_scene* s, const Job& job, uint32_t n_items, const uint32_t* n_dev = nullptr,
                  uint32_t* queue = nullptr) {
    launch_trace<ANY>(s->ctx, scene_view(s), job, n_items, n_dev, queue);
}
