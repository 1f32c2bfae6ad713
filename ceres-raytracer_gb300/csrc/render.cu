// Batched wavefront path tracer and LiDAR scans: do_render (src/crt/do_render.hpp:28-141) with
// unidirectional (path_tracing/unidirectional.hpp:24-96), restated as stage kernels over compacted
// queues that serve many requests (renders and LiDAR grids, possibly on different resident scenes)
// per launch:
//
//   begin     copy this wave's descriptor, reset the queue counters          (k_wave_begin)
//   primary   LiDAR beams of the batch + camera ray per (pixel, sample)       (persistent trace)
//             (+ the sun rays of one SRP range in crt_batch_mixed waves, whose shade and specular
//             segments follow: srp_wave_stages)
//   shade     surface point, one shadow ray per light, bounce ray             (k_shade)
//   shadow    any hit for the shadow queue                                     (persistent trace)
//   accum     sum lights, clamp after the first bounce, times path weight      (k_accum; folded into
//             k_update when the wave has at most one bounce: bounce 0's weight is the constant
//             2 pi and its radiance starts at zero, so neither is stored)
//   bounce    closest hit for the continuing-path queue                        (persistent trace)
//   update    per-pixel running mean and adaptive stop, samples in order       (k_update; with a
//             fixed sample count the request's last slice also stores the outputs)
//   finalize  RGBA float and clamp(v * 256, 0, 255) bytes per request          (k_finalize; the
//             adaptive requests)
//
// A wave is a list of slices, each slice = samples [s0, s0 + ns) of the pixel set of one request.
// Path p of a slice maps to sample s0 + q / npix and pixel q % npix (q = p - slice.path_base), and
// k_update consumes a pixel's samples in order, so images do not depend on how requests and samples
// are grouped into waves: a request renders bit-identically alone or in a batch.  Random numbers
// come from Philox4x32-10 keyed by (seed, request) with counter (pixel, sample, bounce<<8 | purpose,
// request).  Every stage kernel reads the wave from device memory, so when no request samples
// adaptively the whole wave plan is uploaded once and each wave is one CUDA-graph replay.
//
// FP32 secondary-ray origins: the reference offsets the hit point by 1e-4 along the flat normal
// (unidirectional.hpp:59-61).  In FP32 at kilometre coordinates 1e-4 is about one ulp, so the
// offset used here is max(1e-4, 4 ulp of the largest coordinate), and the triangle a bounce ray
// leaves is not re-tested unless the ray points into its plane (smooth shading: the reference then
// meets that triangle again, and so does the device ray).  A shadow ray that points into the surface
// meets the plane of its own triangle in the reference; the shade stage decides from the reference's
// geometry whether that crossing lies inside the triangle (mark_self_occluded) and traces the others
// with their own triangle tested like any other, so that the watertight test settles crossings at
// its edges.
#include "common.cuh"
#include "srp.cuh"
#include "trace.cuh"

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

namespace {

constexpr int MAX_LIGHTS = 16;
constexpr int MAX_SLICES = 128;
constexpr int MAX_LIDAR = 256;

struct LightDev {
    int type;
    float intensity;
    float pos[3];
    float R[9];
    float size[2];
};

struct RenderCtl {
    uint32_t W, H;
    int min_samples, max_samples;
    float noise_threshold;
    int num_bounces;
    uint32_t seed_lo, seed_hi, request;
};

struct RReq {            // render request
    SceneView sv;
    CamBasis cam;
    RenderCtl c;
    uint32_t light_base, n_lights;
    uint32_t pix_base, npix;
    uchar4* rgba;        // device outputs (staging when the caller passed host memory)
    float4* rad;
    uint32_t fin_update; // 1: the request's last slice stores the outputs (k_update), not k_finalize
};

struct LReq {            // LiDAR beam-grid request
    SceneView sv;
    double o[3];
    double rt[9];        // R^T row-major
    double zsign;
    uint32_t nx, ny;
    uint32_t tan_base;   // nx + ny tangents in the batch table
    uint32_t item_base;  // first primary item (8 x 4 tile order)
    double* range;
    uint32_t* prim;
};

struct Slice {
    uint32_t req, s0, ns, npix;
    uint32_t path_base, upd_base;
    const uint32_t* active;   // pixel set of the slice (nullptr: every pixel of the request)
};

struct WaveDesc {
    uint32_t n_lidar_items, n_lreq, n_paths, n_primary;
    uint32_t n_slices, n_update, n_srp_items, pad0;
    Slice slices[MAX_SLICES];
    SrpStage srp;         // SRP items of the wave (crt_batch_mixed, serving): one request's sun rays,
                          // after the LiDAR beams and camera paths in the primary trace
};

struct Batch {
    const RReq* rr;
    const LReq* lr;
    const LightDev* lights;
    const double* tan;
    const WaveDesc* descs;
    WaveDesc* cur;
    uint32_t* wave_idx;
    uint32_t* counts;          // [0] |bounce queue in| [1] |bounce queue out| [2] |shadow queue|
    uint32_t L;                // light stride per path
    float4* ray;
    uint32_t* skip;
    float4* hit;
    float4* wgt[2];            // path weight at bounce b >= 1 in wgt[b & 1] (bounce 0: path_weight's constant)
    float4* rad;               // radiance gathered so far (written from bounce 0's accumulation on)
    uint32_t* preq;
    uint32_t* ppix;
    uint32_t* psample;
    float4* contrib;
    uint8_t* occ;
    float4* sray;              // shadow ray of path p, light l at p * L + l: (origin, skip slot bits) (dir, tmax)
    uint2* sidx;               // shadow queue: (p * L + l, request) of each shadow ray to trace, in path order
    float4* pix;               // per-pixel running mean (all render requests)
    uint32_t* taken;
    uint8_t* done;
};

__device__ __forceinline__ void rng2(const RenderCtl& c, uint32_t pixel, uint32_t sample, uint32_t bounce,
                                     uint32_t purpose, float& a, float& b) {
    uint32_t ctr[4] = {pixel, sample, (bounce << 8) | purpose, c.request};
    philox4x32(ctr, c.seed_lo, c.seed_hi);
    a = unif24(ctr[0]);
    b = unif24(ctr[1]);
}

// cosine_importance (materials/brdfs.hpp:18-42): Malley's method about a left-handed normal
__device__ __forceinline__ float3 cosine_importance(float3 n, float r1, float r2) {
    const float r = sqrtf(r1);
    const float theta = r2 * 2.0f * 3.1415926f;
    float s, c;
    sincosf(theta, &s, &c);
    const float x = -r * c, y = -r * s;
    const float z = -sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y));
    float3 nx;
    if (fabsf(n.x) > fabsf(n.y)) nx = f3(n.z, 0.0f, -n.x) * (1.0f / sqrtf(n.x * n.x + n.z * n.z));
    else nx = f3(0.0f, n.z, -n.y) * (1.0f / sqrtf(n.y * n.y + n.z * n.z));
    const float3 ny = cross3(n, nx);
    return nx * x + ny * y + n * z;
}

__device__ __forceinline__ float origin_offset(float3 x) {
    const float m = fmaxf(fabsf(x.x), fmaxf(fabsf(x.y), fabsf(x.z)));
    int e;
    frexpf(m, &e);
    return fmaxf(1e-4f, ldexpf(1.0f, e - 24 + 2));   // 4 ulps of m
}

__device__ __forceinline__ uint32_t find_slice_by_path(const WaveDesc& w, uint32_t p) {
    uint32_t lo = 0, hi = w.n_slices;   // last slice with path_base <= p
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (w.slices[mid].path_base <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Pixel of path slot j of a full-image slice: 8 x 4 tiles in row-major tile order, so a warp's 32
// camera rays cover one tile (which shares more BVH nodes than 32 pixels of one row: about 12 %
// faster primary and shadow traversal).  A bijection of [0, W*H) for any W, H: rows are grouped in
// bands of 4 (the last band may be lower) and a band's last tile is W mod 8 wide.
__device__ __forceinline__ uint32_t tile_slot_pixel(uint32_t j, uint32_t W, uint32_t H) {
    const uint32_t y0 = j / (4u * W) * 4u;
    const uint32_t hb = min(4u, H - y0);
    const uint32_t r = j - y0 * W;
    const uint32_t full = W >> 3;
    const uint32_t tx = min(r / (8u * hb), full);
    const uint32_t rr = r - tx * 8u * hb;
    const uint32_t wt = tx < full ? 8u : W - 8u * full;   // r < hb * W keeps wt > 0 here
    return (y0 + rr / wt) * W + tx * 8u + rr % wt;
}

__device__ __forceinline__ bool tile_px(uint32_t i, uint32_t W, uint32_t H, uint32_t& px, uint32_t& py) {
    const uint32_t tiles_x = (W + 7) >> 3;
    const uint32_t tile = i >> 5, w = i & 31u;
    px = (tile % tiles_x) * 8u + (w & 7u);
    py = (tile / tiles_x) * 4u + (w >> 3);
    return px < W && py < H;
}

// ---------------------------------------------------------------- primary stage
// Primary segment of a wave: items [0, LiDAR) are beams, then camera paths, then (SRP) the sun rays
// of the wave's SRP request.  Batches without SRP requests use the SRP = false instantiation.
template <bool SRP>
struct PrimaryJobT {
    Batch B;
    struct Item {
        uint32_t req;
        uint32_t lidar;   // 0 camera path, 1 LiDAR beam, 2 SRP sun ray
    };
    __device__ SceneView view(const SceneView&, const Item& it) const {
        if (SRP && it.lidar == 2) return B.cur->srp.sv;
        return it.lidar ? B.lr[it.req].sv : B.rr[it.req].sv;
    }
    __device__ void beam64(const LReq& L, uint32_t px, uint32_t py, double d[3]) const {
        const double s0 = B.tan[L.tan_base + px], s1 = B.tan[L.tan_base + L.nx + py], s2 = L.zsign;
        const double inv = rsqrt64(s0 * s0 + s1 * s1 + s2 * s2);
        for (int k = 0; k < 3; ++k) d[k] = (L.rt[3 * k] * s0 + L.rt[3 * k + 1] * s1 + L.rt[3 * k + 2] * s2) * inv;
    }
    __device__ int ray(uint32_t i, TRay& r, Item& it) const {   // k_trace job contract (0, 1, 2)
        const WaveDesc& w = *B.cur;
        if (i < w.n_lidar_items) {
            uint32_t lo = 0, hi = w.n_lreq;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (B.lr[mid].item_base <= i) lo = mid;
                else hi = mid;
            }
            const LReq& L = B.lr[lo];
            uint32_t px, py;
            if (!tile_px(i - L.item_base, L.nx, L.ny, px, py)) return false;
            double d[3];
            beam64(L, px, py, d);
            r.o = f3((float)L.o[0], (float)L.o[1], (float)L.o[2]);
            r.d = f3((float)d[0], (float)d[1], (float)d[2]);
            r.tmin = 0.f;
            r.tmax = 3.402823466e38f;
            it.req = lo;
            it.lidar = 1;
            return true;
        }
        if (SRP && i >= w.n_lidar_items + w.n_paths) {
            const uint32_t k = i - w.n_lidar_items - w.n_paths;
            it.req = k;
            it.lidar = 2;
            return srp_primary_ray(w.srp.W, k, r);
        }
        const uint32_t p = i - w.n_lidar_items;
        const Slice& S = w.slices[find_slice_by_path(w, p)];
        const uint32_t q = p - S.path_base;
        const uint32_t a = q % S.npix;
        const uint32_t sample = S.s0 + q / S.npix;
        const RReq& R = B.rr[S.req];
        const uint32_t pixel = S.active ? S.active[a] : tile_slot_pixel(a, R.c.W, R.c.H);
        float u = (float)(pixel % R.c.W), v = (float)(pixel / R.c.W);
        if (R.c.max_samples != 1) {   // do_render.hpp:76-82: pixel corner for a single sample
            float ja, jb;
            rng2(R.c, pixel, sample, 0, 0, ja, jb);
            u += ja - 0.5f;
            v += jb - 0.5f;
        }
        r = camera_ray(R.cam, u, v);
        B.preq[p] = S.req;
        B.ppix[p] = pixel;
        B.psample[p] = sample;
        it.req = S.req;
        it.lidar = 0;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t i, const TRay&, const THit& h, const Item& it) const {
        if (SRP && it.lidar == 2) {
            srp_store_primary(B.cur->srp.W, it.req, h);
            return;
        }
        if (it.lidar) {
            const LReq& L = B.lr[it.req];
            uint32_t px, py;
            tile_px(i - L.item_base, L.nx, L.ny, px, py);
            const size_t k = (size_t)py * L.nx + px;
            double rng = 0.0;
            if (h.slot != CRT_MISS) {
                double d[3];
                beam64(L, px, py, d);
                const double t = plane_t64(L.sv.tris, h.slot, L.o, d);
                rng = isfinite(t) ? t : (double)h.t;
            }
            L.range[k] = rng;
            if (L.prim) L.prim[k] = h.slot != CRT_MISS ? L.sv.leaf_prim[h.slot] : CRT_MISS;
            return;
        }
        const uint32_t p = i - B.cur->n_lidar_items;
        B.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    }
};

struct ShadowJob {
    Batch B;
    struct Item {
        uint32_t req, k;
    };
    __device__ SceneView view(const SceneView&, const Item& it) const { return B.rr[it.req].sv; }
    __device__ bool ray(uint32_t i, TRay& r, Item& it) const {
        const uint2 q = B.sidx[i];
        const uint32_t k = q.x;
        const float4 a = B.sray[2ull * k], b = B.sray[2ull * k + 1];
        r.o = f3(a.x, a.y, a.z);
        r.tmin = 0.0f;
        r.skip = __float_as_uint(a.w);
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        it.req = q.y;
        it.k = k;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t, const TRay&, const THit& h, const Item& it) const {
        if (h.slot != CRT_MISS) B.occ[it.k] = 1;
    }
};

struct BounceJob {
    Batch B;
    const uint32_t* q;
    struct Item {
        uint32_t req;
        uint32_t p;
    };
    __device__ SceneView view(const SceneView&, const Item& it) const { return B.rr[it.req].sv; }
    __device__ bool ray(uint32_t i, TRay& r, Item& it) const {
        const uint32_t p = q[i];
        const float4 a = B.ray[2ull * p], b = B.ray[2ull * p + 1];
        r.o = f3(a.x, a.y, a.z);
        r.tmin = a.w;
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        r.skip = B.skip[p];
        it.req = B.preq[p];
        it.p = p;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t, const TRay&, const THit& h, const Item& it) const {
        B.hit[it.p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    }
};

// warp-aggregated append of `cnt` entries per participating lane (counts may differ between lanes:
// lanes of one warp can belong to requests with different light counts); returns the lane's first index
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, uint32_t cnt) {
    const uint32_t mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t prefix = 0, total = 0;
    for (uint32_t m = mask; m; m &= m - 1) {
        const int j = __ffs(m) - 1;
        const uint32_t c = __shfl_sync(mask, cnt, j);
        if (j < lane) prefix += c;
        total += c;
    }
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, total);
    base = __shfl_sync(mask, base, leader);
    return base + prefix;
}

__global__ void k_wave_begin(Batch B) {
    const WaveDesc* src = B.descs + *B.wave_idx;
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(B.cur);
    for (uint32_t k = threadIdx.x; k < sizeof(WaveDesc) / 4; k += blockDim.x) d[k] = s[k];
    if (threadIdx.x == 0) B.counts[0] = B.counts[1] = B.counts[2] = 0;
}
__global__ void k_wave_end(Batch B) { *B.wave_idx += 1; }
__global__ void k_queue_rotate(uint32_t* counts) {
    counts[0] = counts[1];
    counts[1] = 0;
    counts[2] = 0;
}

// Path weight at bounce b: Color(2*M_PI) at the camera vertex (unidirectional.hpp:38), then
// multiplied by (1 - r1) per bounce (k_shade)
__device__ __forceinline__ float4 path_weight(const Batch& B, uint32_t p, int bounce) {
    const float w0 = (float)(2.0 * 3.14159265358979323846);
    return bounce == 0 ? make_float4(w0, w0, w0, 0.f) : B.wgt[bounce & 1][p];
}

// ---------------------------------------------------------------- shade
// Block-wide ordered append of two counts per thread (n0 <= 16 lights, n1 <= 1, 256-thread blocks: each
// block total fits 16 bits of a packed word): one atomicAdd per counter and block instead of one per
// warp, since every append of a stage goes to the same counter and atomics on one address serialise
// in one L2 slice.  Every thread of the block calls it; returns the thread's first index in each queue.
__device__ __forceinline__ uint2 block_append2(uint32_t* c0, uint32_t n0, uint32_t* c1, uint32_t n1) {
    __shared__ uint32_t s_off[32];
    __shared__ uint32_t s_base[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t v = n0 | (n1 << 16);
    uint32_t x = v;   // inclusive scan over the warp
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_off[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < nw ? s_off[lane] : 0u;
        uint32_t incl = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane < nw) s_off[lane] = incl - w;
        if (lane == 31) {   // block totals
            const uint32_t t0 = incl & 0xFFFFu, t1 = incl >> 16;
            s_base[0] = t0 ? atomicAdd(c0, t0) : 0u;
            s_base[1] = t1 ? atomicAdd(c1, t1) : 0u;
        }
    }
    __syncthreads();
    const uint32_t ex = s_off[warp] + x - v;
    const uint2 r = make_uint2(s_base[0] + (ex & 0xFFFFu), s_base[1] + (ex >> 16));
    __syncthreads();   // the shared words are rewritten by the next call
    return r;
}

// Block-wide append of at most one entry per thread into 8 buckets (key 0..7; 8: none), for 256-thread
// blocks: one atomicAdd per block; within the block's range the entries are ordered by bucket, then
// by thread.  Every thread of the block calls it; returns the thread's index (undefined for key 8).
__device__ __forceinline__ uint32_t block_append_buckets8(uint32_t* counter, uint32_t key) {
    __shared__ uint32_t s_cnt[8][8];   // [warp][bucket]: counts, then offsets
    __shared__ uint32_t s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t rank = 0;
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, key == k);
        if (lane == 0) s_cnt[warp][k] = __popc(m);
        if (key == k) rank = __popc(m & ((1u << lane) - 1u));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int k = 0; k < 8; ++k)
            for (int w = 0; w < 8; ++w) {
                const uint32_t c = s_cnt[w][k];
                s_cnt[w][k] = t;
                t += c;
            }
        s_base = t ? atomicAdd(counter, t) : 0u;
    }
    __syncthreads();
    const uint32_t r = key < 8u ? s_base + s_cnt[warp][key] + rank : 0u;
    __syncthreads();   // the shared words are rewritten by the next call
    return r;
}

// Flat unit normal of path p's current triangle (xyz) and the distance from its hit point to the
// nearest edge of the triangle (barycentric x height, w).  w is NaN for a degenerate triangle.
// Reloads the hit and the triangle (cached) instead of keeping them live in k_shade.
__device__ __forceinline__ float4 edge_clearance(const Batch& B, uint32_t p, const RReq& R) {
    const float4 hv = B.hit[p];
    const float4* tp = R.sv.tris + 3ull * __float_as_uint(hv.w);
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    const float3 p0 = f3(a.x, a.y, a.z), p1 = f3(a.w, b.x, b.y), p2 = f3(b.z, b.w, c.x), n = f3(c.y, c.z, c.w);
    const float3 e1 = p0 - p1, e2 = p2 - p0;       // triangle.hpp:31-33
    const float an = sqrtf(dot3(n, n));            // twice the area
    const float w = 1.0f - hv.y - hv.z;
    const float d1 = hv.y * an / sqrtf(dot3(e2, e2));            // edge p0-p2, opposite p1
    const float d2 = hv.z * an / sqrtf(dot3(e1, e1));            // edge p0-p1, opposite p2
    const float d0 = w * an / sqrtf(dot3(p2 - p1, p2 - p1));     // edge p1-p2, opposite p0
    const float3 fn = n * (1.0f / an);   // normalize3(n), as surface_point
    return make_float4(fn.x, fn.y, fn.z, fminf(fminf(d0, d1), d2));
}

// Whether the reference's shadow ray toward `dir` (light at distance `dist`) stops on the triangle it
// leaves.  The reference starts it at x - 1e-4 n (unidirectional.hpp:55-57, n the flat normal), so
// for c = d . n > 0 it meets that triangle's plane at t = 1e-4 / c, 1e-4 tan(theta) from x, and the
// any-hit traversal stops there when that point lies inside the triangle (triangle.hpp:140-160, t in
// [0, tmax]): the light is occluded by the surface itself.  The device ray starts farther off the
// surface (origin_offset: 4 ulps, more than 1e-4 at kilometre coordinates), which moves a grazing
// ray's crossing away from the hit point, so the crossing is decided here, from the FP32 surface
// point and the reference's offset: inside when the tangential shift is shorter than the distance to
// the nearest edge.  The rays that cross the plane outside the triangle are traced, their own
// triangle included: the watertight test then gives a crossing at an edge to this triangle or to its
// neighbour, never to neither (skipping this triangle would let such rays through the edge).
__device__ __forceinline__ bool shadow_self_occluded(float3 dir, float dist, float3 flat_n, float clear) {
    const float c = dot3(dir, flat_n);
    if (!(c > 0.0f)) return false;
    const float shift = 1.01e-4f * sqrtf(fmaxf(0.0f, 1.0f - c * c)) / c;   // 1e-4 tan(theta), +1 %
    return shift < clear && 1e-4f < 0.5f * dist * c;                       // inside; t = 1e-4 / c < tmax
}

// Of the shadow rays of path p whose lights are in `cross` (rays toward the surface's plane), those
// that stop on the path's own triangle (shadow_self_occluded) are occluded now and dropped from the
// returned mask of rays to trace; the others are traced without skipping that triangle.
__device__ __noinline__ uint32_t mark_self_occluded(const Batch& B, uint32_t p, const RReq& R, uint32_t cross,
                                                    uint32_t keep) {
    const float4 nc = edge_clearance(B, p, R);
    for (uint32_t m = cross; m; m &= m - 1) {
        const uint32_t l = __ffs(m) - 1;
        const size_t k = (size_t)p * B.L + l;
        const float4 db = B.sray[2 * k + 1];   // direction and distance as written by shade_path
        if (shadow_self_occluded(f3(db.x, db.y, db.z), db.w, f3(nc.x, nc.y, nc.z), nc.w)) {
            B.occ[k] = 1;
            keep &= ~(1u << l);
        } else {
            B.sray[2 * k].w = __uint_as_float(CRT_MISS);
        }
    }
    return keep;
}

// One live path at bounce `bounce`: surface point, a shadow ray per light at p * L + l, and when the
// path continues its bounce ray.  Returns the lights whose shadow ray has to be traced (bits 0..15)
// and the octant of the bounce ray (bits 16..18).
__device__ __forceinline__ uint32_t shade_path(const Batch& B, int bounce, uint32_t p, uint32_t req, const THit& h,
                                               bool cont) {
    const RReq& R = B.rr[req];
    const uint32_t pixel = B.ppix[p], sample = B.psample[p];
    const SceneView sv = R.sv;
    const SurfacePoint sp = surface_point(sv, h);
    const EntityDev& E = sv.entities[sp.entity];
    const float3 col = f3(E.color[0], E.color[1], E.color[2]);
    const float3 x = sp.x - origin_offset(sp.x) * sp.flat_n;   // intersect_point - 1e-4 normal
    const uint32_t nl = R.n_lights;
    uint32_t cross = 0;   // lights whose shadow ray points into the plane of the triangle
    uint32_t oct = 0;    // octant of the bounce ray
    for (uint32_t l = 0; l < nl; ++l) {
        const LightDev& lt = B.lights[R.light_base + l];
        float3 lp = f3(lt.pos[0], lt.pos[1], lt.pos[2]);
        float inten;
        if (lt.type == 1) {   // AreaLight::sample_ray / get_intensity (area_light.hpp:54-72)
            float a, b;
            rng2(R.c, pixel, sample, (uint32_t)bounce, 2u + l, a, b);
            const float xc = lt.size[0] * a - lt.size[0] / 2, yc = lt.size[1] * b - lt.size[1] / 2;
            lp = f3(lt.R[0] * xc + lt.R[1] * yc, lt.R[3] * xc + lt.R[4] * yc, lt.R[6] * xc + lt.R[7] * yc) + lp;
            const float3 dd = x - lp;
            inten = lt.intensity / dot3(dd, dd);
        } else {              // PointLight (point_light.hpp:32-39)
            const float3 dd = x - lp;
            inten = fminf(lt.intensity / dot3(dd, dd), 10000.0f);
        }
        const float3 to = lp - x;
        const float dist = sqrtf(dot3(to, to));
        const float3 dir = to * (1.0f / dist);
        // ColoredLambertianMaterial::compute (material.hpp:100-103): colour * (-L . N), unclamped
        const float ldn = -dot3(dir, sp.shading_n);
        const float3 cb = col * ldn;
        B.contrib[(size_t)p * B.L + l] = make_float4(cb.x * inten, cb.y * inten, cb.z * inten, 0.f);
        B.occ[(size_t)p * B.L + l] = 0;
        if (dot3(dir, sp.flat_n) > 0.0f) cross |= 1u << l;   // checked below
        const size_t k = (size_t)p * B.L + l;
        B.sray[2 * k] = make_float4(x.x, x.y, x.z, __uint_as_float(h.slot));   // tmin 0; skip the origin triangle
        B.sray[2 * k + 1] = make_float4(dir.x, dir.y, dir.z, dist);
    }
    if (cont) {
        float r1, r2;
        rng2(R.c, pixel, sample, (uint32_t)bounce, 1u, r1, r2);
        const float3 nd = cosine_importance(sp.shading_n, r1, r2);
        B.ray[2ull * p] = make_float4(x.x, x.y, x.z, 0.f);
        B.ray[2ull * p + 1] = make_float4(nd.x, nd.y, nd.z, 3.402823466e38f);
        // the triangle the ray leaves is not tested, unless the ray points into its plane (a direction
        // sampled about a smooth-shading normal): the reference meets that triangle again there
        B.skip[p] = dot3(nd, sp.flat_n) > 0.0f ? CRT_MISS : h.slot;
        const float bc = 1.0f - r1;
        const float4 wt = path_weight(B, p, bounce);
        B.wgt[(bounce + 1) & 1][p] = make_float4(wt.x * bc, wt.y * bc, wt.z * bc, 0.f);
        oct = (__float_as_uint(nd.x) >> 31) | ((__float_as_uint(nd.y) >> 31) << 1) | ((__float_as_uint(nd.z) >> 31) << 2);
    }
    // shadow rays that stop on their own triangle (at every bounce): occluded now, not traced
    const uint32_t all = (1u << nl) - 1u;   // nl <= 16
    const uint32_t keep = cross ? mark_self_occluded(B, p, R, cross, all) : all;
    return keep | (oct << 16);
}

// 256-thread blocks (block_append2); the loop's trip count is uniform over a block.  The shadow queue
// receives the shadow rays still to trace after the shade, in path order within a block; rays that
// their own triangle stops (mark_self_occluded) are not queued, and the counting build (counters
// non-null) counts them among the rays resolved without a traversal (counters[3]).
__global__ void __launch_bounds__(256) k_shade(Batch B, int bounce, const uint32_t* __restrict__ q_in,
                                               uint32_t* __restrict__ q_out, bool any_cont,
                                               unsigned long long* __restrict__ counters) {
    const uint32_t n = bounce == 0 ? B.cur->n_paths : B.counts[0];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t p = 0, req = 0;
        bool live = false, cont = false;
        THit h;
        h.t = h.u = h.v = 0.f;
        h.slot = CRT_MISS;
        if (i < n) {
            p = bounce == 0 ? i : q_in[i];
            const float4 hv = B.hit[p];
            h.t = hv.x; h.u = hv.y; h.v = hv.z;
            h.slot = __float_as_uint(hv.w);
            if (h.slot != CRT_MISS) {
                req = B.preq[p];
                const RenderCtl& c = B.rr[req].c;
                live = bounce < c.num_bounces;
                cont = bounce < c.num_bounces - 1;
            }
        }
        const uint32_t sp = live ? shade_path(B, bounce, p, req, h, cont) : 0u;
        const uint32_t keep = sp & 0xFFFFu;
        if (counters) {   // uniform: a kernel argument
            const uint32_t resolved = live ? B.rr[req].n_lights - __popc(keep) : 0u;
            const uint32_t wsum = __reduce_add_sync(0xFFFFFFFFu, resolved);
            if ((threadIdx.x & 31) == 0 && wsum) atomicAdd(counters + 3, (unsigned long long)wsum);
        }
        const uint2 at = block_append2(&B.counts[2], __popc(keep), &B.counts[1], 0u);
        uint32_t e = at.x;
        for (uint32_t m = keep; m; m &= m - 1) B.sidx[e++] = make_uint2(p * B.L + (uint32_t)(__ffs(m) - 1), req);
        // bounce queue grouped by ray octant within the block: warps of the bounce trace take rays
        // with one near-to-far child order
        if (any_cont) {   // false at the wave's last bounce: no path continues
            const uint32_t qi = block_append_buckets8(&B.counts[1], cont ? (sp >> 16) & 7u : 8u);
            if (cont) q_out[qi] = p;
        }
    }
}

// ---------------------------------------------------------------- accumulate
// Light reaching path p's current vertex (unidirectional.hpp:62-80): the unoccluded contributions
// in light order, clamped to [0, 1] after the first bounce, times the path weight.  Shared by
// k_accum and the fused accumulate of k_update, with explicit roundings, so both give the same bits.
__device__ __forceinline__ float4 add_light(const Batch& B, uint32_t p, uint32_t n_lights, int bounce, float4 r) {
    float3 lr = f3(0.f, 0.f, 0.f);
    for (uint32_t l = 0; l < n_lights; ++l) {
        // both loads issued together (the contribution slot exists whether or not it was written)
        const uint8_t oc = B.occ[(size_t)p * B.L + l];
        const float4 cb = B.contrib[(size_t)p * B.L + l];
        if (!oc) lr = f3(__fadd_rn(lr.x, cb.x), __fadd_rn(lr.y, cb.y), __fadd_rn(lr.z, cb.z));
    }
    if (bounce >= 1) {   // unidirectional.hpp:74-78
        lr.x = fminf(fmaxf(lr.x, 0.f), 1.f);
        lr.y = fminf(fmaxf(lr.y, 0.f), 1.f);
        lr.z = fminf(fmaxf(lr.z, 0.f), 1.f);
    }
    const float4 wa = path_weight(B, p, bounce);
    return make_float4(__fmaf_rn(lr.x, wa.x, r.x), __fmaf_rn(lr.y, wa.y, r.y), __fmaf_rn(lr.z, wa.z, r.z), 0.f);
}

__global__ void k_accum(Batch B, int bounce, const uint32_t* __restrict__ q_in) {
    const uint32_t n = bounce == 0 ? B.cur->n_paths : B.counts[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = bounce == 0 ? i : q_in[i];
        const bool hit = __float_as_uint(B.hit[p].w) != CRT_MISS;
        const RReq& R = B.rr[B.preq[p]];
        if (bounce == 0) {   // every path of the wave: its radiance starts here
            const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
            B.rad[p] = hit && R.c.num_bounces > 0 ? add_light(B, p, R.n_lights, 0, zero) : zero;
        } else if (hit && bounce < R.c.num_bounces) {
            B.rad[p] = add_light(B, p, R.n_lights, bounce, B.rad[p]);
        }
    }
}

// ---------------------------------------------------------------- pixel update (do_render.hpp:84-114)
// Final RGBA float and clamp(v * 256, 0, 255) bytes of a pixel (do_render.hpp:118-134)
__device__ __forceinline__ void store_pixel(const RReq& R, uint32_t pixel, float4 m) {
    const float v[4] = {m.x, m.y, m.z, 1.0f};
    if (R.rad) R.rad[pixel] = make_float4(v[0], v[1], v[2], v[3]);
    if (R.rgba) {
        uint8_t qv[4];
        for (int k = 0; k < 4; ++k) qv[k] = (uint8_t)fminf(fmaxf(v[k] * 256.0f, 0.0f), 255.0f);
        R.rgba[pixel] = make_uchar4(qv[0], qv[1], qv[2], qv[3]);
    }
}

// ACC0: the wave's only bounce is bounce 0 and its light is added here instead of by k_accum.
// A request with a fixed sample count (fin_update) gets its outputs from its last slice here.
template <bool ACC0>
__global__ void __launch_bounds__(256, 5) k_update(Batch B) {
    const WaveDesc& w = *B.cur;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < w.n_update; u += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = w.n_slices;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (w.slices[mid].upd_base <= u) lo = mid;
            else hi = mid;
        }
        const Slice& S = w.slices[lo];
        const uint32_t a = u - S.upd_base;
        const RReq& R = B.rr[S.req];
        const uint32_t pixel = S.active ? S.active[a] : tile_slot_pixel(a, R.c.W, R.c.H);
        const size_t g = (size_t)R.pix_base + pixel;
        // a slice that starts at sample 0 holds the pixel's first samples: its state is still the
        // zeroed one (running mean, count and done flag), so it is not read
        const bool fresh = S.s0 == 0;
        if (!fresh && B.done[g]) continue;
        float4 m = fresh ? make_float4(0.f, 0.f, 0.f, 0.f) : B.pix[g];
        uint32_t t = fresh ? 0u : B.taken[g];
        for (uint32_t k = 0; k < S.ns; ++k) {
            const uint32_t sample = S.s0 + k + 1;   // 1-based as in the reference loop
            const size_t p = (size_t)S.path_base + (size_t)k * S.npix + a;
            float4 L;
            if (ACC0) {
                // the lights' flags and contributions are read with the hit flag, not after it (a missed
                // path's slots hold stale values, which are not used)
                const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                const bool hit = __float_as_uint(B.hit[p].w) != CRT_MISS;
                const float4 Lh = add_light(B, (uint32_t)p, R.n_lights, 0, zero);
                L = R.c.num_bounces > 0 && hit ? Lh : zero;
            } else {
                L = B.rad[p];
            }
            const float inv = 1.0f / (float)sample;
            const float dx = (L.x - m.x) * inv, dy = (L.y - m.y) * inv, dz = (L.z - m.z) * inv;
            m.x += dx; m.y += dy; m.z += dz;
            t = sample;
            if ((int)sample >= R.c.min_samples) {
                const float noise = sqrtf(dx * dx + dy * dy + dz * dz);
                if (noise < R.c.noise_threshold) {
                    B.done[g] = 1;
                    break;
                }
            }
        }
        B.pix[g] = m;
        B.taken[g] = t;
        if (R.fin_update && S.s0 + S.ns == (uint32_t)R.c.max_samples) store_pixel(R, pixel, m);
    }
}

// still-active pixels of an adaptive request, in the order of its previous pixel set (tile order
// at first), so that the camera rays of a warp stay close together
__global__ void k_compact(const uint32_t* __restrict__ active, uint32_t n_active, const uint8_t* __restrict__ done,
                          uint32_t pix_base, uint32_t W, uint32_t H, uint32_t* __restrict__ out,
                          uint32_t* __restrict__ count) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n_active; a += gridDim.x * blockDim.x) {
        const uint32_t pixel = active ? active[a] : tile_slot_pixel(a, W, H);
        if (!done[pix_base + pixel]) out[warp_append(count, 1u)] = pixel;
    }
}

__global__ void k_finalize(Batch B, uint32_t n_req, uint32_t n_total) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n_total; g += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_req;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (B.rr[mid].pix_base <= g) lo = mid;
            else hi = mid;
        }
        const RReq& R = B.rr[lo];
        if (R.fin_update) continue;   // stored by its last update
        store_pixel(R, g - R.pix_base, B.pix[g]);
    }
}

// finalize of one request (the serving engine completes requests one by one)
__global__ void k_finalize_one(Batch B, uint32_t slot) {
    const RReq& R = B.rr[slot];
    for (uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < R.npix; pixel += gridDim.x * blockDim.x)
        store_pixel(R, pixel, B.pix[(size_t)R.pix_base + pixel]);
}

__global__ void k_tan_table2(double* __restrict__ out, uint32_t nx, uint32_t ny, double hx, double hy) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx) out[i] = tan(-hx + (i + 0.5) * 2.0 * hx / nx);
    else if (i < nx + ny) out[i] = tan(-hy + ((i - nx) + 0.5) * 2.0 * hy / ny);
}

// Grid of a grid-stride kernel: at most one resident wave (SMs x the kernel's resident blocks per SM
// at this block size, from its register and shared-memory use), fewer blocks when n needs fewer.  A
// larger grid would run a partial second wave of blocks on a part of the GPU.
template <typename... Args>
uint32_t grid_for(crt_context* ctx, void (*kernel)(Args...), size_t n, int block = 256) {
    static std::mutex mu;
    static std::map<const void*, int> per_sm_of;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = per_sm_of.find((const void*)kernel);
        if (it != per_sm_of.end()) per_sm = it->second;
    }
    if (!per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            per_sm = 1;
        }
        std::lock_guard<std::mutex> lock(mu);
        per_sm_of[(const void*)kernel] = per_sm;
    }
    const size_t want = (n + block - 1) / block;
    return (uint32_t)std::max<size_t>(1, std::min<size_t>(want, (size_t)ctx->sm_count * per_sm));
}
inline uint32_t tiles_items(uint32_t W, uint32_t H) { return ((W + 7) / 8) * ((H + 3) / 4) * 32u; }

// ---------------------------------------------------------------- host side
// The stage sequence of one wave on the context stream.  Every launch reads the wave from B.cur
// (filled by k_wave_begin from B.descs[*B.wave_idx]), so the sequence can be captured once and
// replayed.  P: path capacity, NL: light stride, lidar_items: bound on the wave's LiDAR items.
// srp_items: bound on the wave's SRP items (crt_batch_mixed, serving); when non-zero the primary
// trace also traces the wave's SRP sun rays and srp_stages (launches of the SRP shade and specular
// segments) runs right after it.  srp_mask (when given): the SRP hit mask, zeroed before the primary
// trace.  With srp_stages reading the wave's range from the device descriptor (srp_wave_stages_dev)
// the sequence is the same for every wave and can be captured and replayed.
void launch_wave_kernels(crt_context* ctx, const Batch& B, size_t P, size_t NL, uint32_t lidar_items,
                         int max_bounces, uint32_t* qa, uint32_t* qb, uint32_t* tqueue, uint32_t srp_items = 0,
                         const std::function<void()>* srp_stages = nullptr, uint32_t* srp_mask = nullptr,
                         size_t srp_mask_len = 0) {
    cudaStream_t st = ctx->stream;
    const uint32_t g_shade = grid_for(ctx, k_shade, P), g_accum = grid_for(ctx, k_accum, P);
    const uint32_t g_update = max_bounces <= 1 ? grid_for(ctx, k_update<true>, P) : grid_for(ctx, k_update<false>, P);
    k_wave_begin<<<1, 128, 0, st>>>(B);
    check_launch(ctx, "k_wave_begin");
    if (srp_mask) CRT_CUDA(cudaMemsetAsync(srp_mask, 0, srp_mask_len, st));
    if (srp_items) {
        launch_trace<false>(ctx, SceneView{}, PrimaryJobT<true>{B},
                            (uint32_t)std::min<size_t>(P + lidar_items + srp_items, 0xFFFFFF00u), &B.cur->n_primary,
                            tqueue);
        if (srp_stages) (*srp_stages)();
    } else {
        launch_trace<false>(ctx, SceneView{}, PrimaryJobT<false>{B},
                            (uint32_t)std::min<size_t>(P + lidar_items, 0xFFFFFF00u), &B.cur->n_primary, tqueue);
    }
    const uint32_t* q_in = nullptr;
    uint32_t* q_out = qa;
    const bool fuse = max_bounces <= 1;   // k_update adds the light of the only bounce (if any)
    for (int b = 0; b < max_bounces; ++b) {
        k_shade<<<g_shade, 256, 0, st>>>(B, b, q_in, q_out, b < max_bounces - 1,
                                         ctx->counting ? ctx->d_counters : nullptr);
        check_launch(ctx, "k_shade");
        launch_trace<true>(ctx, SceneView{}, ShadowJob{B}, (uint32_t)std::min<size_t>(P * NL, 0xFFFFFF00u),
                           &B.counts[2], tqueue);
        if (!fuse) {
            k_accum<<<g_accum, 256, 0, st>>>(B, b, q_in);
            check_launch(ctx, "k_accum");
        }
        if (b < max_bounces - 1) {
            launch_trace<false>(ctx, SceneView{}, BounceJob{B, q_out}, (uint32_t)P, &B.counts[1], tqueue);
            k_queue_rotate<<<1, 1, 0, st>>>(B.counts);
            check_launch(ctx, "k_queue_rotate");
            q_in = q_out;
            q_out = (q_out == qa) ? qb : qa;
        }
    }
    if (fuse) k_update<true><<<g_update, 256, 0, st>>>(B);
    else k_update<false><<<g_update, 256, 0, st>>>(B);
    check_launch(ctx, "k_update");
    k_wave_end<<<1, 1, 0, st>>>(B);
    check_launch(ctx, "k_wave_end");
}

struct HostReq {
    const crt_request* src;
    bool adaptive;
    uint32_t next_sample;     // first sample not yet scheduled
    uint32_t total;           // max_samples
    uint32_t n_active;        // adaptive requests: current pixel-set size
    const uint32_t* active;   // adaptive requests: current pixel set (device)
    uint32_t* act_buf[2];
    int act_sel;
    uint32_t rr_index;
};

void check_request(const crt_request& q) {
    CRT_CHECK(q.scene, CRT_ERR_INVALID, "request without a scene");
    if (q.kind == CRT_REQUEST_RENDER) {
        CRT_CHECK(q.camera && q.params, CRT_ERR_INVALID, "render request needs a camera and parameters");
        CRT_CHECK(q.n_lights <= (uint32_t)MAX_LIGHTS, CRT_ERR_INVALID, "at most 16 lights per render");
        CRT_CHECK(!q.n_lights || q.lights, CRT_ERR_INVALID, "null light list");
        CRT_CHECK(q.rgba8 || q.radiance, CRT_ERR_INVALID, "render request without an output buffer");
        const double W = std::floor(q.camera->resolution[0]), H = std::floor(q.camera->resolution[1]);
        CRT_CHECK(W >= 1 && H >= 1 && W * H < (double)(1u << 28), CRT_ERR_INVALID, "bad camera resolution");
    } else if (q.kind == CRT_REQUEST_LIDAR) {
        CRT_CHECK(q.lidar && q.range, CRT_ERR_INVALID, "LiDAR request needs a beam grid and a range buffer");
        const crt_lidar_grid_desc& g = *q.lidar;
        CRT_CHECK(g.nx > 0 && g.ny > 0 && (uint64_t)g.nx * g.ny < (1ull << 28), CRT_ERR_INVALID, "bad beam grid");
        CRT_CHECK(g.half_angle_x >= 0 && g.half_angle_x < 1.5 && g.half_angle_y >= 0 && g.half_angle_y < 1.5,
                  CRT_ERR_INVALID, "half angles must lie in [0, 1.5) rad");
    } else {
        throw CrtError{CRT_ERR_INVALID, "unknown request kind"};
    }
}

// Outputs the kernels write in place: device memory, or mapped page-locked host memory (the last
// update or k_finalize and the LiDAR trace store each value once, so the stores cross the host link
// while the kernels run and no copy follows); other host memory is staged in device scratch and
// copied back.
bool direct_out(const void* p) { return is_device_ptr(p) || is_host_mapped(p); }

// srps: SRP requests of a mixed batch (crt_batch_mixed); their sun rays ride in the waves' primary
// traces after the LiDAR beams and camera paths, one request's item range per wave.
void run_batch(crt_context* ctx, const crt_request* reqs, size_t n, crt_batch_stats* stats,
               const crt_server_request* const* srps = nullptr, size_t n_srp = 0) {
    for (size_t i = 0; i < n; ++i) {
        check_request(reqs[i]);
        CRT_CHECK(reqs[i].scene->ctx && reqs[i].scene->ctx->device == ctx->device, CRT_ERR_INVALID,
                  "request scene lives on another device");
    }
    std::vector<SrpPlan> splans(n_srp);
    for (size_t j = 0; j < n_srp; ++j) {
        const crt_server_request& q = *srps[j];
        CRT_CHECK(q.base.scene && q.srp && (q.n_att == 0 || (q.quaternions && q.force && q.torque)), CRT_ERR_INVALID,
                  "incomplete SRP request");
        CRT_CHECK(q.base.scene->ctx && q.base.scene->ctx->device == ctx->device, CRT_ERR_INVALID,
                  "request scene lives on another device");
        srp_plan(q.base.scene, q.srp, q.quaternions, q.n_att, splans[j]);
    }
    if (!n && !n_srp) return;
    CRT_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;

    // ---- request tables
    std::vector<RReq> rr;
    std::vector<LReq> lr;
    std::vector<LightDev> lights;
    std::vector<HostReq> hreq;
    uint32_t pix_total = 0, lidar_items = 0, tan_total = 0, L = 1;
    size_t host_out_bytes = 0;
    for (size_t i = 0; i < n; ++i) {
        const crt_request& q = reqs[i];
        if (q.kind == CRT_REQUEST_RENDER) {
            RReq R;
            R.sv = scene_view(q.scene);
            R.cam = make_camera_basis(q.camera);
            const crt_render_params& p = *q.params;
            R.c = RenderCtl{R.cam.width, R.cam.height, p.min_samples, p.max_samples, (float)p.noise_threshold,
                            p.num_bounces, (uint32_t)p.seed, (uint32_t)(p.seed >> 32), p.request};
            R.light_base = (uint32_t)lights.size();
            R.n_lights = q.n_lights;
            for (uint32_t l = 0; l < q.n_lights; ++l) {
                LightDev d;
                d.type = q.lights[l].type;
                d.intensity = (float)q.lights[l].intensity;
                for (int k = 0; k < 3; ++k) d.pos[k] = (float)q.lights[l].position[k];
                for (int k = 0; k < 9; ++k) d.R[k] = (float)q.lights[l].rotation[k];
                d.size[0] = (float)q.lights[l].size[0];
                d.size[1] = (float)q.lights[l].size[1];
                lights.push_back(d);
            }
            L = std::max<uint32_t>(L, q.n_lights);
            R.npix = R.cam.width * R.cam.height;
            R.pix_base = pix_total;
            pix_total += R.npix;
            R.rgba = nullptr;
            R.rad = nullptr;
            if (q.rgba8 && !direct_out(q.rgba8)) host_out_bytes += (size_t)R.npix * 4;
            if (q.radiance && !direct_out(q.radiance)) host_out_bytes += (size_t)R.npix * 16;
            HostReq h;
            h.src = &q;
            h.adaptive = p.noise_threshold > 0 && p.min_samples < p.max_samples;
            h.next_sample = 0;
            h.total = (uint32_t)std::max(0, p.max_samples);
            h.n_active = R.npix;
            h.active = nullptr;
            h.act_sel = 0;
            h.rr_index = (uint32_t)rr.size();
            // a fixed sample count: every pixel's last sample is in the request's last slice, whose
            // update stores the outputs
            R.fin_update = !h.adaptive && h.total > 0 ? 1u : 0u;
            hreq.push_back(h);
            rr.push_back(R);
        } else {
            CRT_CHECK(lr.size() < (size_t)MAX_LIDAR, CRT_ERR_INVALID, "at most 256 LiDAR requests per batch");
            const crt_lidar_grid_desc& g = *q.lidar;
            LReq Lq;
            Lq.sv = scene_view(q.scene);
            for (int k = 0; k < 3; ++k) Lq.o[k] = g.position[k];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Lq.rt[3 * a + b] = g.rotation[3 * b + a];
            Lq.zsign = g.z_positive ? 1.0 : -1.0;
            Lq.nx = g.nx;
            Lq.ny = g.ny;
            Lq.tan_base = tan_total;
            tan_total += g.nx + g.ny;
            Lq.item_base = lidar_items;
            lidar_items += tiles_items(g.nx, g.ny);
            Lq.range = nullptr;
            Lq.prim = nullptr;
            if (!direct_out(q.range)) host_out_bytes += (size_t)g.nx * g.ny * 8;
            if (q.prim && !direct_out(q.prim)) host_out_bytes += (size_t)g.nx * g.ny * 4;
            lr.push_back(Lq);
        }
    }

    // ---- wave plan for every render sample; adaptive requests schedule sample by sample later
    std::vector<WaveDesc> plan;
    const uint32_t cap = std::max<uint32_t>(ctx->wave_paths, 1u << 16);
    uint32_t max_paths = 0;
    int max_bounces = 0;
    for (const RReq& R : rr) max_bounces = std::max(max_bounces, R.c.num_bounces);
    auto new_wave = [&]() {
        WaveDesc w;
        std::memset(&w, 0, sizeof(w));
        plan.push_back(w);
    };
    auto add_slice = [&](WaveDesc& w, uint32_t req, uint32_t s0, uint32_t ns, uint32_t npix, const uint32_t* active) {
        Slice& S = w.slices[w.n_slices++];
        S.req = req;
        S.s0 = s0;
        S.ns = ns;
        S.npix = npix;
        S.path_base = w.n_paths;
        S.upd_base = w.n_update;
        S.active = active;
        w.n_paths += ns * npix;
        w.n_update += npix;
    };
    // non-adaptive samples, plus the non-adaptive prefix (samples < min_samples) of adaptive requests
    new_wave();
    for (HostReq& h : hreq) {
        const RReq& R = rr[h.rr_index];
        const uint32_t upto = h.adaptive ? (uint32_t)std::min<int>(std::max(R.c.min_samples, 1), (int)h.total) : h.total;
        while (h.next_sample < upto) {
            WaveDesc* w = &plan.back();
            const uint32_t room = w->n_paths < cap ? cap - w->n_paths : 0;
            uint32_t ns = std::min<uint32_t>(upto - h.next_sample, room / R.npix);
            if (ns == 0) {
                if (w->n_slices == 0) ns = 1;   // a single sample larger than the wave cap
                else { new_wave(); continue; }
            }
            if (w->n_slices == MAX_SLICES) { new_wave(); continue; }
            add_slice(*w, h.rr_index, h.next_sample, ns, R.npix, nullptr);
            h.next_sample += ns;
        }
    }
    if (plan.back().n_slices == 0 && plan.size() > 1) plan.pop_back();
    plan[0].n_lidar_items = lidar_items;
    plan[0].n_lreq = (uint32_t)lr.size();
    // SRP: each request's items cut into ranges of at most the wave size (whole attitudes, or a part of
    // one attitude); range k rides in wave k, with waves of SRP items only when there are more ranges
    struct SrpRange {
        size_t req;
        uint64_t i0, n;
    };
    std::vector<SrpRange> sranges;
    uint64_t srp_max = 0;
    uint32_t srp_nb = 0;
    const uint64_t srp_cap = std::max<uint64_t>((uint64_t)cap / SRP_BLOCK_ITEMS * SRP_BLOCK_ITEMS, SRP_BLOCK_ITEMS);
    for (size_t j = 0; j < n_srp; ++j) {
        const SrpPlan& SP = splans[j];
        for (uint64_t i0 = 0; i0 < SP.total;) {
            const uint64_t m = srp_wave_items(SP, srp_cap, i0);
            sranges.push_back(SrpRange{j, i0, m});
            srp_max = std::max(srp_max, m);
            i0 += m;
        }
        srp_nb = std::max(srp_nb, SP.nb);
    }
    while (plan.size() < sranges.size()) new_wave();
    for (size_t k = 0; k < sranges.size(); ++k) plan[k].n_srp_items = (uint32_t)sranges[k].n;
    for (WaveDesc& w : plan) {
        w.n_primary = w.n_lidar_items + w.n_paths + w.n_srp_items;
        max_paths = std::max(max_paths, w.n_paths);
    }
    bool any_adaptive = false;
    for (const HostReq& h : hreq)
        if (h.adaptive && h.next_sample < h.total) any_adaptive = true;
    if (any_adaptive) max_paths = std::max(max_paths, std::min<uint32_t>(cap, pix_total));
    for (const RReq& R : rr) max_paths = std::max(max_paths, std::min<uint32_t>(R.npix, std::max(cap, R.npix)));

    // ---- device memory (context scratch, reused across batches)
    const size_t P = std::max<uint32_t>(max_paths, 1), NL = L;
    const size_t WD = sizeof(WaveDesc);
    char* base = nullptr;
    Batch B;
    std::memset(&B, 0, sizeof(B));
    std::vector<SrpAtt*> s_att(n_srp);
    std::vector<double*> s_partial(n_srp), s_force(n_srp), s_torque(n_srp);
    char* s_state = nullptr;
    uint32_t* s_bq = nullptr;
    uint32_t* s_bcount = nullptr;
    auto carve = [&](char* b) {
        size_t off = 0;
        auto take = [&](size_t bytes) {
            off = (off + 255) & ~size_t(255);
            char* q = b ? b + off : nullptr;
            off += bytes;
            return q;
        };
        B.rr = (const RReq*)take(sizeof(RReq) * std::max<size_t>(rr.size(), 1));
        B.lr = (const LReq*)take(sizeof(LReq) * std::max<size_t>(lr.size(), 1));
        B.lights = (const LightDev*)take(sizeof(LightDev) * std::max<size_t>(lights.size(), 1));
        B.tan = (const double*)take(8 * std::max<uint32_t>(tan_total, 1));
        B.descs = (const WaveDesc*)take(WD * plan.size());
        B.cur = (WaveDesc*)take(WD);
        B.wave_idx = (uint32_t*)take(64);
        B.counts = (uint32_t*)take(64);
        B.ray = (float4*)take(P * 32);
        B.skip = (uint32_t*)take(P * 4);
        B.hit = (float4*)take(P * 16);
        B.wgt[0] = (float4*)take(P * 16);
        B.wgt[1] = (float4*)take(P * 16);
        B.rad = (float4*)take(P * 16);
        B.preq = (uint32_t*)take(P * 4);
        B.ppix = (uint32_t*)take(P * 4);
        B.psample = (uint32_t*)take(P * 4);
        B.contrib = (float4*)take(P * NL * 16);
        B.occ = (uint8_t*)take(P * NL);
        B.sray = (float4*)take(P * NL * 32);
        B.sidx = (uint2*)take(P * NL * 8);
        B.pix = (float4*)take((size_t)std::max<uint32_t>(pix_total, 1) * 16);
        B.taken = (uint32_t*)take((size_t)std::max<uint32_t>(pix_total, 1) * 4);
        B.done = (uint8_t*)take(std::max<uint32_t>(pix_total, 1));
        for (size_t j = 0; j < n_srp; ++j) {   // SRP: attitude table, partial sums, staged outputs
            const SrpPlan& SP = splans[j];
            const size_t na = std::max<size_t>(SP.n_att(), 1);
            s_att[j] = (SrpAtt*)take(sizeof(SrpAtt) * na);
            s_partial[j] = (double*)take(sizeof(double) * 6 * std::max<uint64_t>(SP.blocks_per_att, 1) * na);
            s_force[j] = is_device_ptr(srps[j]->force) ? srps[j]->force : (double*)take(24 * na);
            s_torque[j] = is_device_ptr(srps[j]->torque) ? srps[j]->torque : (double*)take(24 * na);
        }
        if (n_srp) {   // one wave's SRP item state, shared by the requests' ranges
            s_state = (char*)take(srp_state_bytes(std::max<uint64_t>(srp_max, 1), srp_nb));
            s_bq = srp_nb ? (uint32_t*)take(srp_max * 4 + 256) : nullptr;
            s_bcount = (uint32_t*)take(256);
        }
        return off;
    };
    const size_t total_bytes = carve(nullptr);
    base = (char*)ctx_scratch(ctx, SCR_WAVE2, total_bytes);
    carve(base);
    uint32_t* queues = (uint32_t*)ctx_scratch(ctx, SCR_WAVE3, P * 8 + 256);
    uint32_t* qa = queues;
    uint32_t* qb = queues + P;
    uint32_t* actbuf = any_adaptive ? (uint32_t*)ctx_scratch(ctx, SCR_WAVE4, (size_t)pix_total * 8 + 256) : nullptr;
    char* stage = host_out_bytes ? (char*)ctx_scratch(ctx, SCR_OUT2, host_out_bytes) : nullptr;
    size_t stage_off = 0;

    // outputs: caller device memory or staging
    size_t ri = 0, li = 0;
    for (size_t i = 0; i < n; ++i) {
        const crt_request& q = reqs[i];
        if (q.kind == CRT_REQUEST_RENDER) {
            RReq& R = rr[ri++];
            if (q.rgba8) {
                if (direct_out(q.rgba8)) R.rgba = (uchar4*)q.rgba8;
                else { R.rgba = (uchar4*)(stage + stage_off); stage_off += (size_t)R.npix * 4; }
            }
            if (q.radiance) {
                stage_off = (stage_off + 15) & ~size_t(15);
                if (direct_out(q.radiance)) R.rad = (float4*)q.radiance;
                else { R.rad = (float4*)(stage + stage_off); stage_off += (size_t)R.npix * 16; }
            }
        } else {
            LReq& Lq = lr[li++];
            stage_off = (stage_off + 15) & ~size_t(15);
            if (direct_out(q.range)) Lq.range = q.range;
            else { Lq.range = (double*)(stage + stage_off); stage_off += (size_t)Lq.nx * Lq.ny * 8; }
            if (q.prim) {
                if (direct_out(q.prim)) Lq.prim = q.prim;
                else { Lq.prim = (uint32_t*)(stage + stage_off); stage_off += (size_t)Lq.nx * Lq.ny * 4; }
            }
        }
    }
    if (host_out_bytes) CRT_CHECK(stage_off <= host_out_bytes + 64 * n, CRT_ERR_INVALID, "staging overflow");

    for (size_t k = 0; k < sranges.size(); ++k) {
        const SrpRange& R = sranges[k];
        crt_scene* sc = srps[R.req]->base.scene;
        plan[k].srp = srp_stage(scene_view(sc), srp_wave(splans[R.req], s_att[R.req], s_state, srp_max, R.i0, R.n, (int)srp_nb),
                                (uint32_t)R.n, splans[R.req], s_partial[R.req], (uint32_t)sc->n_tris);
    }

    // ---- uploads (pinned staging ring: no wait for the previous call's kernels)
    size_t srp_up = 0;
    for (const SrpPlan& SP : splans) srp_up += sizeof(SrpAtt) * SP.n_att() + 256;
    const size_t up_bytes = sizeof(RReq) * rr.size() + sizeof(LReq) * lr.size() + sizeof(LightDev) * lights.size() +
                            WD * plan.size() + srp_up + 1024;
    PinnedStaging staging(ctx, up_bytes);
    char* pin = staging.p;
    size_t po = 0;
    auto up = [&](const void* dst, const void* src, size_t bytes) {
        if (!bytes) return;
        std::memcpy(pin + po, src, bytes);
        CRT_CUDA(cudaMemcpyAsync((void*)dst, pin + po, bytes, cudaMemcpyHostToDevice, st));
        po += (bytes + 255) & ~size_t(255);
    };
    up(B.rr, rr.data(), sizeof(RReq) * rr.size());
    up(B.lr, lr.data(), sizeof(LReq) * lr.size());
    up(B.lights, lights.data(), sizeof(LightDev) * lights.size());
    up(B.descs, plan.data(), WD * plan.size());
    for (size_t j = 0; j < n_srp; ++j) up(s_att[j], splans[j].att.data(), sizeof(SrpAtt) * splans[j].n_att());
    staging.release();   // the adaptive loop below rewrites `pin` only after synchronising the stream
    CRT_CUDA(cudaMemsetAsync(B.wave_idx, 0, 4, st));
    if (pix_total) {
        // every pixel of a request that takes samples gets its mean and count from its first slice
        // (k_update); only requests without samples (max_samples 0) read the zeroed state
        bool unsampled = false;
        for (const HostReq& h : hreq) unsampled |= h.total == 0;
        if (unsampled) {
            CRT_CUDA(cudaMemsetAsync(B.pix, 0, (size_t)pix_total * 16, st));
            CRT_CUDA(cudaMemsetAsync(B.taken, 0, (size_t)pix_total * 4, st));
        }
        CRT_CUDA(cudaMemsetAsync(B.done, 0, pix_total, st));
    }
    for (size_t k = 0; k < lr.size(); ++k) {
        const crt_lidar_grid_desc& g = *([&]() {
            size_t c = 0;
            for (size_t i = 0; i < n; ++i)
                if (reqs[i].kind == CRT_REQUEST_LIDAR && c++ == k) return reqs[i].lidar;
            return (const crt_lidar_grid_desc*)nullptr;
        })();
        const uint32_t nt = g.nx + g.ny;
        k_tan_table2<<<(nt + 255) / 256, 256, 0, st>>>((double*)B.tan + lr[k].tan_base, g.nx, g.ny, g.half_angle_x,
                                                        g.half_angle_y);
        check_launch(ctx, "k_tan_table2");
    }
    B.L = (uint32_t)NL;

    // ---- one wave: every launch reads the wave from B.cur (graph-capturable)
    uint32_t* tqueue = (uint32_t*)ctx_scratch(ctx, SCR_QUEUE, 256);
    auto launch_wave = [&]() { launch_wave_kernels(ctx, B, P, NL, lidar_items, max_bounces, qa, qb, tqueue); };

    size_t waves_run = 0;
    const bool graph_ok = ctx->use_graphs && !ctx->counting && plan.size() > 1;
    const bool with_srp = n_srp && srp_max > 0;
    if (graph_ok) {
        // waves carrying SRP items run their SRP stages from the wave descriptor (B.cur->srp), for
        // every wave (no-ops in waves without SRP items): the sequence does not change between waves
        std::function<void()> srp_stages;
        uint32_t* srp_mask = nullptr;
        if (with_srp) {
            const SrpStage* d_stage = &B.cur->srp;
            srp_stages = [&, d_stage]() {
                srp_wave_stages_dev(ctx, d_stage, (uint32_t)srp_max, srp_nb, s_bq, s_bcount, tqueue);
            };
            srp_mask = (uint32_t*)(s_state + srp_mask_offset(srp_max, srp_nb));
        }
        // capture one wave, replay it for every wave of the plan; the graph and its executable are
        // destroyed on every exit (replays already enqueued still run)
        struct GraphHold {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            ~GraphHold() {
                if (ge) cudaGraphExecDestroy(ge);
                if (g) cudaGraphDestroy(g);
            }
        } gh;
        CRT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const uint64_t before = ctx->launches;
        try {
            if (with_srp)
                launch_wave_kernels(ctx, B, P, NL, lidar_items, max_bounces, qa, qb, tqueue, (uint32_t)srp_max,
                                    &srp_stages, srp_mask, srp_mask_bytes(srp_max));
            else
                launch_wave();
        } catch (...) {
            cudaStreamEndCapture(st, &gh.g);
            throw;
        }
        CRT_CUDA(cudaStreamEndCapture(st, &gh.g));
        const uint64_t per_wave = ctx->launches - before;
        CRT_CUDA(cudaGraphInstantiate(&gh.ge, gh.g, 0));
        ctx->launches = before;
        for (size_t w = 0; w < plan.size(); ++w) {
            CRT_CUDA(cudaGraphLaunch(gh.ge, st));
            ctx->launches += per_wave;
        }
        waves_run = plan.size();
    } else if (with_srp) {
        // waves with SRP items launched one by one: the SRP stages of the wave's range follow its
        // primary trace
        for (size_t w = 0; w < plan.size(); ++w) {
            std::function<void()> stages;
            if (w < sranges.size()) {
                const SrpRange& R = sranges[w];
                crt_scene* sc = srps[R.req]->base.scene;
                CRT_CUDA(cudaMemsetAsync(plan[w].srp.W.hitmask, 0, srp_mask_bytes(R.n), st));   // before the trace
                stages = [&, w, sc]() {
                    srp_wave_stages(ctx, scene_view(sc), plan[w].srp.W, (uint32_t)R.n, splans[R.req], s_partial[R.req],
                                    nullptr, (uint32_t)sc->n_tris, s_bq, s_bcount);
                };
            }
            launch_wave_kernels(ctx, B, P, NL, lidar_items, max_bounces, qa, qb, tqueue,
                                (uint32_t)std::max<uint64_t>(srp_max, 1), stages ? &stages : nullptr);
        }
        waves_run = plan.size();
    } else {
        for (size_t w = 0; w < plan.size(); ++w) launch_wave();
        waves_run = plan.size();
    }

    // ---- adaptive requests: one sample per wave over the still-active pixels
    if (any_adaptive) {
        uint32_t* acount = B.counts + 8;
        uint32_t offs = 0;
        for (HostReq& h : hreq) {
            if (!h.adaptive) continue;
            h.act_buf[0] = actbuf + offs;
            h.act_buf[1] = actbuf + offs + rr[h.rr_index].npix;
            offs += 2 * rr[h.rr_index].npix;
        }
        while (true) {
            // compact the pixel sets of adaptive requests that still have samples
            std::vector<HostReq*> live;
            for (HostReq& h : hreq)
                if (h.adaptive && h.next_sample < h.total && h.n_active > 0) live.push_back(&h);
            if (live.empty()) break;
            for (HostReq* h : live) {
                uint32_t* out = h->act_buf[h->act_sel];
                CRT_CUDA(cudaMemsetAsync(acount, 0, 4, st));
                const RReq& R = rr[h->rr_index];
                k_compact<<<grid_for(ctx, k_compact, h->n_active), 256, 0, st>>>(h->active, h->n_active, B.done, R.pix_base,
                                                                       R.c.W, R.c.H, out, acount);
                check_launch(ctx, "k_compact");
                uint32_t cnt = 0;
                CRT_CUDA(cudaMemcpyAsync(&cnt, acount, 4, cudaMemcpyDeviceToHost, st));
                CRT_CUDA(cudaStreamSynchronize(st));
                h->n_active = cnt;
                h->active = out;
                h->act_sel ^= 1;
            }
            WaveDesc w;
            std::memset(&w, 0, sizeof(w));
            for (HostReq* h : live) {
                if (!h->n_active || w.n_slices == MAX_SLICES) continue;
                add_slice(w, h->rr_index, h->next_sample, 1, h->n_active, h->active);
                h->next_sample += 1;
            }
            if (!w.n_slices) break;
            w.n_primary = w.n_paths;
            CRT_CHECK(w.n_paths <= P, CRT_ERR_INVALID, "adaptive wave exceeds the path buffers");
            std::memcpy(pin, &w, WD);
            CRT_CUDA(cudaMemcpyAsync((void*)B.descs, pin, WD, cudaMemcpyHostToDevice, st));
            CRT_CUDA(cudaMemsetAsync(B.wave_idx, 0, 4, st));
            launch_wave();
            ++waves_run;
            CRT_CUDA(cudaStreamSynchronize(st));   // the pinned descriptor is rewritten next round
        }
    }

    // ---- finalize (requests whose last update did not store their outputs) and copy host outputs
    bool any_finalize = false;
    for (const RReq& R : rr) any_finalize = any_finalize || !R.fin_update;
    if (pix_total && any_finalize) {
        k_finalize<<<grid_for(ctx, k_finalize, pix_total), 256, 0, st>>>(B, (uint32_t)rr.size(), pix_total);
        check_launch(ctx, "k_finalize");
    }
    ri = 0;
    li = 0;
    bool host_out = false;
    for (size_t i = 0; i < n; ++i) {
        const crt_request& q = reqs[i];
        if (q.kind == CRT_REQUEST_RENDER) {
            const RReq& R = rr[ri++];
            if (q.rgba8 && (void*)R.rgba != (void*)q.rgba8) out_finish(ctx, q.rgba8, R.rgba, (size_t)R.npix * 4);
            if (q.radiance && (void*)R.rad != (void*)q.radiance) out_finish(ctx, q.radiance, R.rad, (size_t)R.npix * 16);
            host_out = host_out || host_output(q.rgba8) || host_output(q.radiance);
        } else {
            const LReq& Lq = lr[li++];
            if ((void*)Lq.range != (void*)q.range) out_finish(ctx, q.range, Lq.range, (size_t)Lq.nx * Lq.ny * 8);
            if (q.prim && (void*)Lq.prim != (void*)q.prim) out_finish(ctx, q.prim, Lq.prim, (size_t)Lq.nx * Lq.ny * 4);
            host_out = host_out || host_output(q.range) || host_output(q.prim);
        }
    }
    for (size_t j = 0; j < n_srp; ++j) {   // per-attitude totals in a fixed order, as crt_srp
        const crt_server_request& q = *srps[j];
        srp_reduce(ctx, s_partial[j], splans[j], s_force[j], s_torque[j]);
        if (s_force[j] != q.force) { out_finish(ctx, q.force, s_force[j], q.n_att * 24); host_out = true; }
        if (s_torque[j] != q.torque) { out_finish(ctx, q.torque, s_torque[j], q.n_att * 24); host_out = true; }
    }
    if (stats) {
        stats->waves = waves_run;
        stats->render_paths = 0;
        for (const WaveDesc& w : plan) stats->render_paths += w.n_paths;
        stats->lidar_beams = 0;
        for (const LReq& Lq : lr) stats->lidar_beams += (uint64_t)Lq.nx * Lq.ny;
    }
    if (host_out) check_device_error(ctx, "crt_batch");
}

// ---------------------------------------------------------------- serving engine
// Continuous batching at wave granularity: requests join a lane's engine while others are on the
// GPU and leave it as soon as their last wave has run.  Per-request pixel state (running mean,
// sample count, done flag) lives in a unit arena (one unit per pixel), host-output staging,
// adaptive pixel sets and LiDAR tangent tables in a byte arena; both are first-fit allocators over
// fixed device buffers sized from the lane budget, so admission is by free memory.  Each step plans
// one wave shortest-remaining-work first (LiDAR scans first: one launch finishes them), runs the
// same stage kernels as crt_batch, finalizes the requests whose work is complete and synchronises.
// Random streams and per-pixel sample order are those of crt_render, so results do not depend on
// what else shares the waves.

class Ranges {   // first-fit allocator over [0, cap)
  public:
    void reset(size_t cap) {
        free_.clear();
        cap_ = cap;
        if (cap) free_[0] = cap;
    }
    size_t cap() const { return cap_; }
    bool alloc(size_t n, size_t& off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            off = it->first;
            const size_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[off + n] = rest;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n) {
        if (!n) return;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

  private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0;
};

constexpr uint32_t ENGINE_SLOTS = 1024;      // resident render requests per engine
constexpr size_t UNIT_BYTES = 16 + 4 + 1;    // pix, taken, done
inline size_t up256(size_t n) { return (n + 255) & ~size_t(255); }

struct EReq {
    uint64_t tag = 0, seq = 0;
    crt_request q;
    bool lidar = false, finished = false;
    uint32_t slot = 0, npix = 0, W = 0, H = 0;
    size_t unit_off = 0, units = 0, byte_off = 0, bytes = 0;
    bool adaptive = false;
    uint32_t next_sample = 0, upto = 0, total = 0, n_active = 0;
    const uint32_t* active = nullptr;
    uint32_t* act_buf[2] = {nullptr, nullptr};
    int act_sel = 0;
    int num_bounces = 0;
    uint32_t n_lights = 0, skipped = 0;
    uchar4* rgba = nullptr;
    float4* rad = nullptr;
    double* range = nullptr;
    uint32_t* prim = nullptr;
    double* tan = nullptr;
    // SRP query: its sun-ray items ride in the waves' primary traces, one range per wave
    bool srp = false;
    std::shared_ptr<SrpPlan> splan;
    uint64_t srp_next = 0;                // next item to put in a wave
    SrpAtt* d_att = nullptr;
    double* partial = nullptr;
    double* force = nullptr;              // device: the caller's memory or arena staging
    double* torque = nullptr;
    double* out_force = nullptr;          // the caller's buffers
    double* out_torque = nullptr;
    uint64_t remaining() const {
        if (srp) return splan ? splan->total - srp_next : 0;
        if (lidar) return 0;
        return (uint64_t)(total - next_sample) * (adaptive && next_sample >= upto ? n_active : npix);
    }
};

}  // namespace

struct WaveEngine {
    crt_context* ctx = nullptr;
    size_t budget = 0;
    uint32_t P = 0, NL = 0, want_P = 0, want_NL = 1;
    char* paths = nullptr;
    char* units_mem = nullptr;
    char* bytes_mem = nullptr;
    char* fixed = nullptr;           // request tables, wave descriptor, counters
    Ranges units, bytes;
    std::vector<uint32_t> free_slots;
    std::vector<EReq> res;
    uint64_t seq = 0;
    struct Up {
        void* dst;
        size_t off, n;
    };
    std::vector<char> up_data;
    std::vector<Up> ups;
    char* pinned[2] = {nullptr, nullptr};   // upload buffers, alternating between consecutive waves
    size_t pinned_bytes[2] = {0, 0};
    int parity = 0;
    // completion of the wave in flight: host outputs land in pinned staging (hout) by async copies
    // and reach the caller's memory when the wave's event has completed
    struct OutCopy {
        void* dst;
        size_t off, n;
    };
    struct Flight {
        bool active = false;
        cudaEvent_t ev = nullptr;
        int err_slot = 0;
        std::vector<uint64_t> tags;
        std::vector<OutCopy> copies;
    };
    Flight flights[2];
    int cur_flight = 0;
    char* hout = nullptr;                    // pinned host staging of outputs
    Ranges hout_r;
    uint32_t* err_pin = nullptr;             // pinned copies of the device error word, one per flight
    std::vector<uint64_t> failed;            // tags of a wave whose device check failed
    // fixed device tables
    RReq* d_rr = nullptr;
    LightDev* d_lights = nullptr;
    LReq* d_lr = nullptr;
    WaveDesc* d_desc = nullptr;
    WaveDesc* d_cur = nullptr;
    uint32_t* d_wave_idx = nullptr;
    uint32_t* d_counts = nullptr;
    uint32_t* d_acount = nullptr;
    uint32_t* d_tqueue = nullptr;
    // SRP items of one wave (allocated at the first SRP admission): state, continuation queue, counters
    uint64_t srp_cap = 0;
    char* srp_state = nullptr;
    uint32_t* srp_bq = nullptr;
    uint32_t* srp_bcount = nullptr;
    // executable graphs of one wave, per (bounce count, specular segments of the wave's SRP range, -1
    // without one), valid for the buffers they were captured with (their addresses are kernel
    // arguments): every launch of a wave reads the wave from d_cur, so one capture serves every wave
    // of the same shape
    struct WaveGraph {
        int bounces, srp_nb;
        const void *paths, *units, *bytes;
        cudaGraphExec_t exec;
        uint64_t launches;
    };
    std::vector<WaveGraph> graphs;

    float4* pix() const { return (float4*)units_mem; }
    uint32_t* taken() const { return (uint32_t*)(units_mem + up256(units.cap() * 16)); }
    uint8_t* done() const { return (uint8_t*)(units_mem + up256(units.cap() * 16) + up256(units.cap() * 4)); }
    static size_t path_bytes(size_t P, size_t NL) {
        return P * (32 + 4 + 16 * 5 + 12 + 8) + P * NL * (16 + 1 + 32 + 8) + 64 * 256;
    }
};

namespace {

void engine_alloc_units(WaveEngine* e, size_t cap) {
    CRT_CHECK(cap < (1ull << 32), CRT_ERR_OOM, "serving pixel arena limited to 2^32 pixels");
    if (e->units_mem) CRT_CUDA(cudaFree(e->units_mem));
    e->units_mem = nullptr;
    e->units.reset(0);
    const size_t b = up256(cap * 16) + up256(cap * 4) + up256(cap);
    CRT_CUDA(cudaMalloc(&e->units_mem, b));
    e->units.reset(cap);
}

void engine_alloc_bytes(WaveEngine* e, size_t cap) {
    CRT_CHECK(cap < (32ull << 30), CRT_ERR_OOM, "serving byte arena limited to 32 GiB");
    if (e->bytes_mem) CRT_CUDA(cudaFree(e->bytes_mem));
    e->bytes_mem = nullptr;
    e->bytes.reset(0);
    cap = up256(cap);
    CRT_CUDA(cudaMalloc(&e->bytes_mem, cap));
    e->bytes.reset(cap);
}

void engine_upload(WaveEngine* e, void* dst, const void* src, size_t n) {
    const size_t off = e->up_data.size();
    e->up_data.resize(off + up256(n));
    std::memcpy(e->up_data.data() + off, src, n);
    e->ups.push_back({dst, off, n});
}

// Copies the queued uploads through this wave's pinned buffer.  The buffer was last used two waves
// ago, and that wave has been drained (its event completed) before this one is planned.
void engine_flush_uploads(WaveEngine* e) {
    if (e->ups.empty()) return;
    const size_t need = e->up_data.size();
    const int b = e->parity;
    if (e->pinned_bytes[b] < need) {
        CRT_CUDA(cudaStreamSynchronize(e->ctx->stream));
        if (e->pinned[b]) CRT_CUDA(cudaFreeHost(e->pinned[b]));
        e->pinned[b] = nullptr;
        e->pinned_bytes[b] = 0;
        const size_t cap = (need + need / 2 + 4095) & ~size_t(4095);
        CRT_CUDA(cudaMallocHost(&e->pinned[b], cap));
        e->pinned_bytes[b] = cap;
    }
    std::memcpy(e->pinned[b], e->up_data.data(), need);
    for (const WaveEngine::Up& u : e->ups)
        CRT_CUDA(cudaMemcpyAsync(u.dst, e->pinned[b] + u.off, u.n, cudaMemcpyHostToDevice, e->ctx->stream));
    e->ups.clear();
    e->up_data.clear();
}

// Completes a wave in flight: waits for its event, checks its copy of the device error word, copies
// the staged host outputs to the callers' buffers and reports the finished requests.
// Host copies of a flight's staged outputs (its copies into the staging must have completed).
void engine_flush_copies(WaveEngine* e, WaveEngine::Flight& f) {
    for (const WaveEngine::OutCopy& c : f.copies) {
        std::memcpy(c.dst, e->hout + c.off, c.n);
        e->hout_r.release(c.off, up256(c.n));
    }
    f.copies.clear();
}

void engine_drain_flight(WaveEngine* e, WaveEngine::Flight& f, std::vector<uint64_t>& completed) {
    if (!f.active) return;
    f.active = false;
    CRT_CUDA(cudaEventSynchronize(f.ev));
    const uint32_t h = e->err_pin[f.err_slot];
    e->err_pin[f.err_slot] = 0;
    engine_flush_copies(e, f);
    std::vector<uint64_t> tags;
    tags.swap(f.tags);
    if (h) {
        e->failed.insert(e->failed.end(), tags.begin(), tags.end());
        std::string m = "serving wave: device check failed (";
        if (h & DEVERR_STACK_OVERFLOW) m += " traversal-stack-overflow";
        if (h & DEVERR_BAD_INDEX) m += " bad-index";
        m += " )";
        throw CrtError{CRT_ERR_DEVICE, m};
    }
    completed.insert(completed.end(), tags.begin(), tags.end());
}

void engine_drain_all(WaveEngine* e, std::vector<uint64_t>& completed) {
    // the older flight first
    WaveEngine::Flight& older = e->flights[e->cur_flight ^ 1];
    WaveEngine::Flight& newer = e->flights[e->cur_flight];
    engine_drain_flight(e, older, completed);
    engine_drain_flight(e, newer, completed);
}

// Stages a device output for the caller's host buffer: async copy into pinned staging now, host copy
// when the wave completes.  When the staging is full, the stream is synchronised and this flight's
// copies are done early; a single output larger than the staging grows it.
void engine_stage_out(WaveEngine* e, WaveEngine::Flight& f, void* dst, const void* src, size_t n) {
    if (!dst || !n) return;
    size_t off = 0;
    if (!e->hout_r.alloc(up256(n), off)) {
        // every copy issued so far has completed after the synchronise: move both flights' staged
        // outputs to their callers now (the flights still report their requests when drained)
        CRT_CUDA(cudaStreamSynchronize(e->ctx->stream));
        for (WaveEngine::Flight& g : e->flights) engine_flush_copies(e, g);
        if (!e->hout_r.alloc(up256(n), off)) {
            // nothing is staged in the buffer any more
            CRT_CUDA(cudaFreeHost(e->hout));
            e->hout = nullptr;
            const size_t cap = up256(n + n / 2);
            CRT_CUDA(cudaMallocHost(&e->hout, cap));
            e->hout_r.reset(cap);
            e->hout_r.alloc(up256(n), off);
        }
    }
    CRT_CUDA(cudaMemcpyAsync(e->hout + off, src, n, cudaMemcpyDeviceToHost, e->ctx->stream));
    f.copies.push_back({dst, off, n});
}

void engine_release(WaveEngine* e, EReq& r) {
    if (r.units) e->units.release(r.unit_off, r.units);
    if (r.bytes) e->bytes.release(r.byte_off, r.bytes);
    if (!r.lidar && !r.srp) e->free_slots.push_back(r.slot);
    r.units = r.bytes = 0;
}

}  // namespace

WaveEngine* engine_create(crt_context* ctx, size_t budget_bytes) {
    WaveEngine* e = new WaveEngine();
    e->ctx = ctx;
    e->budget = budget_bytes;
    try {
        CRT_CUDA(cudaSetDevice(ctx->device));
        const size_t fixed = up256(sizeof(RReq) * ENGINE_SLOTS) + up256(sizeof(LightDev) * ENGINE_SLOTS * MAX_LIGHTS) +
                             up256(sizeof(LReq) * MAX_LIDAR) + 2 * up256(sizeof(WaveDesc)) + 4 * 256 +
                             up256(4 * ENGINE_SLOTS);
        CRT_CUDA(cudaMalloc(&e->fixed, fixed));
        char* f = e->fixed;
        auto take = [&](size_t n) { char* q = f; f += up256(n); return q; };
        e->d_rr = (RReq*)take(sizeof(RReq) * ENGINE_SLOTS);
        e->d_lights = (LightDev*)take(sizeof(LightDev) * ENGINE_SLOTS * MAX_LIGHTS);
        e->d_lr = (LReq*)take(sizeof(LReq) * MAX_LIDAR);
        e->d_desc = (WaveDesc*)take(sizeof(WaveDesc));
        e->d_cur = (WaveDesc*)take(sizeof(WaveDesc));
        e->d_wave_idx = (uint32_t*)take(256);
        e->d_counts = (uint32_t*)take(256);
        e->d_tqueue = (uint32_t*)take(256);
        take(256);
        e->d_acount = (uint32_t*)take(4 * ENGINE_SLOTS);
        for (uint32_t s = ENGINE_SLOTS; s > 0; --s) e->free_slots.push_back(s - 1);
        CRT_CUDA(cudaMallocHost(&e->err_pin, 2 * sizeof(uint32_t)));
        e->err_pin[0] = e->err_pin[1] = 0;
        for (WaveEngine::Flight& f : e->flights) CRT_CUDA(cudaEventCreateWithFlags(&f.ev, cudaEventDisableTiming));
        const size_t hcap = std::min<size_t>(std::max<size_t>(budget_bytes / 8, 16u << 20), 512u << 20);
        CRT_CUDA(cudaMallocHost(&e->hout, hcap));
        e->hout_r.reset(hcap);
        // budget: path buffers for one wave, then pixel state and staging (2 : 3)
        e->want_P = std::max<uint32_t>(ctx->wave_paths, 1u << 16);
        // (a request larger than what is left runs alone, its arena growing to fit it)
        const size_t pb = WaveEngine::path_bytes(e->want_P, 1);
        const size_t rest = budget_bytes > pb ? budget_bytes - pb : 0;
        engine_alloc_units(e, std::max<size_t>(rest * 2 / 5 / UNIT_BYTES, 1));
        engine_alloc_bytes(e, std::max<size_t>(rest * 3 / 5, 256));
    } catch (...) {
        engine_destroy(e);
        throw;
    }
    return e;
}

void engine_destroy(WaveEngine* e) {
    if (!e) return;
    cudaSetDevice(e->ctx->device);
    cudaStreamSynchronize(e->ctx->stream);
    cudaFree(e->paths);
    cudaFree(e->units_mem);
    cudaFree(e->bytes_mem);
    cudaFree(e->fixed);
    cudaFree(e->srp_state);
    for (char* p : e->pinned)
        if (p) cudaFreeHost(p);
    if (e->hout) cudaFreeHost(e->hout);
    if (e->err_pin) cudaFreeHost(e->err_pin);
    for (WaveEngine::Flight& f : e->flights)
        if (f.ev) cudaEventDestroy(f.ev);
    for (WaveEngine::WaveGraph& g : e->graphs) cudaGraphExecDestroy(g.exec);
    delete e;
}

// Admits a request when its state fits the free arenas now (false: retry after requests finish).
// A request larger than an arena is admitted alone, the arena growing to fit it.
bool engine_admit(WaveEngine* e, const crt_request& q, uint64_t tag) {
    check_request(q);
    CRT_CHECK(q.scene->ctx && q.scene->ctx->device == e->ctx->device, CRT_ERR_INVALID,
              "request scene lives on another device");
    crt_context* ctx = e->ctx;
    cudaStream_t st = ctx->stream;
    EReq r;
    std::memset(&r.q, 0, sizeof(r.q));
    r.q = q;
    r.tag = tag;
    if (q.kind == CRT_REQUEST_RENDER) {
        if (e->free_slots.empty()) return false;
        const CamBasis cam = make_camera_basis(q.camera);
        const crt_render_params& p = *q.params;
        r.npix = cam.width * cam.height;
        r.W = cam.width;
        r.H = cam.height;
        const bool host_rgba = q.rgba8 && !is_device_ptr(q.rgba8);
        const bool host_rad = q.radiance && !is_device_ptr(q.radiance);
        r.adaptive = p.noise_threshold > 0 && p.min_samples < p.max_samples;
        r.total = (uint32_t)std::max(0, p.max_samples);
        r.upto = r.adaptive ? (uint32_t)std::min<int>(std::max(p.min_samples, 1), (int)r.total) : r.total;
        r.n_active = r.npix;
        r.num_bounces = p.num_bounces;
        r.n_lights = q.n_lights;
        const size_t b_rgba = host_rgba ? up256((size_t)r.npix * 4) : 0;
        const size_t b_rad = host_rad ? up256((size_t)r.npix * 16) : 0;
        const size_t b_act = r.adaptive ? 2 * up256((size_t)r.npix * 4) : 0;
        r.units = r.npix;
        r.bytes = b_rgba + b_rad + b_act;
        const bool alone = e->res.empty();
        if (alone && (r.units > e->units.cap() || r.bytes > e->bytes.cap()))
            CRT_CUDA(cudaStreamSynchronize(st));   // a completed wave's copies may still be in flight
        if (r.units > e->units.cap() && alone) engine_alloc_units(e, r.units + r.units / 4);
        if (r.bytes > e->bytes.cap() && alone) engine_alloc_bytes(e, r.bytes + r.bytes / 4);
        if (!e->units.alloc(r.units, r.unit_off)) return false;
        if (r.bytes && !e->bytes.alloc(r.bytes, r.byte_off)) {
            e->units.release(r.unit_off, r.units);
            return false;
        }
        r.slot = e->free_slots.back();
        e->free_slots.pop_back();
        char* b = e->bytes_mem + r.byte_off;
        r.rgba = q.rgba8 ? (host_rgba ? (uchar4*)b : (uchar4*)q.rgba8) : nullptr;
        b += b_rgba;
        r.rad = q.radiance ? (host_rad ? (float4*)b : (float4*)q.radiance) : nullptr;
        b += b_rad;
        if (r.adaptive) {
            r.act_buf[0] = (uint32_t*)b;
            r.act_buf[1] = (uint32_t*)(b + up256((size_t)r.npix * 4));
        }
        RReq R;
        std::memset(&R, 0, sizeof(R));
        R.sv = scene_view(q.scene);
        R.cam = cam;
        R.c = RenderCtl{cam.width, cam.height, p.min_samples, p.max_samples, (float)p.noise_threshold, p.num_bounces,
                        (uint32_t)p.seed, (uint32_t)(p.seed >> 32), p.request};
        R.light_base = r.slot * MAX_LIGHTS;
        R.n_lights = q.n_lights;
        R.pix_base = (uint32_t)r.unit_off;
        R.npix = r.npix;
        R.rgba = r.rgba;
        R.rad = r.rad;
        LightDev lights[MAX_LIGHTS];
        for (uint32_t l = 0; l < q.n_lights; ++l) {
            LightDev& d = lights[l];
            d.type = q.lights[l].type;
            d.intensity = (float)q.lights[l].intensity;
            for (int k = 0; k < 3; ++k) d.pos[k] = (float)q.lights[l].position[k];
            for (int k = 0; k < 9; ++k) d.R[k] = (float)q.lights[l].rotation[k];
            d.size[0] = (float)q.lights[l].size[0];
            d.size[1] = (float)q.lights[l].size[1];
        }
        engine_upload(e, e->d_rr + r.slot, &R, sizeof(R));
        if (q.n_lights) engine_upload(e, e->d_lights + R.light_base, lights, sizeof(LightDev) * q.n_lights);
        if (r.total == 0) {   // otherwise the first slice writes the mean and count (k_update)
            CRT_CUDA(cudaMemsetAsync(e->pix() + r.unit_off, 0, (size_t)r.npix * 16, st));
            CRT_CUDA(cudaMemsetAsync(e->taken() + r.unit_off, 0, (size_t)r.npix * 4, st));
        }
        CRT_CUDA(cudaMemsetAsync(e->done() + r.unit_off, 0, r.npix, st));
        e->want_P = std::max(e->want_P, r.npix);
        e->want_NL = std::max(e->want_NL, std::max<uint32_t>(q.n_lights, 1));
    } else {
        r.lidar = true;
        const crt_lidar_grid_desc& g = *q.lidar;
        const size_t n = (size_t)g.nx * g.ny;
        const bool host_range = !is_device_ptr(q.range);
        const bool host_prim = q.prim && !is_device_ptr(q.prim);
        const size_t b_tan = up256(8 * ((size_t)g.nx + g.ny));
        const size_t b_range = host_range ? up256(n * 8) : 0;
        const size_t b_prim = host_prim ? up256(n * 4) : 0;
        r.bytes = b_tan + b_range + b_prim;
        if (r.bytes > e->bytes.cap() && e->res.empty()) {
            CRT_CUDA(cudaStreamSynchronize(st));
            engine_alloc_bytes(e, r.bytes + r.bytes / 4);
        }
        if (!e->bytes.alloc(r.bytes, r.byte_off)) return false;
        char* b = e->bytes_mem + r.byte_off;
        r.tan = (double*)b;
        b += b_tan;
        r.range = host_range ? (double*)b : q.range;
        b += b_range;
        r.prim = q.prim ? (host_prim ? (uint32_t*)b : q.prim) : nullptr;
        const uint32_t nt = g.nx + g.ny;
        k_tan_table2<<<(nt + 255) / 256, 256, 0, st>>>(r.tan, g.nx, g.ny, g.half_angle_x, g.half_angle_y);
        check_launch(ctx, "k_tan_table2");
    }
    r.seq = e->seq++;
    e->res.push_back(r);
    return true;
}

// Admits an SRP query when its attitude table, partial sums and output staging fit the byte arena; its
// sun-ray items then ride in the waves' primary traces, one range of at most srp_cap items per wave
// (earliest admitted query first).  The SRP wave state (srp_cap items, 53 bytes each) is allocated at
// the engine's first SRP admission.
bool engine_admit_srp(WaveEngine* e, crt_scene* scene, const crt_srp_desc& desc, const double* quats, size_t n_att,
                      double* force, double* torque, uint64_t tag) {
    CRT_CHECK(scene && scene->ctx && scene->ctx->device == e->ctx->device, CRT_ERR_INVALID,
              "request scene lives on another device");
    CRT_CHECK(n_att == 0 || (quats && force && torque), CRT_ERR_INVALID, "incomplete SRP request");
    cudaStream_t st = e->ctx->stream;
    auto plan = std::make_shared<SrpPlan>();
    srp_plan(scene, &desc, quats, n_att, *plan);
    if (!e->srp_state) {
        const uint64_t cap = std::max<uint64_t>((uint64_t)e->want_P / SRP_BLOCK_ITEMS * SRP_BLOCK_ITEMS, SRP_BLOCK_ITEMS);
        const size_t b_state = up256(srp_state_bytes(cap, 1)), b_q = up256(cap * 4);
        CRT_CUDA(cudaMalloc(&e->srp_state, b_state + b_q + 256));
        e->srp_cap = cap;
        e->srp_bq = (uint32_t*)(e->srp_state + b_state);
        e->srp_bcount = (uint32_t*)(e->srp_state + b_state + b_q);
    }
    EReq r;
    std::memset(&r.q, 0, sizeof(r.q));
    r.q.kind = CRT_REQUEST_SRP;
    r.q.scene = scene;
    r.tag = tag;
    r.srp = true;
    r.splan = plan;
    const size_t na = std::max<size_t>(n_att, 1);
    const bool host_f = !is_device_ptr(force), host_t = !is_device_ptr(torque);
    const size_t b_att = up256(sizeof(SrpAtt) * na);
    const size_t b_part = up256(sizeof(double) * 6 * std::max<uint64_t>(plan->blocks_per_att, 1) * na);
    const size_t b_f = host_f ? up256(24 * na) : 0, b_t = host_t ? up256(24 * na) : 0;
    r.bytes = b_att + b_part + b_f + b_t;
    if (r.bytes > e->bytes.cap() && e->res.empty()) {
        CRT_CUDA(cudaStreamSynchronize(st));   // a completed wave's copies may still be in flight
        engine_alloc_bytes(e, r.bytes + r.bytes / 4);
    }
    if (!e->bytes.alloc(r.bytes, r.byte_off)) return false;
    char* b = e->bytes_mem + r.byte_off;
    r.d_att = (SrpAtt*)b;
    b += b_att;
    r.partial = (double*)b;
    b += b_part;
    r.force = host_f ? (double*)b : force;
    b += b_f;
    r.torque = host_t ? (double*)b : torque;
    r.out_force = force;
    r.out_torque = torque;
    if (n_att) engine_upload(e, r.d_att, plan->att.data(), sizeof(SrpAtt) * n_att);
    r.finished = plan->total == 0;
    r.seq = e->seq++;
    e->res.push_back(r);
    return true;
}

// Drops every resident request and the waves in flight (after a failed step); returns their tags.
void engine_abort(WaveEngine* e, std::vector<uint64_t>& dropped) {
    cudaStreamSynchronize(e->ctx->stream);
    cudaGetLastError();
    for (EReq& r : e->res) {
        engine_release(e, r);
        dropped.push_back(r.tag);
    }
    e->res.clear();
    for (WaveEngine::Flight& f : e->flights) {
        for (const WaveEngine::OutCopy& c : f.copies) e->hout_r.release(c.off, up256(c.n));
        f.copies.clear();
        dropped.insert(dropped.end(), f.tags.begin(), f.tags.end());
        f.tags.clear();
        f.active = false;
    }
    dropped.insert(dropped.end(), e->failed.begin(), e->failed.end());
    e->failed.clear();
    e->err_pin[0] = e->err_pin[1] = 0;
    cudaMemsetAsync(e->ctx->d_error, 0, sizeof(uint32_t), e->ctx->stream);
    e->ups.clear();
    e->up_data.clear();
}

// Runs one wave over the resident requests.  The wave is launched, then the previous wave (which ran
// while this one was planned) is completed, so the GPU does not wait for the host between waves;
// the tags of the requests completed by that earlier wave (and by this one, when nothing is left to
// run) are appended to `completed`.
void engine_step(WaveEngine* e, std::vector<uint64_t>& completed) {
    crt_context* ctx = e->ctx;
    cudaStream_t st = ctx->stream;
    CRT_CUDA(cudaSetDevice(ctx->device));
    if (e->res.empty()) {
        engine_drain_all(e, completed);
        return;
    }
    const int slot = e->cur_flight ^ 1;   // flight slot and upload buffer of the wave two steps back
    WaveEngine::Flight& f = e->flights[slot];
    engine_drain_flight(e, f, completed);   // normally drained already at the end of the last step
    e->parity = slot;
    // path buffers (wave-local state only; resizing waits for the wave in flight)
    if (e->want_P > e->P || e->want_NL > e->NL) {
        engine_drain_all(e, completed);
        if (e->paths) CRT_CUDA(cudaFree(e->paths));
        e->paths = nullptr;
        e->P = e->NL = 0;
        CRT_CUDA(cudaMalloc(&e->paths, WaveEngine::path_bytes(e->want_P, e->want_NL)));
        e->P = e->want_P;
        e->NL = e->want_NL;
    }
    const size_t P = e->P, NL = e->NL;
    Batch B;
    std::memset(&B, 0, sizeof(B));
    {
        char* b = e->paths;
        auto take = [&](size_t n) { char* q = b; b += up256(n); return q; };
        B.ray = (float4*)take(P * 32);
        B.skip = (uint32_t*)take(P * 4);
        B.hit = (float4*)take(P * 16);
        B.wgt[0] = (float4*)take(P * 16);
        B.wgt[1] = (float4*)take(P * 16);
        B.rad = (float4*)take(P * 16);
        B.preq = (uint32_t*)take(P * 4);
        B.ppix = (uint32_t*)take(P * 4);
        B.psample = (uint32_t*)take(P * 4);
        B.contrib = (float4*)take(P * NL * 16);
        B.occ = (uint8_t*)take(P * NL);
        B.sray = (float4*)take(P * NL * 32);
        B.sidx = (uint2*)take(P * NL * 8);
    }
    // the two path queues follow the path buffers (path_bytes reserves 8 bytes per path for them)
    uint32_t* qa = (uint32_t*)((char*)B.sidx + up256(P * NL * 8));
    uint32_t* qb = qa + P;
    B.rr = e->d_rr;
    B.lr = e->d_lr;
    B.lights = e->d_lights;
    B.tan = (const double*)e->bytes_mem;
    B.descs = e->d_desc;
    B.cur = e->d_cur;
    B.wave_idx = e->d_wave_idx;
    B.counts = e->d_counts;
    B.L = (uint32_t)NL;
    B.pix = e->pix();
    B.taken = e->taken();
    B.done = e->done();
    for (EReq& r : e->res)
        if (!r.lidar && !r.srp && r.next_sample >= r.total && (!r.adaptive || r.next_sample >= r.upto))
            r.finished = true;

    // adaptive requests past their fixed prefix: compact the still-active pixels (reads counts back,
    // so the wave in flight is completed first)
    std::vector<EReq*> compacting;
    for (EReq& r : e->res)
        if (!r.lidar && !r.srp && r.adaptive && r.next_sample >= r.upto && r.next_sample < r.total && r.n_active > 0)
            compacting.push_back(&r);
    if (!compacting.empty()) {
        engine_drain_all(e, completed);
        CRT_CUDA(cudaMemsetAsync(e->d_acount, 0, 4 * compacting.size(), st));
        for (size_t k = 0; k < compacting.size(); ++k) {
            EReq& r = *compacting[k];
            k_compact<<<grid_for(ctx, k_compact, r.n_active), 256, 0, st>>>(r.active, r.n_active, B.done, (uint32_t)r.unit_off,
                                                                 r.W, r.H, r.act_buf[r.act_sel], e->d_acount + k);
            check_launch(ctx, "k_compact");
        }
        std::vector<uint32_t> cnt(compacting.size());
        CRT_CUDA(cudaMemcpyAsync(cnt.data(), e->d_acount, 4 * cnt.size(), cudaMemcpyDeviceToHost, st));
        CRT_CUDA(cudaStreamSynchronize(st));
        for (size_t k = 0; k < compacting.size(); ++k) {
            EReq& r = *compacting[k];
            r.n_active = cnt[k];
            r.active = r.act_buf[r.act_sel];
            r.act_sel ^= 1;
            if (r.n_active == 0) r.finished = true;
        }
    }

    // plan one wave: LiDAR scans, then renders by least remaining work
    WaveDesc w;
    std::memset(&w, 0, sizeof(w));
    std::vector<LReq> lreqs;
    std::vector<EReq*> wave_lidar;
    uint32_t lidar_items = 0;
    for (EReq& r : e->res) {
        if (!r.lidar || lreqs.size() == (size_t)MAX_LIDAR) continue;
        const crt_lidar_grid_desc& g = *r.q.lidar;
        LReq L;
        std::memset(&L, 0, sizeof(L));
        L.sv = scene_view(r.q.scene);
        for (int k = 0; k < 3; ++k) L.o[k] = g.position[k];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) L.rt[3 * a + b] = g.rotation[3 * b + a];
        L.zsign = g.z_positive ? 1.0 : -1.0;
        L.nx = g.nx;
        L.ny = g.ny;
        L.tan_base = (uint32_t)(r.byte_off / 8);   // byte arena < 32 GiB (checked at creation)
        L.item_base = lidar_items;
        L.range = r.range;
        L.prim = r.prim;
        const uint32_t items = tiles_items(g.nx, g.ny);
        if ((uint64_t)lidar_items + items > 0xF0000000ull) break;
        lidar_items += items;
        lreqs.push_back(L);
        wave_lidar.push_back(&r);
    }
    w.n_lidar_items = lidar_items;
    w.n_lreq = (uint32_t)lreqs.size();
    std::vector<EReq*> order;
    for (EReq& r : e->res)
        if (!r.lidar && !r.srp && !r.finished && r.next_sample < r.total) order.push_back(&r);
    // least remaining work first; a request passed over for 4 waves goes first (no starvation)
    std::stable_sort(order.begin(), order.end(), [](const EReq* a, const EReq* b) {
        const bool sa = a->skipped >= 4, sb = b->skipped >= 4;
        if (sa != sb) return sa;
        if (sa) return a->seq < b->seq;
        const uint64_t ra = a->remaining(), rb = b->remaining();
        return ra != rb ? ra < rb : a->seq < b->seq;
    });
    int max_bounces = 0;
    for (EReq* rp : order) {
        EReq& r = *rp;
        if (w.n_slices == MAX_SLICES) break;
        const uint32_t room = (uint32_t)(P - w.n_paths);
        Slice& S = w.slices[w.n_slices];
        if (r.next_sample < r.upto) {
            const uint32_t ns = std::min<uint32_t>(r.upto - r.next_sample, room / r.npix);
            if (ns == 0) {
                ++r.skipped;
                continue;
            }
            S.req = r.slot;
            S.s0 = r.next_sample;
            S.ns = ns;
            S.npix = r.npix;
            S.active = nullptr;
        } else {
            if (r.n_active > room) {
                ++r.skipped;
                continue;
            }
            S.req = r.slot;
            S.s0 = r.next_sample;
            S.ns = 1;
            S.npix = r.n_active;
            S.active = r.active;
        }
        S.path_base = w.n_paths;
        S.upd_base = w.n_update;
        w.n_paths += S.ns * S.npix;
        w.n_update += S.npix;
        w.n_slices++;
        r.next_sample += S.ns;
        r.skipped = 0;
        max_bounces = std::max(max_bounces, r.num_bounces);
        if (r.next_sample >= r.total) r.finished = true;
    }
    // one SRP range per wave, from the earliest admitted query with items left
    EReq* sq = nullptr;
    for (EReq& r : e->res)
        if (r.srp && !r.finished && r.srp_next < r.splan->total && (!sq || r.seq < sq->seq)) sq = &r;
    uint64_t srp_n = 0;
    if (sq) {
        const SrpPlan& SP = *sq->splan;
        srp_n = srp_wave_items(SP, e->srp_cap, sq->srp_next);
        w.n_srp_items = (uint32_t)srp_n;
        // state laid out for specular segments (as allocated) whatever the request, so that the hit
        // mask sits at one address for every wave
        w.srp = srp_stage(scene_view(sq->q.scene),
                          srp_wave(SP, sq->d_att, e->srp_state, e->srp_cap, sq->srp_next, srp_n, 1),
                          (uint32_t)srp_n, SP, sq->partial, (uint32_t)sq->q.scene->n_tris);
        sq->srp_next += srp_n;
    }
    w.n_primary = w.n_lidar_items + w.n_paths + w.n_srp_items;

    // run it
    // launch
    const bool any_work = w.n_primary > 0;
    if (any_work) {
        if (lreqs.size()) engine_upload(e, e->d_lr, lreqs.data(), sizeof(LReq) * lreqs.size());
        engine_upload(e, e->d_desc, &w, sizeof(WaveDesc));
    }
    engine_flush_uploads(e);
    const bool graph = any_work && ctx->use_graphs && !ctx->counting;
    if (graph) {
        CRT_CUDA(cudaMemsetAsync(e->d_wave_idx, 0, 4, st));
        const int srp_nb = sq ? (int)sq->splan->nb : -1;
        WaveEngine::WaveGraph* g = nullptr;
        for (size_t k = 0; k < e->graphs.size();) {
            WaveEngine::WaveGraph& c = e->graphs[k];
            if (c.paths != e->paths || c.units != e->units_mem || c.bytes != e->bytes_mem) {   // stale
                cudaGraphExecDestroy(c.exec);
                e->graphs.erase(e->graphs.begin() + (long)k);
                continue;
            }
            if (c.bounces == max_bounces && c.srp_nb == srp_nb) g = &c;
            ++k;
        }
        if (!g) {
            // capture the wave's launches once for this shape: the primary trace's item bound is the
            // largest any wave can have (its grid is the persistent one), SRP stages read the range
            // from d_cur and launch srp_nb segments over the wave capacity
            std::function<void()> stages;
            uint32_t* mask = nullptr;
            if (srp_nb >= 0) {
                const SrpStage* d_stage = &e->d_cur->srp;
                stages = [&, d_stage]() {
                    srp_wave_stages_dev(ctx, d_stage, (uint32_t)e->srp_cap, (uint32_t)srp_nb, e->srp_bq,
                                        e->srp_bcount, e->d_tqueue);
                };
                mask = (uint32_t*)(e->srp_state + srp_mask_offset(e->srp_cap, 1));
            }
            cudaGraph_t cg = nullptr;
            cudaGraphExec_t ge = nullptr;
            CRT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const uint64_t before = ctx->launches;
            try {
                launch_wave_kernels(ctx, B, P, NL, 0xF0000000u, max_bounces, qa, qb, e->d_tqueue,
                                    srp_nb >= 0 ? (uint32_t)e->srp_cap : 0u, srp_nb >= 0 ? &stages : nullptr, mask,
                                    srp_nb >= 0 ? srp_mask_bytes(e->srp_cap) : 0);
            } catch (...) {
                cudaStreamEndCapture(st, &cg);
                if (cg) cudaGraphDestroy(cg);
                throw;
            }
            CRT_CUDA(cudaStreamEndCapture(st, &cg));
            const cudaError_t ie = cudaGraphInstantiate(&ge, cg, 0);
            cudaGraphDestroy(cg);
            CRT_CUDA(ie);
            e->graphs.push_back(WaveEngine::WaveGraph{max_bounces, srp_nb, e->paths, e->units_mem, e->bytes_mem, ge,
                                                      ctx->launches - before});
            ctx->launches = before;
            g = &e->graphs.back();
        }
        CRT_CUDA(cudaGraphLaunch(g->exec, st));
        ctx->launches += g->launches;
    } else if (any_work) {
        CRT_CUDA(cudaMemsetAsync(e->d_wave_idx, 0, 4, st));
        std::function<void()> stages;
        if (sq) {
            const SrpWave W = w.srp.W;
            CRT_CUDA(cudaMemsetAsync(W.hitmask, 0, srp_mask_bytes(srp_n), st));   // before the trace
            stages = [&, W]() {
                srp_wave_stages(ctx, scene_view(sq->q.scene), W, (uint32_t)srp_n, *sq->splan, sq->partial, nullptr,
                                (uint32_t)sq->q.scene->n_tris, e->srp_bq, e->srp_bcount);
            };
        }
        launch_wave_kernels(ctx, B, P, NL, lidar_items, max_bounces, qa, qb, e->d_tqueue,
                            sq ? (uint32_t)e->srp_cap : 0u, sq ? &stages : nullptr);
    }
    // an SRP query whose last range ran in this wave: per-attitude totals, outputs staged
    if (sq && sq->srp_next >= sq->splan->total) {
        const size_t na = sq->splan->n_att();
        srp_reduce(ctx, sq->partial, *sq->splan, sq->force, sq->torque);
        if (sq->force != sq->out_force) engine_stage_out(e, f, sq->out_force, sq->force, na * 24);
        if (sq->torque != sq->out_torque) engine_stage_out(e, f, sq->out_torque, sq->torque, na * 24);
        sq->finished = true;
    }
    // completions of this wave: finalize, stage host outputs, release device state (later work on
    // the stream reuses it only after these copies)
    for (EReq* r : wave_lidar) {
        const crt_lidar_grid_desc& g = *r->q.lidar;
        const size_t n = (size_t)g.nx * g.ny;
        if ((void*)r->range != (void*)r->q.range) engine_stage_out(e, f, r->q.range, r->range, n * 8);
        if (r->q.prim && (void*)r->prim != (void*)r->q.prim) engine_stage_out(e, f, r->q.prim, r->prim, n * 4);
        r->finished = true;
    }
    for (EReq& r : e->res) {
        if (r.lidar || r.srp || !r.finished) continue;
        k_finalize_one<<<grid_for(ctx, k_finalize_one, r.npix), 256, 0, st>>>(B, r.slot);
        check_launch(ctx, "k_finalize_one");
        if (r.q.rgba8 && (void*)r.rgba != (void*)r.q.rgba8)
            engine_stage_out(e, f, r.q.rgba8, r.rgba, (size_t)r.npix * 4);
        if (r.q.radiance && (void*)r.rad != (void*)r.q.radiance)
            engine_stage_out(e, f, r.q.radiance, r.rad, (size_t)r.npix * 16);
    }
    CRT_CUDA(cudaMemcpyAsync(e->err_pin + slot, ctx->d_error, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CRT_CUDA(cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), st));
    CRT_CUDA(cudaEventRecord(f.ev, st));
    f.active = true;
    f.err_slot = slot;
    std::vector<EReq> keep;
    keep.reserve(e->res.size());
    for (EReq& r : e->res) {
        if (r.finished) {
            engine_release(e, r);
            f.tags.push_back(r.tag);
        } else {
            keep.push_back(r);
        }
    }
    e->res.swap(keep);
    e->cur_flight = slot;
    // the previous wave ran while this one was planned: complete it now
    engine_drain_flight(e, e->flights[slot ^ 1], completed);
    // nothing left to run: complete this wave too
    if (e->res.empty()) engine_drain_flight(e, f, completed);
}

namespace {
}  // namespace

void batch_run(crt_context* ctx, const crt_request* reqs, size_t n, crt_batch_stats* stats) {
    run_batch(ctx, reqs, n, stats);
}
void batch_check_request(const crt_request& q) { check_request(q); }

extern "C" int crt_batch(crt_context* ctx, const crt_request* reqs, size_t n, crt_batch_stats* stats) {
    if (!ctx || (n && !reqs)) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] { run_batch(ctx, reqs, n, stats); });
}

extern "C" int crt_batch_mixed(crt_context* ctx, const crt_server_request* reqs, size_t n, crt_batch_stats* stats) {
    if (!ctx || (n && !reqs)) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] {
        std::vector<crt_request> base;
        std::vector<const crt_server_request*> srp;
        for (size_t i = 0; i < n; ++i) {
            if (reqs[i].base.kind == CRT_REQUEST_SRP) srp.push_back(&reqs[i]);
            else base.push_back(reqs[i].base);
        }
        run_batch(ctx, base.data(), base.size(), stats, srp.data(), srp.size());
    });
}

extern "C" int crt_render(crt_scene* s, const crt_camera_desc* cam, const crt_light_desc* lights, uint32_t n_lights,
                          const crt_render_params* p, uint8_t* rgba8, float* radiance) {
    if (!s || !cam || !p || (n_lights && !lights)) return CRT_ERR_INVALID;
    crt_request q;
    std::memset(&q, 0, sizeof(q));
    q.kind = CRT_REQUEST_RENDER;
    q.scene = s;
    q.camera = cam;
    q.lights = lights;
    q.n_lights = n_lights;
    q.params = p;
    q.rgba8 = rgba8;
    q.radiance = radiance;
    return crt_guard(s->ctx, [&] { run_batch(s->ctx, &q, 1, nullptr); });
}
