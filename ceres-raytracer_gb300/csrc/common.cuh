// Internal declarations shared by the CUDA translation units of libcrt_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include <mutex>

#include "crt_gpu.h"

// ------------------------------------------------------------------ error plumbing
struct CrtError {
    int status;
    std::string msg;
};

#define CRT_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            throw CrtError{e_ == cudaErrorMemoryAllocation ? CRT_ERR_OOM : CRT_ERR_CUDA,      \
                           std::string(#call) + ": " + cudaGetErrorString(e_)};               \
    } while (0)

#define CRT_CHECK(cond, status, msg)                                                          \
    do {                                                                                      \
        if (!(cond)) throw CrtError{(status), (msg)};                                         \
    } while (0)

// ------------------------------------------------------------------ device error word bits
enum : uint32_t {
    DEVERR_STACK_OVERFLOW = 1u << 0,
    DEVERR_BUILD_OVERFLOW = 1u << 1,
    DEVERR_QUANT_RANGE = 1u << 2,
    DEVERR_WAIT_LIMIT = 1u << 3,
    DEVERR_BAD_INDEX = 1u << 4,
};

// ------------------------------------------------------------------ context
enum ScratchSlot {
    SCR_QUEUE = 0,      // persistent-kernel work counters
    SCR_RAYS,           // staged rays / hits
    SCR_OUT0,
    SCR_OUT1,
    SCR_OUT2,
    SCR_IN0,
    SCR_IN1,
    SCR_BUILD0,
    SCR_BUILD1,
    SCR_BUILD2,
    SCR_BUILD3,
    SCR_BUILD4,
    SCR_BUILD5,
    SCR_BUILD6,
    SCR_BUILD7,
    SCR_WAVE0,
    SCR_WAVE1,
    SCR_WAVE2,
    SCR_WAVE3,
    SCR_WAVE4,
    SCR_WAVE5,
    SCR_WAVE6,
    SCR_WAVE7,
    SCR_COUNT
};

struct crt_context {
    int device = 0;
    int sm_count = 0;
    int max_threads_per_sm = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;
    bool counting = false;
    unsigned long long* d_counters = nullptr;   // rays, nodes, tris, resolved
    uint32_t* d_error = nullptr;                // device error word
    uint64_t launches = 0;
    void* scratch[SCR_COUNT] = {};
    size_t scratch_bytes[SCR_COUNT] = {};
    // upload staging: a ring of two grow-only pinned buffers, each with the event after its last copy
    void* pinned[2] = {nullptr, nullptr};
    size_t pinned_bytes[2] = {0, 0};
    cudaEvent_t pinned_ev[2] = {nullptr, nullptr};
    int pinned_next = 0;
    // tuning (crt_context_set_tuning; the autotuner picks these per GPU and scene class)
    uint32_t queue_chunk = 1;        // 32-item groups per atomic grab of the ray queue
    uint32_t wave_paths = 1u << 23;  // render paths per wavefront wave
    int use_graphs = 1;              // replay batched waves as CUDA graphs
    int build_sah = 1;               // scene builds: binned-SAH topology (1) or Karras radix tree (0)
    float collapse_tri_cost = 0.15f; // scene builds: triangle-test cost of the 8-wide collapse (node = 1)
    uint32_t treelet_passes = 1;     // scene builds: treelet-restructuring passes over the binary tree
};

// Grow-only device scratch buffer for one purpose.  Synchronises the stream before reallocating.
void* ctx_scratch(crt_context* ctx, ScratchSlot slot, size_t bytes);
// Pinned host staging for one call's uploads, from a ring of two grow-only buffers.  Acquiring waits
// only until the copies out of the buffer's previous use have run, not for the whole stream, so the
// host prepares a call while the GPU still runs the previous one.  release() records that point on
// the stream once the copies out of the buffer are enqueued (later reuse of the buffer within the
// call must synchronise itself); the destructor records it if release() was not reached.
struct PinnedStaging {
    crt_context* ctx;
    int slot;
    char* p;
    bool released = false;
    PinnedStaging(crt_context* c, size_t bytes);
    void release();
    ~PinnedStaging();
    PinnedStaging(const PinnedStaging&) = delete;
    PinnedStaging& operator=(const PinnedStaging&) = delete;
};
bool is_device_ptr(const void* p);
// Page-locked host memory that the device writes at the same address (cudaHostAlloc'd or registered).
bool is_host_mapped(const void* p);
// Host memory (any kind): a call writing it completes before returning.
inline bool host_output(const void* p) { return p && !is_device_ptr(p); }
// Copy helpers: ensure `bytes` of `src` are readable on the device; return a device pointer.
const void* to_device(crt_context* ctx, const void* src, size_t bytes, ScratchSlot slot);
// Output staging: returns a device pointer to write into (dst itself when it is device memory).
void* out_device(crt_context* ctx, void* dst, size_t bytes, ScratchSlot slot);
// As out_device, and dst itself also when it is mapped page-locked host memory: the kernel's stores
// cross the host link while it runs, instead of a copy after it (outputs written once, not read).
void* out_direct(crt_context* ctx, void* dst, size_t bytes, ScratchSlot slot);
// Copy a staged output back to host memory (no-op for device outputs); synchronous for host outputs.
void out_finish(crt_context* ctx, void* dst, const void* staged, size_t bytes);
void check_launch(crt_context* ctx, const char* what);
// Read and clear the device error word; throws CRT_ERR_DEVICE when set.
void check_device_error(crt_context* ctx, const char* what);

template <typename F>
int crt_guard(crt_context* ctx, F&& f) {
    try {
        f();
        return CRT_OK;
    } catch (const CrtError& e) {
        if (ctx) ctx->last_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->last_error = "host allocation failed";
        return CRT_ERR_OOM;
    } catch (const std::exception& e) {
        if (ctx) ctx->last_error = e.what();
        return CRT_ERR_INVALID;
    }
}

// ------------------------------------------------------------------ scene
// 8-wide compressed node, 128 bytes = 8 x float4:
//  w0: origin p (float x3), exponents ex/ey/ez (int8) + imask (uint8)
//  w1: child_base (uint32), tri_base (uint32), meta[0..7] (uint8)
//  w2..w4: qlo_x[8], qlo_y[8], qlo_z[8]     w5..w7: qhi_x[8], qhi_y[8], qhi_z[8]
//  each plane q (0..255, in quanta 2^e from p) stored as the half 0x5C00 | q = 256 + q / 4: the
//  traversal converts it with one half-to-float conversion on the FMA pipe, where a byte extraction
//  (PRMT) would load the ALU pipe that the slab test's min / max already keeps busy.
// meta per slot: 0 = empty; internal child: (1 << 5) | (24 + slot);
//                leaf: (unary triangle count << 5) | offset from tri_base (< 24).
// Internal children are stored contiguously from child_base in slot order.
struct WideNode {
    float4 w[8];
};
static_assert(sizeof(WideNode) == 128, "wide node must be 128 bytes");

struct EntityDev {
    float color[3];
    uint32_t smooth;
    uint32_t id;
    float rho_s, rho_d;
    uint32_t pad;
};

struct crt_scene {
    crt_context* ctx = nullptr;
    size_t n_tris = 0;
    uint32_t n_entities = 0;
    size_t n_nodes = 0;
    uint32_t depth = 0;
    WideNode* nodes = nullptr;
    float4* tris = nullptr;           // 3 float4 per leaf slot: (p0, p1.x) (p1.yz, p2.xy) (p2.z, n)
    uint32_t* leaf_prim = nullptr;    // leaf slot -> scene primitive index
    float4* leaf_vn = nullptr;        // 3 float4 per leaf slot: vertex normals vn0, vn1, vn2 (xyz)
    uint32_t* leaf_entity = nullptr;  // leaf slot -> entity index
    EntityDev* entities = nullptr;
    float bounds[6] = {0, 0, 0, 0, 0, 0};
    double build_ms = 0;
    size_t device_bytes = 0;
    std::vector<EntityDev> host_entities;
};

void scene_build(crt_scene* s, const crt_entity_desc* ents, uint32_t n);   // bvh_build.cu

// render.cu: batched wavefront on an explicit context (its stream, scratch and error word)
void batch_run(crt_context* ctx, const crt_request* reqs, size_t n, crt_batch_stats* stats);
void batch_check_request(const crt_request& q);
// serving engine (render.cu): resident requests, one wave per step
struct WaveEngine;
WaveEngine* engine_create(crt_context* ctx, size_t budget_bytes);
void engine_destroy(WaveEngine* e);
bool engine_admit(WaveEngine* e, const crt_request& q, uint64_t tag);
bool engine_admit_srp(WaveEngine* e, crt_scene* scene, const crt_srp_desc& desc, const double* quats, size_t n_att,
                      double* force, double* torque, uint64_t tag);
void engine_step(WaveEngine* e, std::vector<uint64_t>& completed);
void engine_abort(WaveEngine* e, std::vector<uint64_t>& dropped);
// srp.cu: radiation pressure on an explicit context
void srp_run(crt_context* ctx, crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att,
             double* force, double* torque, double* facet_power);

// ------------------------------------------------------------------ device math
__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize3(float3 a) { return a * (1.0f / sqrtf(dot3(a, a))); }

// Ray in registers for traversal.
struct TRay {
    float3 o, d;
    float tmin, tmax;
    uint32_t skip = CRT_MISS;   // leaf slot not tested (origin triangle of a secondary ray)
};

// Result of the triangle test in leaf-slot space.
struct THit {
    float t, u, v;
    uint32_t slot;   // CRT_MISS when nothing was hit
};

// Per-ray constants of the watertight triangle test: the shear of Woop, Benthin and Wald ("Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013) that maps the ray onto its dominant axis kz, written as
// two vectors, x' = (p - o) . bx and y' = (p - o) . by with bx = e_kx - (d_kx / d_kz) e_kz (by
// likewise), so the projection of a vertex needs no per-vertex permutation of components; ox, oy are
// the projected origin (o . bx, o . by, set by the caller).
struct TShear {
    float3 bx, by;
    float ox, oy;
};
__device__ __forceinline__ TShear make_shear(float3 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
    const float dz = kz == 0 ? d.x : (kz == 1 ? d.y : d.z);
    if (dz < 0.0f) {   // keeps the winding of the projected triangle
        const int k = kx;
        kx = ky;
        ky = k;
    }
    const float rz = 1.0f / dz;
    const float sx = (kx == 0 ? d.x : (kx == 1 ? d.y : d.z)) * rz;
    const float sy = (ky == 0 ? d.x : (ky == 1 ? d.y : d.z)) * rz;
    TShear s;
    s.bx = f3(kx == 0 ? 1.0f : (kz == 0 ? -sx : 0.0f), kx == 1 ? 1.0f : (kz == 1 ? -sx : 0.0f),
              kx == 2 ? 1.0f : (kz == 2 ? -sx : 0.0f));
    s.by = f3(ky == 0 ? 1.0f : (kz == 0 ? -sy : 0.0f), ky == 1 ? 1.0f : (kz == 1 ? -sy : 0.0f),
              ky == 2 ? 1.0f : (kz == 2 ? -sy : 0.0f));
    return s;
}

// Point u p1 + v p2 + (1 - u - v) p0 of the triangle record (a, b, c) (passes.hpp:53), evaluated as
// p0 + u (p1 - p0) + v (p2 - p0): the edge differences are exact for the nearby vertices of a mesh.
__device__ __forceinline__ float3 tri_point(const float4 a, const float4 b, const float4 c, float u, float v) {
    return f3(__fmaf_rn(v, b.z - a.x, __fmaf_rn(u, a.w - a.x, a.x)), __fmaf_rn(v, b.w - a.y, __fmaf_rn(u, b.x - a.y, a.y)),
              __fmaf_rn(v, c.x - a.z, __fmaf_rn(u, b.y - a.z, a.z)));
}

// Watertight form of Triangle::intersect (lib/bvh/triangle.hpp:140-160), same acceptance: the ray
// meets the triangle (barycentrics u, v, w >= 0) at tmin <= t <= tmax.  The vertices are sheared onto
// the ray's dominant axis and moved to the ray origin (p . b - o . b, three fused multiply-adds per
// coordinate); each vertex's 2-D image depends only on the vertex and the ray, and the edge functions
// are products and one difference without fused multiply-adds, so the two triangles on an edge
// compute the same value with opposite signs and no ray passes between them (the FP32 form of
// c = p0 - o, (d x c) . e of every triangle from its own p0 leaves cracks about one ulp of the ray's
// coordinates wide along shared edges).  A ray on an edge (an edge function exactly zero) hits both
// sides.  The image's rounding is that of the coordinates (about 2^-24 |p|), the FP32 vertices' own.
// t is the plane distance (n . (p0 - o)) / (n . d) as in the reference; the weights of p1 and p2 come
// back unnormalised (wv, ww, their sum with the weight of p0 in det): u = wv / det, v = ww / det,
// divided once for the final hit.
__device__ __forceinline__ float shear_proj(float3 a, float3 b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ float edge_fn(float px, float py, float qx, float qy) {
    return __fsub_rn(__fmul_rn(qx, py), __fmul_rn(qy, px));
}
__device__ __forceinline__ bool tri_test(const float4 a, const float4 b, const float4 c4, const TRay& r,
                                         const TShear& s, float& t, float& wv, float& ww, float& det) {
    const float ax = __fmaf_rn(a.z, s.bx.z, __fmaf_rn(a.y, s.bx.y, __fmaf_rn(a.x, s.bx.x, -s.ox)));
    const float ay = __fmaf_rn(a.z, s.by.z, __fmaf_rn(a.y, s.by.y, __fmaf_rn(a.x, s.by.x, -s.oy)));
    const float bx = __fmaf_rn(b.y, s.bx.z, __fmaf_rn(b.x, s.bx.y, __fmaf_rn(a.w, s.bx.x, -s.ox)));
    const float by = __fmaf_rn(b.y, s.by.z, __fmaf_rn(b.x, s.by.y, __fmaf_rn(a.w, s.by.x, -s.oy)));
    const float cx = __fmaf_rn(c4.x, s.bx.z, __fmaf_rn(b.w, s.bx.y, __fmaf_rn(b.z, s.bx.x, -s.ox)));
    const float cy = __fmaf_rn(c4.x, s.by.z, __fmaf_rn(b.w, s.by.y, __fmaf_rn(b.z, s.by.x, -s.oy)));
    const float3 A = f3(a.x - r.o.x, a.y - r.o.y, a.z - r.o.z);
    const float U = edge_fn(bx, by, cx, cy);   // edge p1 -> p2: weight of p0
    const float V = edge_fn(cx, cy, ax, ay);   // edge p2 -> p0: weight of p1
    const float W = edge_fn(ax, ay, bx, by);   // edge p0 -> p1: weight of p2
    if (fminf(U, fminf(V, W)) < 0.0f && fmaxf(U, fmaxf(V, W)) > 0.0f) return false;
    const float dt = U + V + W;
    if (!(fabsf(dt) > 0.0f)) return false;   // also rejects NaN
    const float3 n = f3(c4.y, c4.z, c4.w);
    const float tt = __fdividef(dot3(n, A), dot3(n, r.d));
    if (!(tt >= r.tmin && tt <= r.tmax)) return false;
    t = tt;
    wv = V;
    ww = W;
    det = dt;
    return true;
}

// Vector::safe_inverse (lib/bvh/vector.hpp:75-80) in FP32.
__device__ __forceinline__ float safe_rcp(float x) {
    const float eps = 1.1920929e-07f;
    return 1.0f / (fabsf(x) < eps ? copysignf(eps, x) : x);
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter (c0..c3), key (k0, k1).
__host__ __device__ __forceinline__ void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
// 24-bit uniform in [0, 1), exactly representable in float and double
__host__ __device__ __forceinline__ float unif24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Host-side FP64 -> FP32 camera basis: direction(u, v) = normalize(a + u b + v c).
struct CamBasis {
    float o[3];
    float a[3], b[3], c[3];
    double o64[3], a64[3], b64[3], c64[3];   // the same basis in FP64 (reported distances)
    uint32_t width, height;
};

// Distance along an FP64 ray (o, d) to the plane of the FP32 triangle stored at leaf `slot`
// (p0 and n of the record): the traversal picks the triangle in FP32, the reported hit point and
// range are then evaluated along the FP64 ray of the FP64 pose, as the reference evaluates them.
// FP64 reciprocal and inverse square root from an FP32 seed and one Newton-Raphson step
// (y <- y (2 - x y), y <- y (3 - x y^2) / 2): the seed's relative error e becomes about e^2, i.e.
// ~1e-14, far below the 1e-5 the FP64 epilogues need, for a few FP64 fused multiply-adds instead of
// a full-precision FP64 division or square root (GB300 runs FP64 at a small fraction of its FP32
// rate).  Inputs outside the FP32 normal range give a non-finite result; callers test isfinite.
__device__ __forceinline__ double rcp64(double x) {
    const double y = (double)__frcp_rn((float)x);
    return y * fma(-x, y, 2.0);
}
__device__ __forceinline__ double rsqrt64(double x) {
    const double y = (double)rsqrtf((float)x);
    return y * fma(-0.5 * x, y * y, 1.5);
}

__device__ __forceinline__ double plane_t64(const float4* __restrict__ tris, uint32_t slot, const double o[3],
                                            const double d[3]) {
    const float4 a = __ldg(tris + 3ull * slot), c = __ldg(tris + 3ull * slot + 2);
    const double n0 = c.y, n1 = c.z, n2 = c.w;
    const double den = n0 * d[0] + n1 * d[1] + n2 * d[2];
    const double num = n0 * ((double)a.x - o[0]) + n1 * ((double)a.y - o[1]) + n2 * ((double)a.z - o[2]);
    return num * rcp64(den);
}

// Barycentric u, v of the FP64 ray (o, d) on the FP32 triangle at leaf `slot`, with the reference's
// formula (triangle.hpp:140-160) in FP64; false if the determinant vanishes.
__device__ __forceinline__ bool bary64(const float4* __restrict__ tris, uint32_t slot, const double o[3],
                                       const double d[3], double& u, double& v) {
    const float4 a = __ldg(tris + 3ull * slot), b = __ldg(tris + 3ull * slot + 1), c4 = __ldg(tris + 3ull * slot + 2);
    const double p0[3] = {a.x, a.y, a.z}, n[3] = {c4.y, c4.z, c4.w};
    // e1 = p0 - p1, e2 = p2 - p0 (triangle.hpp:31-33), exact in FP64 from the FP32 vertices
    const double e1[3] = {p0[0] - (double)a.w, p0[1] - (double)b.x, p0[2] - (double)b.y};
    const double e2[3] = {(double)b.z - p0[0], (double)b.w - p0[1], (double)c4.x - p0[2]};
    const double c[3] = {p0[0] - o[0], p0[1] - o[1], p0[2] - o[2]};
    const double r[3] = {d[1] * c[2] - d[2] * c[1], d[2] * c[0] - d[0] * c[2], d[0] * c[1] - d[1] * c[0]};
    const double det = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
    if (det == 0.0) return false;
    const double inv = rcp64(det);
    u = (r[0] * e2[0] + r[1] * e2[1] + r[2] * e2[2]) * inv;
    v = (r[0] * e1[0] + r[1] * e1[1] + r[2] * e1[2]) * inv;
    return isfinite(u) && isfinite(v);
}
CamBasis make_camera_basis(const crt_camera_desc* cam);

// Kernel launch helpers
int occupancy_grid(crt_context* ctx, const void* kernel, int block, size_t smem);
