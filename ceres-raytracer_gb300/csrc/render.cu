// Wavefront unidirectional path tracer: do_render (src/crt/do_render.hpp:28-141) with
// unidirectional (path_tracing/unidirectional.hpp:24-96) restated as separate stage kernels over
// compacted queues:
//
//   primary   camera ray per (pixel, sample) + closest hit          (persistent trace kernel)
//   shade     surface point, one shadow ray per light, bounce ray   (k_shade, appends to queues)
//   shadow    any hit for the shadow queue                          (persistent trace kernel)
//   accum     sum lights, clamp after the first bounce, add weight  (k_accum)
//   bounce    closest hit for the continuing-path queue             (persistent trace kernel)
//   update    per-pixel running mean and adaptive stop              (k_update, k_compact)
//   finalize  RGBA float and clamp(v * 256, 0, 255) bytes           (k_finalize)
//
// A wave holds k consecutive samples of every still-active pixel (path p -> sample p / n_active,
// pixel active[p % n_active]); the update kernel consumes a pixel's samples in order, so the
// running mean and the stopping rule match the reference's sequential loop.  Random numbers come
// from Philox4x32-10 keyed by (seed, request) with counter (pixel, sample, bounce<<8 | purpose,
// request), so an image does not depend on how its samples are grouped into waves or requests.
//
// FP32 secondary-ray origins: the reference offsets the hit point by 1e-4 along the flat normal
// (unidirectional.hpp:59-61).  In FP32 at kilometre coordinates 1e-4 is about one ulp, so the
// offset used here is max(1e-4, 4 ulp of the largest coordinate) and the triangle the ray leaves
// is not re-tested (in FP64 the reference only meets it again when the ray points into the
// surface, which on closed meshes the rest of the mesh occludes anyway).
#include "common.cuh"
#include "trace.cuh"

#include <algorithm>
#include <cmath>

namespace {

constexpr int MAX_LIGHTS = 16;
constexpr uint32_t WAVE_CAP = 1u << 23;   // paths per wave

struct LightDev {
    int type;
    float intensity;
    float pos[3];
    float R[9];
    float size[2];
};
struct LightSet {
    LightDev l[MAX_LIGHTS];
    uint32_t n;
};

struct RenderCtl {
    uint32_t W, H;
    int min_samples, max_samples;
    float noise_threshold;
    int num_bounces;
    uint32_t seed_lo, seed_hi, request;
    float color_scale_unused;
};

struct WaveBufs {
    uint32_t n_active;
    const uint32_t* active;   // nullptr: identity (every pixel)
    uint32_t sample_base;
    uint32_t k;
    float4* ray;      // 2 per path
    uint32_t* skip;
    float4* hit;
    float4* weight;
    float4* wacc;
    float4* rad;
    float4* contrib;  // P * L
    uint8_t* occ;     // P * L
    uint32_t* q_cur;
    uint32_t* q_next;
    uint32_t* counts; // [0] |q_cur|, [1] |q_next|, [2] |shadow|
    float4* sray;     // 2 per shadow entry
    uint32_t* sidx;
    uint32_t* sskip;
};

__device__ __forceinline__ void rng2(const RenderCtl& c, uint32_t pixel, uint32_t sample, uint32_t bounce,
                                     uint32_t purpose, float& a, float& b) {
    uint32_t ctr[4] = {pixel, sample, (bounce << 8) | purpose, c.request};
    philox4x32(ctr, c.seed_lo, c.seed_hi);
    a = unif24(ctr[0]);
    b = unif24(ctr[1]);
}

__device__ __forceinline__ void path_ids(const WaveBufs& w, uint32_t p, uint32_t& pixel, uint32_t& sample) {
    const uint32_t a = p % w.n_active;
    sample = w.sample_base + p / w.n_active;
    pixel = w.active ? w.active[a] : a;
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

// ---------------------------------------------------------------- primary rays
struct PrimaryJob {
    CamBasis cam;
    RenderCtl c;
    WaveBufs w;
    __device__ bool ray(uint32_t p, TRay& r) const {
        uint32_t pixel, sample;
        path_ids(w, p, pixel, sample);
        const uint32_t i = pixel % c.W, j = pixel / c.W;
        float u = (float)i, v = (float)j;
        if (c.max_samples != 1) {   // do_render.hpp:76-82: integer coordinates for a single sample
            float a, b;
            rng2(c, pixel, sample, 0, 0, a, b);
            u += a - 0.5f;
            v += b - 0.5f;
        }
        r = camera_ray(cam, u, v);
        return true;
    }
    __device__ void write(const SceneView&, uint32_t p, const TRay&, const THit& h) const {
        w.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
        const float w0 = (float)(2.0 * 3.14159265358979323846);   // Color(2*M_PI), unidirectional.hpp:38
        w.weight[p] = make_float4(w0, w0, w0, 0.f);
        w.rad[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
};

struct ShadowJob {
    WaveBufs w;
    __device__ bool ray(uint32_t i, TRay& r) const {
        const float4 a = w.sray[2ull * i], b = w.sray[2ull * i + 1];
        r.o = f3(a.x, a.y, a.z);
        r.tmin = a.w;
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        r.skip = w.sskip[i];
        return true;
    }
    __device__ void write(const SceneView&, uint32_t i, const TRay&, const THit& h) const {
        if (h.slot != CRT_MISS) w.occ[w.sidx[i]] = 1;
    }
};

struct BounceJob {
    WaveBufs w;
    __device__ bool ray(uint32_t i, TRay& r) const {
        const uint32_t p = w.q_next[i];
        const float4 a = w.ray[2ull * p], b = w.ray[2ull * p + 1];
        r.o = f3(a.x, a.y, a.z);
        r.tmin = a.w;
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        r.skip = w.skip[p];
        return true;
    }
    __device__ void write(const SceneView&, uint32_t i, const TRay&, const THit& h) const {
        const uint32_t p = w.q_next[i];
        w.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    }
};

// warp-aggregated append of `cnt` entries per participating lane; returns the lane's first index
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, uint32_t cnt) {
    const uint32_t mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const uint32_t below = __popc(mask & ((1u << lane) - 1u));
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask) * cnt);
    base = __shfl_sync(mask, base, leader);
    return base + below * cnt;
}

// ---------------------------------------------------------------- shade
__global__ void k_shade(SceneView sv, RenderCtl c, WaveBufs w, LightSet L, int bounce, uint32_t n_all) {
    const uint32_t n = bounce == 0 ? n_all : w.counts[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = bounce == 0 ? i : w.q_cur[i];
        const float4 hv = w.hit[p];
        THit h;
        h.t = hv.x; h.u = hv.y; h.v = hv.z;
        h.slot = __float_as_uint(hv.w);
        if (h.slot == CRT_MISS) continue;
        uint32_t pixel, sample;
        path_ids(w, p, pixel, sample);
        const SurfacePoint sp = surface_point(sv, h);
        const EntityDev& E = sv.entities[sp.entity];
        const float3 col = f3(E.color[0], E.color[1], E.color[2]);
        const float3 x = sp.x - origin_offset(sp.x) * sp.flat_n;   // intersect_point - 1e-4 normal
        const uint32_t sbase = warp_append(&w.counts[2], L.n);
        for (uint32_t l = 0; l < L.n; ++l) {
            const LightDev& lt = L.l[l];
            float3 lp = f3(lt.pos[0], lt.pos[1], lt.pos[2]);
            float inten;
            if (lt.type == 1) {   // AreaLight::sample_ray / get_intensity (area_light.hpp:54-72)
                float a, b;
                rng2(c, pixel, sample, (uint32_t)bounce, 2u + l, a, b);
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
            w.contrib[(size_t)p * L.n + l] = make_float4(cb.x * inten, cb.y * inten, cb.z * inten, 0.f);
            w.occ[(size_t)p * L.n + l] = 0;
            const uint32_t e = sbase + l;
            w.sray[2ull * e] = make_float4(x.x, x.y, x.z, 0.f);
            w.sray[2ull * e + 1] = make_float4(dir.x, dir.y, dir.z, dist);
            w.sidx[e] = p * L.n + l;
            w.sskip[e] = h.slot;
        }
        w.wacc[p] = w.weight[p];
        if (bounce < c.num_bounces - 1) {
            float r1, r2;
            rng2(c, pixel, sample, (uint32_t)bounce, 1u, r1, r2);
            const float3 nd = cosine_importance(sp.shading_n, r1, r2);
            w.ray[2ull * p] = make_float4(x.x, x.y, x.z, 0.f);
            w.ray[2ull * p + 1] = make_float4(nd.x, nd.y, nd.z, 3.402823466e38f);
            w.skip[p] = h.slot;
            const float bc = 1.0f - r1;
            float4 wt = w.weight[p];
            w.weight[p] = make_float4(wt.x * bc, wt.y * bc, wt.z * bc, 0.f);
            w.q_next[warp_append(&w.counts[1], 1u)] = p;
        }
    }
}

// ---------------------------------------------------------------- accumulate
__global__ void k_accum(RenderCtl c, WaveBufs w, uint32_t n_lights, int bounce, uint32_t n_all) {
    const uint32_t n = bounce == 0 ? n_all : w.counts[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = bounce == 0 ? i : w.q_cur[i];
        if (__float_as_uint(w.hit[p].w) == CRT_MISS) continue;
        float3 lr = f3(0.f, 0.f, 0.f);
        for (uint32_t l = 0; l < n_lights; ++l) {
            if (!w.occ[(size_t)p * n_lights + l]) {
                const float4 cb = w.contrib[(size_t)p * n_lights + l];
                lr = lr + f3(cb.x, cb.y, cb.z);
            }
        }
        if (bounce >= 1) {   // unidirectional.hpp:74-78
            lr.x = fminf(fmaxf(lr.x, 0.f), 1.f);
            lr.y = fminf(fmaxf(lr.y, 0.f), 1.f);
            lr.z = fminf(fmaxf(lr.z, 0.f), 1.f);
        }
        const float4 wa = w.wacc[p];
        float4 r = w.rad[p];
        w.rad[p] = make_float4(r.x + lr.x * wa.x, r.y + lr.y * wa.y, r.z + lr.z * wa.z, 0.f);
    }
}

// rotate queues: q_cur <- q_next (count only; the host swaps the pointers)
__global__ void k_queue_rotate(uint32_t* counts) {
    counts[0] = counts[1];
    counts[1] = 0;
    counts[2] = 0;
}

// ---------------------------------------------------------------- pixel update (do_render.hpp:84-114)
__global__ void k_update(RenderCtl c, WaveBufs w, float4* __restrict__ pix, uint32_t* __restrict__ taken,
                         uint8_t* __restrict__ done) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < w.n_active; a += gridDim.x * blockDim.x) {
        const uint32_t pixel = w.active ? w.active[a] : a;
        if (done[pixel]) continue;
        float4 m = pix[pixel];
        uint32_t t = taken[pixel];
        for (uint32_t s = 0; s < w.k; ++s) {
            const uint32_t sample = w.sample_base + s + 1;   // 1-based as in the reference loop
            const float4 L = w.rad[(size_t)s * w.n_active + a];
            const float inv = 1.0f / (float)sample;
            const float dx = (L.x - m.x) * inv, dy = (L.y - m.y) * inv, dz = (L.z - m.z) * inv;
            m.x += dx; m.y += dy; m.z += dz;
            t = sample;
            if ((int)sample >= c.min_samples) {
                const float noise = sqrtf(dx * dx + dy * dy + dz * dz);
                if (noise < c.noise_threshold) {
                    done[pixel] = 1;
                    break;
                }
            }
        }
        pix[pixel] = m;
        taken[pixel] = t;
    }
}

__global__ void k_compact(const uint32_t* __restrict__ active, uint32_t n_active, const uint8_t* __restrict__ done,
                          uint32_t* __restrict__ out, uint32_t* __restrict__ count) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n_active; a += gridDim.x * blockDim.x) {
        const uint32_t pixel = active ? active[a] : a;
        if (!done[pixel]) out[warp_append(count, 1u)] = pixel;
    }
}

__global__ void k_finalize(uint32_t n, const float4* __restrict__ pix, float4* __restrict__ rad,
                           uchar4* __restrict__ rgba) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 m = pix[i];
        const float v[4] = {m.x, m.y, m.z, 1.0f};
        if (rad) rad[i] = make_float4(v[0], v[1], v[2], v[3]);
        if (rgba) {
            uint8_t q[4];
            for (int k = 0; k < 4; ++k) q[k] = (uint8_t)fminf(fmaxf(v[k] * 256.0f, 0.0f), 255.0f);
            rgba[i] = make_uchar4(q[0], q[1], q[2], q[3]);
        }
    }
}

inline uint32_t grid_for(crt_context* ctx, size_t n, int block = 256) {
    const size_t want = (n + block - 1) / block;
    return (uint32_t)std::max<size_t>(1, std::min<size_t>(want, (size_t)ctx->sm_count * 8));
}

}  // namespace

extern "C" int crt_render(crt_scene* s, const crt_camera_desc* cam, const crt_light_desc* lights, uint32_t n_lights,
                          const crt_render_params* p, uint8_t* rgba8, float* radiance) {
    if (!s || !cam || !p || (n_lights && !lights)) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n_lights <= (uint32_t)MAX_LIGHTS, CRT_ERR_INVALID, "at most 16 lights per render");
        CRT_CHECK(rgba8 || radiance, CRT_ERR_INVALID, "no output buffer");
        const CamBasis cb = make_camera_basis(cam);
        CRT_CHECK(cb.width > 0 && cb.height > 0 && (uint64_t)cb.width * cb.height < (1ull << 28), CRT_ERR_INVALID,
                  "bad camera resolution");
        CRT_CUDA(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        const uint32_t npix = cb.width * cb.height;
        RenderCtl c;
        c.W = cb.width;
        c.H = cb.height;
        c.min_samples = p->min_samples;
        c.max_samples = p->max_samples;
        c.noise_threshold = (float)p->noise_threshold;
        c.num_bounces = p->num_bounces;
        c.seed_lo = (uint32_t)p->seed;
        c.seed_hi = (uint32_t)(p->seed >> 32);
        c.request = p->request;
        LightSet L;
        L.n = n_lights;
        for (uint32_t l = 0; l < n_lights; ++l) {
            L.l[l].type = lights[l].type;
            L.l[l].intensity = (float)lights[l].intensity;
            for (int k = 0; k < 3; ++k) L.l[l].pos[k] = (float)lights[l].position[k];
            for (int k = 0; k < 9; ++k) L.l[l].R[k] = (float)lights[l].rotation[k];
            L.l[l].size[0] = (float)lights[l].size[0];
            L.l[l].size[1] = (float)lights[l].size[1];
        }
        // pixel state
        char* ps = (char*)ctx_scratch(ctx, SCR_WAVE0, (size_t)npix * (16 + 4 + 1 + 4 + 4) + 1024);
        float4* pix = (float4*)ps;
        uint32_t* taken = (uint32_t*)(ps + (size_t)npix * 16);
        uint32_t* act_a = (uint32_t*)(ps + (size_t)npix * 20);
        uint32_t* act_b = (uint32_t*)(ps + (size_t)npix * 24);
        uint8_t* done = (uint8_t*)(ps + (size_t)npix * 28);
        uint32_t* acount = (uint32_t*)ctx_scratch(ctx, SCR_WAVE1, 64);
        CRT_CUDA(cudaMemsetAsync(pix, 0, (size_t)npix * 16, st));
        CRT_CUDA(cudaMemsetAsync(taken, 0, (size_t)npix * 4, st));
        CRT_CUDA(cudaMemsetAsync(done, 0, npix, st));

        const bool adaptive = p->noise_threshold > 0 && p->min_samples < p->max_samples;
        const uint32_t nl = std::max<uint32_t>(n_lights, 1);
        uint32_t n_active = npix;
        const uint32_t* active = nullptr;
        int sample_base = 0;
        const int total = std::max(0, p->max_samples);
        const SceneView sv = scene_view(s);
        while (sample_base < total && n_active > 0) {
            int k;
            if (!adaptive) k = total - sample_base;
            else if (sample_base == 0) k = std::max(1, std::min(p->min_samples, total));
            else k = 1;
            k = (int)std::min<uint64_t>((uint64_t)k, std::max<uint64_t>(1, WAVE_CAP / n_active));
            const uint32_t P = n_active * (uint32_t)k;
            // wave buffers
            const size_t per = 32 + 4 + 16 + 16 + 16 + 16 + (size_t)nl * (16 + 1) + 8 + (size_t)nl * (32 + 8);
            char* wb = (char*)ctx_scratch(ctx, SCR_WAVE2, (size_t)P * per + 4096);
            WaveBufs w;
            size_t off = 0;
            auto take = [&](size_t bytes) {
                off = (off + 255) & ~size_t(255);
                char* q = wb + off;
                off += bytes;
                return q;
            };
            w.n_active = n_active;
            w.active = active;
            w.sample_base = (uint32_t)sample_base;
            w.k = (uint32_t)k;
            w.ray = (float4*)take((size_t)P * 32);
            w.skip = (uint32_t*)take((size_t)P * 4);
            w.hit = (float4*)take((size_t)P * 16);
            w.weight = (float4*)take((size_t)P * 16);
            w.wacc = (float4*)take((size_t)P * 16);
            w.rad = (float4*)take((size_t)P * 16);
            w.contrib = (float4*)take((size_t)P * nl * 16);
            w.occ = (uint8_t*)take((size_t)P * nl);
            w.q_cur = (uint32_t*)take((size_t)P * 4);
            w.q_next = (uint32_t*)take((size_t)P * 4);
            w.sray = (float4*)take((size_t)P * nl * 32);
            w.sidx = (uint32_t*)take((size_t)P * nl * 4);
            w.sskip = (uint32_t*)take((size_t)P * nl * 4);
            w.counts = acount + 4;
            CRT_CUDA(cudaMemsetAsync(w.counts, 0, 3 * sizeof(uint32_t), st));

            launch_trace<false>(s, PrimaryJob{cb, c, w}, P);
            for (int b = 0; b < p->num_bounces; ++b) {
                k_shade<<<grid_for(ctx, P), 256, 0, st>>>(sv, c, w, L, b, P);
                check_launch(ctx, "k_shade");
                if (n_lights) {
                    launch_trace<true>(s, ShadowJob{w}, P * n_lights, w.counts + 2);
                }
                k_accum<<<grid_for(ctx, P), 256, 0, st>>>(c, w, n_lights, b, P);
                check_launch(ctx, "k_accum");
                if (b < p->num_bounces - 1) {
                    launch_trace<false>(s, BounceJob{w}, P, w.counts + 1);
                    k_queue_rotate<<<1, 1, 0, st>>>(w.counts);
                    check_launch(ctx, "k_queue_rotate");
                    std::swap(w.q_cur, w.q_next);
                }
            }
            k_update<<<grid_for(ctx, n_active), 256, 0, st>>>(c, w, pix, taken, done);
            check_launch(ctx, "k_update");
            sample_base += k;
            if (adaptive && sample_base < total) {
                uint32_t* out = active == act_a ? act_b : act_a;
                CRT_CUDA(cudaMemsetAsync(acount, 0, sizeof(uint32_t), st));
                k_compact<<<grid_for(ctx, n_active), 256, 0, st>>>(active, n_active, done, out, acount);
                check_launch(ctx, "k_compact");
                uint32_t h = 0;
                CRT_CUDA(cudaMemcpyAsync(&h, acount, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                CRT_CUDA(cudaStreamSynchronize(st));
                n_active = h;
                active = out;
            }
        }
        float4* d_rad = (float4*)out_device(ctx, radiance, (size_t)npix * 16, SCR_OUT0);
        uchar4* d_rgba = (uchar4*)out_device(ctx, rgba8, (size_t)npix * 4, SCR_OUT1);
        k_finalize<<<grid_for(ctx, npix), 256, 0, st>>>(npix, pix, d_rad, d_rgba);
        check_launch(ctx, "k_finalize");
        out_finish(ctx, radiance, d_rad, (size_t)npix * 16);
        out_finish(ctx, rgba8, d_rgba, (size_t)npix * 4);
        if ((radiance && (void*)d_rad != (void*)radiance) || (rgba8 && (void*)d_rgba != (void*)rgba8))
            check_device_error(ctx, "crt_render");
    });
}
