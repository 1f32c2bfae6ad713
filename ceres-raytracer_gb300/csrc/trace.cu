// Ray-query kernels: explicit rays (closest / any hit), primary-ray passes, LiDAR.
//
// One persistent kernel template serves every query.  Warps take 32 work items at a time from an
// atomic counter (the ray queue) until it runs dry; a work item is turned into a ray by the job's
// ray() (camera pixel, LiDAR beam, explicit ray), traversed, and written by the job's write().
// Camera and LiDAR-grid items map 32 consecutive items to an 8 x 4 pixel tile so that a warp's
// rays are coherent.
#include "common.cuh"
#include "trace.cuh"

#include <algorithm>
#include <cmath>

namespace {

// ---------------------------------------------------------------- jobs
struct RayClosestJob : JobBase {
    static constexpr int kMinBlocks = 6;   // resident trace blocks per SM (trace_min_blocks)
    const float4* rays;   // crt_ray as 2 x float4
    crt_hit* hits;
    __device__ bool ray(uint32_t i, TRay& r, Item&) const {
        const float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
        r.o = f3(a.x, a.y, a.z);
        r.tmin = a.w;
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        return true;
    }
    __device__ void write(const SceneView& sv, uint32_t i, const TRay&, const THit& h, const Item&) const {
        crt_hit o;
        if (h.slot != CRT_MISS) {
            o.t = h.t; o.u = h.u; o.v = h.v;
            o.prim = sv.leaf_prim[h.slot];
        } else {
            o.t = o.u = o.v = 0.f;
            o.prim = CRT_MISS;
        }
        reinterpret_cast<float4*>(hits)[i] = make_float4(o.t, o.u, o.v, __uint_as_float(o.prim));
    }
};

struct RayAnyJob : JobBase {
    const float4* rays;
    uint8_t* occluded;
    __device__ bool ray(uint32_t i, TRay& r, Item&) const {
        const float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
        r.o = f3(a.x, a.y, a.z);
        r.tmin = a.w;
        r.d = f3(b.x, b.y, b.z);
        r.tmax = b.w;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t i, const TRay&, const THit& h, const Item&) const {
        occluded[i] = h.slot != CRT_MISS ? 1 : 0;
    }
};

__device__ __forceinline__ bool tile_pixel(uint32_t i, uint32_t W, uint32_t H, uint32_t& px, uint32_t& py) {
    const uint32_t tiles_x = (W + 7) >> 3;
    const uint32_t tile = i >> 5, w = i & 31u;
    px = (tile % tiles_x) * 8u + (w & 7u);
    py = (tile / tiles_x) * 4u + (w >> 3);
    return px < W && py < H;
}

struct PassJob : JobBase {
    CamBasis cam;
    double* xyz;
    uint32_t* ids;
    double* normals;
    __device__ bool ray(uint32_t i, TRay& r, Item&) const {
        uint32_t px, py;
        if (!tile_pixel(i, cam.width, cam.height, px, py)) return false;
        r = camera_ray(cam, (float)px, (float)py);
        return true;
    }
    __device__ void write(const SceneView& sv, uint32_t i, const TRay&, const THit& h, const Item&) const {
        uint32_t px, py;
        tile_pixel(i, cam.width, cam.height, px, py);
        const size_t pix = (size_t)py * cam.width + px;
        double x[3] = {0.0, 0.0, 0.0};
        float3 nrm = f3(0.f, 0.f, 0.f);
        uint32_t id = 0;
        double n64[3] = {0.0, 0.0, 0.0};
        if (h.slot != CRT_MISS) {
            SurfacePoint sp = surface_point(sv, h);
            nrm = sp.shading_n;
            id = sp.id;
            const bool smooth = sv.entities[sp.entity].smooth && sv.leaf_vn;
            if (xyz || (normals && smooth)) {
                // evaluate along the FP64 camera ray of this pixel (pixel_to_ray, simple_camera.hpp:61-81)
                double o[3], d[3];
                for (int k = 0; k < 3; ++k) {
                    o[k] = cam.o64[k];
                    d[k] = cam.a64[k] + (double)px * cam.b64[k] + (double)py * cam.c64[k];
                }
                const double inv = rsqrt64(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (int k = 0; k < 3; ++k) d[k] *= inv;
                if (xyz) {
                    double t = plane_t64(sv.tris, h.slot, o, d);
                    if (!isfinite(t)) t = h.t;
                    for (int k = 0; k < 3; ++k) x[k] = o[k] + t * d[k];
                }
                if (normals && smooth) {
                    double u, v;
                    if (bary64(sv.tris, h.slot, o, d, u, v)) {
                        // normalize(u vn1 + v vn2 + (1 - u - v) vn0) (passes.hpp:179)
                        const float4* vp = sv.leaf_vn + 3ull * h.slot;
                        const float4 v0 = __ldg(vp), v1 = __ldg(vp + 1), v2 = __ldg(vp + 2);
                        const double w = 1.0 - u - v;
                        n64[0] = u * v1.x + v * v2.x + w * v0.x;
                        n64[1] = u * v1.y + v * v2.y + w * v0.y;
                        n64[2] = u * v1.z + v * v2.z + w * v0.z;
                        const double l = rsqrt64(n64[0] * n64[0] + n64[1] * n64[1] + n64[2] * n64[2]);
                        for (int k = 0; k < 3; ++k) n64[k] *= l;
                    } else {
                        n64[0] = nrm.x; n64[1] = nrm.y; n64[2] = nrm.z;
                    }
                } else {
                    n64[0] = nrm.x; n64[1] = nrm.y; n64[2] = nrm.z;
                }
            } else {
                n64[0] = nrm.x; n64[1] = nrm.y; n64[2] = nrm.z;
            }
        }
        if (xyz) {
            xyz[3 * pix] = x[0]; xyz[3 * pix + 1] = x[1]; xyz[3 * pix + 2] = x[2];
        }
        if (normals) {
            normals[3 * pix] = n64[0]; normals[3 * pix + 1] = n64[1]; normals[3 * pix + 2] = n64[2];
        }
        if (ids) ids[pix] = id;
    }
};

struct LidarBatchJob : JobBase {
    const double* pos;
    const double* rot;
    float zsign;
    double* range;
    uint32_t* prim;
    __device__ bool ray(uint32_t i, TRay& r, Item&) const {
        // SimpleLidar::batch_cast_rays: direction R^T (0, 0, +-1) = +-(R[2][0], R[2][1], R[2][2])
        r.o = f3((float)pos[3ull * i], (float)pos[3ull * i + 1], (float)pos[3ull * i + 2]);
        r.d = f3((float)(zsign * rot[9ull * i + 6]), (float)(zsign * rot[9ull * i + 7]), (float)(zsign * rot[9ull * i + 8]));
        r.tmin = 0.f;
        r.tmax = 3.402823466e38f;
        return true;
    }
    __device__ void write(const SceneView& sv, uint32_t i, const TRay&, const THit& h, const Item&) const {
        // do_lidar.hpp:49-59: |hit - position|, 0 on a miss; evaluated along the FP64 pose ray
        double rng = 0.0;
        if (h.slot != CRT_MISS) {
            const double o[3] = {pos[3ull * i], pos[3ull * i + 1], pos[3ull * i + 2]};
            const double d[3] = {zsign * rot[9ull * i + 6], zsign * rot[9ull * i + 7], zsign * rot[9ull * i + 8]};
            const double t = plane_t64(sv.tris, h.slot, o, d);
            const double q = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double len = q * rsqrt64(q);
            rng = isfinite(t) && isfinite(len) ? t * len : (double)h.t;
        }
        range[i] = rng;
        if (prim) prim[i] = h.slot != CRT_MISS ? sv.leaf_prim[h.slot] : CRT_MISS;
    }
};

struct LidarGridJob : JobBase {
    double o[3];
    double rt[9];         // R^T row-major (world = rt * sensor direction)
    double zsign;
    uint32_t nx, ny;
    const double* tx;     // nx tangents
    const double* ty;     // ny tangents
    double* range;
    uint32_t* prim;
    __device__ void beam64(uint32_t px, uint32_t py, double d[3]) const {
        const double s0 = tx[px], s1 = ty[py], s2 = zsign;
        const double inv = rsqrt64(s0 * s0 + s1 * s1 + s2 * s2);
        for (int k = 0; k < 3; ++k) d[k] = (rt[3 * k] * s0 + rt[3 * k + 1] * s1 + rt[3 * k + 2] * s2) * inv;
    }
    __device__ bool ray(uint32_t i, TRay& r, Item&) const {
        uint32_t px, py;
        if (!tile_pixel(i, nx, ny, px, py)) return false;
        double d[3];
        beam64(px, py, d);
        r.o = f3((float)o[0], (float)o[1], (float)o[2]);
        r.d = f3((float)d[0], (float)d[1], (float)d[2]);
        r.tmin = 0.f;
        r.tmax = 3.402823466e38f;
        return true;
    }
    __device__ void write(const SceneView& sv, uint32_t i, const TRay&, const THit& h, const Item&) const {
        uint32_t px, py;
        tile_pixel(i, nx, ny, px, py);
        const size_t k = (size_t)py * nx + px;
        double rng = 0.0;
        if (h.slot != CRT_MISS) {
            double d[3];
            beam64(px, py, d);
            const double t = plane_t64(sv.tris, h.slot, o, d);
            rng = isfinite(t) ? t : (double)h.t;
        }
        range[k] = rng;
        if (prim) prim[k] = h.slot != CRT_MISS ? sv.leaf_prim[h.slot] : CRT_MISS;
    }
};

inline uint32_t tiles_items(uint32_t W, uint32_t H) { return ((W + 7) / 8) * ((H + 3) / 4) * 32u; }

// beam tangents tan(-half + (i + 0.5) 2 half / n) for both axes, FP64, computed on the device so
// the call needs no host staging
__global__ void k_tan_table(double* __restrict__ out, uint32_t nx, uint32_t ny, double hx, double hy) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx) out[i] = tan(-hx + (i + 0.5) * 2.0 * hx / nx);
    else if (i < nx + ny) out[i] = tan(-hy + ((i - nx) + 0.5) * 2.0 * hy / ny);
}

// Shared finish: copy host outputs back and surface device-side failures.
void finish(crt_context* ctx, bool host_out, const char* what) {
    if (host_out) check_device_error(ctx, what);
}

}  // namespace

extern "C" {

int crt_trace_closest(crt_scene* s, const crt_ray* rays, size_t n, crt_hit* hits) {
    if (!s) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n < 0xFFFFFF00u, CRT_ERR_INVALID, "too many rays for one call");
        CRT_CHECK(n == 0 || (rays && hits), CRT_ERR_INVALID, "null buffer");
        if (!n) return;
        CRT_CUDA(cudaSetDevice(ctx->device));
        const float4* d_rays = (const float4*)to_device(ctx, rays, n * sizeof(crt_ray), SCR_IN0);
        crt_hit* d_hits = (crt_hit*)out_direct(ctx, hits, n * sizeof(crt_hit), SCR_OUT0);
        launch_trace<false>(s, RayClosestJob{{}, d_rays, d_hits}, (uint32_t)n);
        out_finish(ctx, hits, d_hits, n * sizeof(crt_hit));
        finish(ctx, host_output(hits), "crt_trace_closest");
    });
}

int crt_trace_any(crt_scene* s, const crt_ray* rays, size_t n, uint8_t* occluded) {
    if (!s) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n < 0xFFFFFF00u, CRT_ERR_INVALID, "too many rays for one call");
        CRT_CHECK(n == 0 || (rays && occluded), CRT_ERR_INVALID, "null buffer");
        if (!n) return;
        CRT_CUDA(cudaSetDevice(ctx->device));
        const float4* d_rays = (const float4*)to_device(ctx, rays, n * sizeof(crt_ray), SCR_IN0);
        uint8_t* d_occ = (uint8_t*)out_direct(ctx, occluded, n, SCR_OUT0);
        launch_trace<true>(s, RayAnyJob{{}, d_rays, d_occ}, (uint32_t)n);
        out_finish(ctx, occluded, d_occ, n);
        finish(ctx, host_output(occluded), "crt_trace_any");
    });
}

int crt_passes(crt_scene* s, const crt_camera_desc* cam, double* xyz, uint32_t* ids, double* normals) {
    if (!s || !cam) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CamBasis cb = make_camera_basis(cam);
        CRT_CHECK(cb.width > 0 && cb.height > 0 && (uint64_t)cb.width * cb.height < (1ull << 31), CRT_ERR_INVALID,
                  "bad camera resolution");
        CRT_CHECK(std::isfinite(cb.a[0] + cb.a[1] + cb.a[2] + cb.b[0] + cb.c[1] + cb.o[0] + cb.o[1] + cb.o[2]),
                  CRT_ERR_INVALID, "camera pose or intrinsics are not finite");
        CRT_CUDA(cudaSetDevice(ctx->device));
        const size_t np = (size_t)cb.width * cb.height;
        double* d_xyz = (double*)out_direct(ctx, xyz, np * 24, SCR_OUT0);
        uint32_t* d_ids = (uint32_t*)out_direct(ctx, ids, np * 4, SCR_OUT1);
        double* d_nrm = (double*)out_direct(ctx, normals, np * 24, SCR_OUT2);
        launch_trace<false>(s, PassJob{{}, cb, d_xyz, d_ids, d_nrm}, tiles_items(cb.width, cb.height));
        out_finish(ctx, xyz, d_xyz, np * 24);
        out_finish(ctx, ids, d_ids, np * 4);
        out_finish(ctx, normals, d_nrm, np * 24);
        finish(ctx, host_output(xyz) || host_output(ids) || host_output(normals), "crt_passes");
    });
}

int crt_lidar_batch(crt_scene* s, const double* positions, const double* rotations, size_t n, int z_positive,
                    double* range, uint32_t* prim) {
    if (!s) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n < 0xFFFFFF00u, CRT_ERR_INVALID, "too many poses for one call");
        CRT_CHECK(n == 0 || (positions && rotations && range), CRT_ERR_INVALID, "null buffer");
        if (!n) return;
        CRT_CUDA(cudaSetDevice(ctx->device));
        const double* d_pos = (const double*)to_device(ctx, positions, n * 24, SCR_IN0);
        const double* d_rot = (const double*)to_device(ctx, rotations, n * 72, SCR_IN1);
        double* d_rng = (double*)out_direct(ctx, range, n * 8, SCR_OUT0);
        uint32_t* d_prim = (uint32_t*)out_direct(ctx, prim, n * 4, SCR_OUT1);
        launch_trace<false>(s, LidarBatchJob{{}, d_pos, d_rot, z_positive ? 1.0f : -1.0f, d_rng, d_prim}, (uint32_t)n);
        out_finish(ctx, range, d_rng, n * 8);
        out_finish(ctx, prim, d_prim, n * 4);
        finish(ctx, host_output(range) || host_output(prim), "crt_lidar_batch");
    });
}

int crt_lidar_grid(crt_scene* s, const crt_lidar_grid_desc* g, double* range, uint32_t* prim) {
    if (!s || !g) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(g->nx > 0 && g->ny > 0 && (uint64_t)g->nx * g->ny < (1ull << 31), CRT_ERR_INVALID, "bad beam grid");
        CRT_CHECK(range, CRT_ERR_INVALID, "null range buffer");
        CRT_CHECK(g->half_angle_x >= 0 && g->half_angle_x < 1.5 && g->half_angle_y >= 0 && g->half_angle_y < 1.5,
                  CRT_ERR_INVALID, "half angles must lie in [0, 1.5) rad");
        CRT_CUDA(cudaSetDevice(ctx->device));
        LidarGridJob J;
        for (int k = 0; k < 3; ++k) J.o[k] = g->position[k];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) J.rt[3 * a + b] = g->rotation[3 * b + a];
        J.zsign = g->z_positive ? 1.0 : -1.0;
        J.nx = g->nx;
        J.ny = g->ny;
        const uint32_t nt = g->nx + g->ny;
        double* d_tan = (double*)ctx_scratch(ctx, SCR_IN0, (size_t)nt * sizeof(double));
        k_tan_table<<<(nt + 255) / 256, 256, 0, ctx->stream>>>(d_tan, g->nx, g->ny, g->half_angle_x, g->half_angle_y);
        check_launch(ctx, "k_tan_table");
        J.tx = d_tan;
        J.ty = d_tan + g->nx;
        const size_t nb = (size_t)g->nx * g->ny;
        J.range = (double*)out_direct(ctx, range, nb * 8, SCR_OUT0);
        J.prim = (uint32_t*)out_direct(ctx, prim, nb * 4, SCR_OUT1);
        launch_trace<false>(s, J, tiles_items(g->nx, g->ny));
        out_finish(ctx, range, J.range, nb * 8);
        out_finish(ctx, prim, J.prim, nb * 4);
        finish(ctx, host_output(range) || host_output(prim), "crt_lidar_grid");
    });
}

}  // extern "C"
