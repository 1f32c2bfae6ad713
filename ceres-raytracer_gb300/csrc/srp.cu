// Solar radiation pressure over parallel sun-ray grids (no counterpart in the reference; its README
// names the feature only).
//
// Model (flat plate, Montenbruck & Gill, Satellite Orbits, sec. 3.4): a ray of power E travelling
// along d that hits a facet with unit normal n facing the ray (cos = -d.n >= 0) transfers
//     dF = (E / c) [ (1 - rs) d - (2 rs cos + 2/3 rd) n ],   dT = (x - c_m) x dF,
// the facet absorbs (1 - rs - rd) E, and the specular part continues along d - 2 (d.n) n with power
// rs E for up to num_bounces further segments.  Facets are two-sided.  rs / rd come from the hit
// triangle's entity.
//
// Per attitude the sun direction is rotated into the body frame in FP64 (s_b = R(q)^T s_i); rays
// start on a grid x grid square of side 2 R_b (R_b = half diagonal of the scene box) centred on the
// box centre, 2 R_b + 1 upstream, one ray per cell centre, power flux * cell area.
//
// crt_srp runs as a wavefront on the shared persistent trace kernel (per-segment trace launches
// into per-ray hits, then k_srp_shade; see the section below).  crt_srp_static, which may not
// allocate, keeps the fused kernel k_srp: each persistent warp takes 16 tiles (8 x 4 rays) of one
// attitude per grab, lanes accumulate force and torque in FP64, the warp reduces them with
// shuffles and lane 0 writes the grab's partial sums to a slot indexed by the grab.
// In both, per-attitude totals are summed by k_srp_reduce in a fixed order (bitwise reproducible);
// facet powers are summed per facet within a warp (FP32, at most 32 terms) and added with FP64
// atomics (reproducible up to the order of additions); warps whose rays all missed skip that step.
#include "common.cuh"
#include "srp.cuh"
#include "trace.cuh"

#include <cmath>
#include <vector>

namespace {

constexpr uint32_t CHUNK = 16;   // tiles per work grab (at most)

struct SrpArgs {
    const SrpAtt* att;
    uint32_t G;
    uint32_t tiles;          // tiles per attitude
    uint32_t grabs_per_att;
    uint32_t chunk;          // tiles per grab
    uint32_t n_att;
    float inv_c;
    float cm[3];
    uint32_t nb;
    double* partial;         // n_att * grabs_per_att * 6
    double* facet;           // n_att * n_tris or null
    uint32_t n_tris;
};

template <bool COUNT>
__global__ void __launch_bounds__(CRT_TRACE_BLOCK) k_srp(SceneView sv, SrpArgs A, uint32_t* __restrict__ queue,
                                                         uint32_t* __restrict__ err,
                                                         unsigned long long* __restrict__ counters) {
    extern __shared__ uint2 sstack[];
    const int lane = threadIdx.x & 31;
    const uint32_t tiles_x = (A.G + 7) >> 3;
    const uint32_t total = A.n_att * A.grabs_per_att;
    TravStats st{0u, 0u};
    uint32_t nrays = 0;
    while (true) {
        uint32_t g = 0;
        if (lane == 0) g = atomicAdd(queue, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= total) break;
        const uint32_t a = g / A.grabs_per_att;
        const uint32_t t0 = (g % A.grabs_per_att) * A.chunk;
        const uint32_t t1 = min(t0 + A.chunk, A.tiles);
        const SrpAtt P = A.att[a];
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (uint32_t tile = t0; tile < t1; ++tile) {
            const uint32_t px = (tile % tiles_x) * 8u + (lane & 7), py = (tile / tiles_x) * 4u + (lane >> 3);
            bool alive = px < A.G && py < A.G;
            TRay r;
            r.o = f3(P.org[0] + px * P.du[0] + py * P.dv[0], P.org[1] + px * P.du[1] + py * P.dv[1],
                     P.org[2] + px * P.du[2] + py * P.dv[2]);
            r.d = f3(P.dir[0], P.dir[1], P.dir[2]);
            r.tmin = 0.f;
            r.tmax = 3.402823466e38f;
            float E = P.E0;
            for (uint32_t seg = 0; seg <= A.nb; ++seg) {
                THit h;
                h.slot = CRT_MISS;
                if (alive) {
                    h = traverse<false, COUNT>(sv, r, sstack + threadIdx.x, CRT_TRACE_BLOCK, st, err);
                    if (COUNT) ++nrays;
                    if (h.slot == CRT_MISS) alive = false;
                }
                __syncwarp();
                const bool hit = h.slot != CRT_MISS;
                float absorbed = 0.f;
                uint32_t key = 0xFFFFFFFFu;
                float3 n = f3(0.f, 0.f, 0.f), x = f3(0.f, 0.f, 0.f);
                float rs = 0.f;
                if (hit) {
                    const SurfacePoint sp = surface_point(sv, h);
                    const EntityDev& Ent = sv.entities[sp.entity];
                    rs = Ent.rho_s;
                    const float rd = Ent.rho_d;
                    n = sp.flat_n * -1.0f;                       // outward for counter-clockwise meshes
                    if (dot3(r.d, n) > 0.f) n = n * -1.0f;       // two-sided: face the incoming ray
                    const float cs = -dot3(r.d, n);
                    const float k1 = E * A.inv_c * (1.0f - rs);
                    const float k2 = E * A.inv_c * (2.0f * rs * cs + (2.0f / 3.0f) * rd);
                    const float3 dF = r.d * k1 - n * k2;
                    x = sp.x;
                    const float3 dT = cross3(x - f3(A.cm[0], A.cm[1], A.cm[2]), dF);
                    acc[0] += dF.x; acc[1] += dF.y; acc[2] += dF.z;
                    acc[3] += dT.x; acc[4] += dT.y; acc[5] += dT.z;
                    absorbed = (1.0f - rs - rd) * E;
                    key = __ldg(sv.leaf_prim + h.slot);
                }
                if (A.facet && __any_sync(0xffffffffu, hit)) {
                    // warp-aggregated facet power: lanes hitting the same facet add once.  The group
                    // sum (at most 32 terms) is FP32, the accumulation across groups FP64 atomics.
                    const uint32_t peers = __match_any_sync(0xffffffffu, key);
                    float sum = absorbed;
                    if (__any_sync(0xffffffffu, hit && peers != (1u << lane))) {
                        sum = 0.f;
#pragma unroll 8
                        for (int j = 0; j < 32; ++j) {
                            const float v = __shfl_sync(0xffffffffu, absorbed, j);
                            if ((peers >> j) & 1u) sum += v;
                        }
                    }
                    if (hit && lane == __ffs(peers) - 1) atomicAdd(&A.facet[(size_t)a * A.n_tris + key], (double)sum);
                }
                if (hit) {
                    if (rs > 0.f && seg < A.nb) {
                        const float3 dn = r.d - n * (2.0f * dot3(r.d, n));
                        const float m = fmaxf(fabsf(x.x), fmaxf(fabsf(x.y), fabsf(x.z)));
                        int e;
                        frexpf(m, &e);
                        const float off = fmaxf(1e-5f, ldexpf(1.0f, e - 24 + 3));
                        r.o = x + n * off;
                        r.d = dn;
                        r.tmin = 0.f;
                        r.tmax = 3.402823466e38f;
                        r.skip = h.slot;
                        E *= rs;
                    } else {
                        alive = false;
                    }
                }
                if (!__any_sync(0xffffffffu, alive)) break;
            }
        }
        for (int k = 0; k < 6; ++k)
            for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (lane == 0)
            for (int k = 0; k < 6; ++k) A.partial[6ull * g + k] = acc[k];
    }
    if (COUNT) {
        unsigned long long a = nrays, b = st.nodes, c = st.tris;
        for (int o = 16; o; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if (lane == 0) {
            atomicAdd(counters + 0, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
        }
    }
}

// one block per attitude, fixed-order tree sum of its partials
__global__ void k_srp_reduce(const double* __restrict__ partial, uint32_t grabs_per_att, double* __restrict__ force,
                             double* __restrict__ torque) {
    __shared__ double sh[256][6];
    const uint32_t a = blockIdx.x;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t g = threadIdx.x; g < grabs_per_att; g += blockDim.x)
        for (int k = 0; k < 6; ++k) acc[k] += partial[6ull * ((size_t)a * grabs_per_att + g) + k];
    for (int k = 0; k < 6; ++k) sh[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 6; ++k) sh[threadIdx.x][k] += sh[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            force[3ull * a + k] = sh[0][k];
            torque[3ull * a + k] = sh[0][3 + k];
        }
    }
}

// ---------------------------------------------------------------- wavefront SRP (crt_srp)
// Items are (attitude, tile, lane) with each attitude's items padded to SRP_BLOCK_ITEMS; a wave is a
// range of items aligned to SRP_BLOCK_ITEMS.  Each segment is one trace launch (the persistent
// ray-queue kernel) writing per-item hits, then one shade launch in which block b sums the force and
// torque of items [b * SRP_BLOCK_ITEMS, (b + 1) * SRP_BLOCK_ITEMS) in a fixed order into partial slot
// b of the attitude.  Specular continuations stay at their item index, so every sum is independent
// of scheduling and the results are bitwise reproducible.
constexpr uint32_t SRP_SHADE_THREADS = 256;

struct SrpPrimaryJob : JobBase {
    SrpWave W;
    __device__ int ray(uint32_t i, TRay& r, Item&) const { return srp_primary_ray(W, i, r); }
    __device__ void write(const SceneView&, uint32_t i, const TRay&, const THit& h, const Item&) const {
        srp_store_primary(W, i, h);
    }
};

// continuing rays: a compacted queue of item indices (hits still land at the item's own slot)
struct SrpBounceJob {
    SrpWave W;
    const uint32_t* q;
    struct Item {
        uint32_t i;
    };
    __device__ __forceinline__ const SceneView& view(const SceneView& sv, const Item&) const { return sv; }
    __device__ bool ray(uint32_t k, TRay& r, Item& it) const {
        const uint32_t i = q[k];
        const float4 o = W.st_o[i], d = W.st_d[i];
        r.o = f3(o.x, o.y, o.z);
        r.d = f3(d.x, d.y, d.z);
        r.tmin = 0.f;
        r.tmax = 3.402823466e38f;
        r.skip = __float_as_uint(d.w);
        it.i = i;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t, const TRay&, const THit& h, const Item& it) const {
        W.hit[it.i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    }
};

// warp-aggregated append of one entry per participating lane
__device__ __forceinline__ uint32_t srp_append(uint32_t* counter) {
    const uint32_t mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

struct SrpShadeArgs {
    uint32_t n_items;         // items in the wave
    uint32_t seg, nb;
    float inv_c;
    float cm[3];
    double* partial;          // 6 per block of SRP_BLOCK_ITEMS items (global block index)
    double* facet;            // n_att * n_tris or null
    uint32_t n_tris;
    uint32_t* q_out;          // continuing items of the next segment
    uint32_t* q_count;
};

// Sums: each thread adds its (at most 4) rays in FP32, the warp tree is FP32 (at most 128 terms, so
// the rounding is below 1e-5 of the summed magnitudes), the 8 warps of a block and all blocks are
// summed in FP64, every step in a fixed order.  Blocks without a hit skip the reduction (GB300 runs
// FP64 at a small fraction of its FP32 rate, and most blocks of a sun grid miss the body).
template <bool FIRST>
__global__ void __launch_bounds__(SRP_SHADE_THREADS) k_srp_shade(SceneView sv, SrpWave W, SrpShadeArgs A) {
    __shared__ double red[SRP_SHADE_THREADS / 32][6];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool any_hit = false;
#pragma unroll 1
    for (uint32_t j = 0; j < SRP_BLOCK_ITEMS / SRP_SHADE_THREADS; ++j) {
        const uint32_t i = blockIdx.x * SRP_BLOCK_ITEMS + j * SRP_SHADE_THREADS + threadIdx.x;
        uint32_t a = 0, px = 0, py = 0, local = 0;
        bool alive = false;
        if (i < A.n_items) {
            if (FIRST) {   // only the hits of the primary segment are stored (hit mask)
                alive = srp_item(W, i, a, px, py) && ((W.hitmask[i >> 5] >> (i & 31u)) & 1u);
            } else {
                alive = W.alive[i] != 0;
                if (alive) a = srp_att(W, i, local);
            }
        }
        THit h;
        h.slot = CRT_MISS;
        float3 d = f3(0.f, 0.f, 0.f);
        float E = 0.f;
        if (alive) {
            const float4 hv = W.hit[i];
            h.t = hv.x;
            h.u = hv.y;
            h.v = hv.z;
            h.slot = __float_as_uint(hv.w);
            if (FIRST) {
                const SrpAtt& P = W.att[a];
                d = f3(P.dir[0], P.dir[1], P.dir[2]);
                E = P.E0;
            } else {
                const float4 o = W.st_o[i], dd = W.st_d[i];
                d = f3(dd.x, dd.y, dd.z);
                E = o.w;
            }
        }
        const bool hit = h.slot != CRT_MISS;
        any_hit |= hit;
        float absorbed = 0.f;
        uint32_t key = 0xFFFFFFFFu;
        bool cont = false;
        if (hit) {
            const SurfacePoint sp = surface_point(sv, h);
            const EntityDev& Ent = sv.entities[sp.entity];
            const float rs = Ent.rho_s, rd = Ent.rho_d;
            float3 n = sp.flat_n * -1.0f;                 // outward for counter-clockwise meshes
            if (dot3(d, n) > 0.f) n = n * -1.0f;          // two-sided: face the incoming ray
            const float cs = -dot3(d, n);
            const float k1 = E * A.inv_c * (1.0f - rs);
            const float k2 = E * A.inv_c * (2.0f * rs * cs + (2.0f / 3.0f) * rd);
            const float3 dF = d * k1 - n * k2;
            const float3 x = sp.x;
            const float3 dT = cross3(x - f3(A.cm[0], A.cm[1], A.cm[2]), dF);
            acc[0] += dF.x; acc[1] += dF.y; acc[2] += dF.z;
            acc[3] += dT.x; acc[4] += dT.y; acc[5] += dT.z;
            absorbed = (1.0f - rs - rd) * E;
            key = __ldg(sv.leaf_prim + h.slot);
            if (rs > 0.f && A.seg < A.nb) {
                const float3 dn = d - n * (2.0f * dot3(d, n));
                const float m = fmaxf(fabsf(x.x), fmaxf(fabsf(x.y), fabsf(x.z)));
                int e;
                frexpf(m, &e);
                const float off = fmaxf(1e-5f, ldexpf(1.0f, e - 24 + 3));
                const float3 o = x + n * off;
                W.st_o[i] = make_float4(o.x, o.y, o.z, E * rs);
                W.st_d[i] = make_float4(dn.x, dn.y, dn.z, __uint_as_float(h.slot));
                cont = true;
                A.q_out[srp_append(A.q_count)] = i;
            }
        }
        if (A.nb > A.seg && i < A.n_items && (FIRST || alive)) W.alive[i] = cont ? 1 : 0;
        if (A.facet && __any_sync(0xffffffffu, hit)) {
            // warp-aggregated facet power (FP32 group sums of at most 32 terms, FP64 atomics)
            const uint32_t peers = __match_any_sync(0xffffffffu, key);
            float sum = absorbed;
            if (__any_sync(0xffffffffu, hit && peers != (1u << lane))) {
                sum = 0.f;
#pragma unroll 8
                for (int q = 0; q < 32; ++q) {
                    const float v = __shfl_sync(0xffffffffu, absorbed, q);
                    if ((peers >> q) & 1u) sum += v;
                }
            }
            if (hit && lane == (uint32_t)(__ffs(peers) - 1))
                atomicAdd(&A.facet[(size_t)a * A.n_tris + key], (double)sum);
        }
    }
    const size_t slot = (size_t)(W.i0 / SRP_BLOCK_ITEMS + blockIdx.x) * 6;
    if (!__syncthreads_or(any_hit)) {
        if (FIRST && threadIdx.x < 6) A.partial[slot + threadIdx.x] = 0.0;
        return;
    }
    for (int k = 0; k < 6; ++k)
        for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (lane == 0)
        for (int k = 0; k < 6; ++k) red[warp][k] = (double)acc[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (uint32_t w = 0; w < SRP_SHADE_THREADS / 32; ++w) t += red[w][threadIdx.x];
        A.partial[slot + threadIdx.x] = FIRST ? t : A.partial[slot + threadIdx.x] + t;
    }
}

}  // namespace

void srp_plan(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att, SrpPlan& P) {
    CRT_CHECK(n_att == 0 || quats, CRT_ERR_INVALID, "null buffer");
    CRT_CHECK(desc->grid > 0 && desc->grid <= 32768, CRT_ERR_INVALID, "grid must be in [1, 32768]");
    CRT_CHECK(desc->c > 0 && std::isfinite(desc->flux), CRT_ERR_INVALID, "bad flux or speed of light");
    CRT_CHECK(desc->num_bounces <= 16, CRT_ERR_INVALID, "at most 16 specular bounces");
    const double sl = std::sqrt(desc->sun_dir_inertial[0] * desc->sun_dir_inertial[0] +
                                desc->sun_dir_inertial[1] * desc->sun_dir_inertial[1] +
                                desc->sun_dir_inertial[2] * desc->sun_dir_inertial[2]);
    CRT_CHECK(sl > 0 && std::isfinite(sl), CRT_ERR_INVALID, "sun direction must be a non-zero vector");
    const double si[3] = {desc->sun_dir_inertial[0] / sl, desc->sun_dir_inertial[1] / sl,
                          desc->sun_dir_inertial[2] / sl};
    // body-frame box of the scene
    double lo[3], hi[3], ctr[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = s->bounds[k];
        hi[k] = s->bounds[3 + k];
        ctr[k] = 0.5 * (lo[k] + hi[k]);
    }
    const double Rb = 0.5 * std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                      (hi[2] - lo[2]) * (hi[2] - lo[2]));
    const uint32_t G = desc->grid;
    const double h = 2.0 * Rb / G;
    std::vector<double> hq(4 * n_att);
    if (n_att && is_device_ptr(quats)) {
        CRT_CUDA(cudaMemcpy(hq.data(), quats, 32 * n_att, cudaMemcpyDeviceToHost));
    } else {
        std::copy(quats, quats + 4 * n_att, hq.begin());
    }
    P.att.resize(n_att);
    for (size_t a = 0; a < n_att; ++a) {
        double w = hq[4 * a], x = hq[4 * a + 1], y = hq[4 * a + 2], z = hq[4 * a + 3];
        const double qn = std::sqrt(w * w + x * x + y * y + z * z);
        CRT_CHECK(qn > 0 && std::isfinite(qn), CRT_ERR_INVALID, "attitude quaternion must be non-zero");
        w /= qn; x /= qn; y /= qn; z /= qn;
        // R(q) maps body vectors into the inertial frame; s_b = R^T s_i
        const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                             2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                             2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
        double sb[3];
        for (int k = 0; k < 3; ++k) sb[k] = R[k] * si[0] + R[3 + k] * si[1] + R[6 + k] * si[2];
        // grid basis perpendicular to s_b (same construction as the oracle)
        double ax[3] = {1, 0, 0};
        if (std::fabs(sb[0]) >= 0.9) { ax[0] = 0; ax[1] = 1; }
        double e1[3] = {sb[1] * ax[2] - sb[2] * ax[1], sb[2] * ax[0] - sb[0] * ax[2], sb[0] * ax[1] - sb[1] * ax[0]};
        const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (int k = 0; k < 3; ++k) e1[k] /= l1;
        const double e2[3] = {sb[1] * e1[2] - sb[2] * e1[1], sb[2] * e1[0] - sb[0] * e1[2], sb[0] * e1[1] - sb[1] * e1[0]};
        for (int k = 0; k < 3; ++k) {
            const double o0 = ctr[k] + sb[k] * (2.0 * Rb + 1.0) + e1[k] * (-Rb + 0.5 * h) + e2[k] * (-Rb + 0.5 * h);
            P.att[a].org[k] = (float)o0;
            P.att[a].du[k] = (float)(e1[k] * h);
            P.att[a].dv[k] = (float)(e2[k] * h);
            P.att[a].dir[k] = (float)(-sb[k]);
        }
        P.att[a].E0 = (float)(desc->flux * h * h);
        P.att[a].pad = 0.f;
    }
    P.G = G;
    P.tiles_x = (G + 7) / 8;
    P.tiles = P.tiles_x * ((G + 3) / 4);
    P.ipa = ((uint64_t)P.tiles * 32 + SRP_BLOCK_ITEMS - 1) / SRP_BLOCK_ITEMS * SRP_BLOCK_ITEMS;
    P.total = P.ipa * n_att;
    P.blocks_per_att = P.ipa / SRP_BLOCK_ITEMS;
    CRT_CHECK(P.blocks_per_att * n_att < (1ull << 31), CRT_ERR_INVALID, "too many rays in one call");
    // specular continuations only when some entity reflects specularly
    bool specular = false;
    for (const EntityDev& E : s->host_entities) specular |= E.rho_s > 0.f;
    P.nb = specular ? desc->num_bounces : 0u;
    P.inv_c = (float)(1.0 / desc->c);
    for (int k = 0; k < 3; ++k) P.cm[k] = (float)desc->center_of_mass[k];
    // rays that miss this box miss every triangle by far more than the FP32 error of the tests
    const double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    const double m = 1e-4 * ext + 1e-5;
    for (int k = 0; k < 3; ++k) {
        P.box_lo[k] = (float)(lo[k] - m - 1e-6 * std::fabs(lo[k]));
        P.box_hi[k] = (float)(hi[k] + m + 1e-6 * std::fabs(hi[k]));
    }
}

uint64_t srp_wave_items(const SrpPlan& P, uint64_t cap, uint64_t i0) {
    const uint64_t att_per_wave = P.ipa <= cap ? cap / P.ipa : 0;
    return att_per_wave ? std::min<uint64_t>(att_per_wave * P.ipa, P.total - i0)
                        : std::min<uint64_t>(cap, P.ipa - i0 % P.ipa);
}

SrpWave srp_wave(const SrpPlan& P, const SrpAtt* d_att, char* state, uint64_t cap, uint64_t i0, uint64_t n) {
    SrpWave W;
    W.att = d_att;
    W.G = P.G;
    W.tiles_x = P.tiles_x;
    W.tiles = P.tiles;
    W.items_per_att = (uint32_t)P.ipa;
    W.i0 = i0;
    W.a0 = (uint32_t)(i0 / P.ipa);
    W.r0 = (uint32_t)(i0 % P.ipa);
    W.multi = (W.r0 == 0 && n >= P.ipa) ? 1u : 0u;   // whole attitudes, else a part of one
    for (int k = 0; k < 3; ++k) {
        W.box_lo[k] = P.box_lo[k];
        W.box_hi[k] = P.box_hi[k];
    }
    W.hit = (float4*)state;
    W.hitmask = (uint32_t*)(state + srp_mask_offset(cap, P.nb));
    W.st_o = P.nb ? (float4*)(state + cap * 16) : nullptr;
    W.st_d = P.nb ? (float4*)(state + cap * 32) : nullptr;
    W.alive = P.nb ? (uint8_t*)(state + cap * 48) : nullptr;
    return W;
}

void srp_wave_stages(crt_context* ctx, const SceneView& sv, const SrpWave& W, uint32_t n, const SrpPlan& P,
                     double* partial, double* facet, uint32_t n_tris, uint32_t* bq, uint32_t* bcount) {
    cudaStream_t st = ctx->stream;
    SrpShadeArgs A;
    A.n_items = n;
    A.nb = P.nb;
    A.inv_c = P.inv_c;
    for (int k = 0; k < 3; ++k) A.cm[k] = P.cm[k];
    A.partial = partial;
    A.facet = facet;
    A.n_tris = n_tris;
    A.q_out = bq;
    const uint32_t nblk = (n + SRP_BLOCK_ITEMS - 1) / SRP_BLOCK_ITEMS;
    for (uint32_t seg = 0; seg <= P.nb; ++seg) {
        A.seg = seg;
        A.q_count = bcount + (seg & 1);          // filled by this segment's shade
        if (seg < P.nb) CRT_CUDA(cudaMemsetAsync(A.q_count, 0, sizeof(uint32_t), st));
        if (seg == 0) {
            k_srp_shade<true><<<nblk, SRP_SHADE_THREADS, 0, st>>>(sv, W, A);
        } else {
            // the queue filled by the previous segment's shade; its count stays on the device
            SrpBounceJob J;
            J.W = W;
            J.q = bq;
            launch_trace<false>(ctx, sv, J, n, bcount + ((seg - 1) & 1));
            k_srp_shade<false><<<nblk, SRP_SHADE_THREADS, 0, st>>>(sv, W, A);
        }
        check_launch(ctx, "k_srp_shade");
    }
}

void srp_reduce(crt_context* ctx, const double* partial, const SrpPlan& P, double* force, double* torque) {
    if (!P.n_att()) return;
    k_srp_reduce<<<(uint32_t)P.n_att(), 256, 0, ctx->stream>>>(partial, (uint32_t)P.blocks_per_att, force, torque);
    check_launch(ctx, "k_srp_reduce");
}

// Runs on `ctx` (stream, scratch, error word), which may differ from the scene's own context on the
// same device (serving lanes).  Throws CrtError.
void srp_run(crt_context* ctx, crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att,
             double* force, double* torque, double* facet_power) {
    [&] {
        CRT_CHECK(n_att == 0 || (quats && force && torque), CRT_ERR_INVALID, "null buffer");
        CRT_CUDA(cudaSetDevice(ctx->device));
        SrpPlan P;
        srp_plan(s, desc, quats, n_att, P);
        if (!n_att) return;
        cudaStream_t st = ctx->stream;
        // a wave: whole attitudes, or a part of one attitude, of up to 2^24 items (about 50 bytes of
        // state each); always a multiple of the reduction block
        const uint64_t wave_cap = 1u << 24;
        const uint64_t wave_items = srp_wave_items(P, wave_cap, 0);
        SrpAtt* d_att = (SrpAtt*)ctx_scratch(ctx, SCR_IN1, sizeof(SrpAtt) * n_att);
        CRT_CUDA(cudaMemcpyAsync(d_att, P.att.data(), sizeof(SrpAtt) * n_att, cudaMemcpyHostToDevice, st));
        double* d_partial = (double*)ctx_scratch(ctx, SCR_WAVE3, sizeof(double) * 6 * P.blocks_per_att * n_att);
        char* state = (char*)ctx_scratch(ctx, SCR_WAVE4, srp_state_bytes(wave_items, P.nb));
        uint32_t* bq = P.nb ? (uint32_t*)ctx_scratch(ctx, SCR_WAVE5, wave_items * 4 + 256) : nullptr;
        uint32_t* bcount = (uint32_t*)ctx_scratch(ctx, SCR_WAVE6, 256);
        double* d_force = (double*)out_device(ctx, force, n_att * 24, SCR_OUT0);
        double* d_torque = (double*)out_device(ctx, torque, n_att * 24, SCR_OUT1);
        double* d_facet = facet_power ? (double*)out_device(ctx, facet_power, n_att * s->n_tris * 8, SCR_OUT2) : nullptr;
        if (d_facet) CRT_CUDA(cudaMemsetAsync(d_facet, 0, n_att * s->n_tris * 8, st));
        const SceneView sv = scene_view(s);
        for (uint64_t i0 = 0; i0 < P.total;) {
            const uint32_t n = (uint32_t)srp_wave_items(P, wave_cap, i0);
            const SrpWave W = srp_wave(P, d_att, state, wave_items, i0, n);
            i0 += n;
            // single 32-ray grabs keep the warps on a narrow band of the grid, so BVH nodes are reused
            // from L1/L2 (measured: larger grabs were slower on the 2M asteroid)
            SrpPrimaryJob J;
            J.W = W;
            CRT_CUDA(cudaMemsetAsync(W.hitmask, 0, srp_mask_bytes(n), st));
            launch_trace<false>(ctx, sv, J, n);
            srp_wave_stages(ctx, sv, W, n, P, d_partial, d_facet, (uint32_t)s->n_tris, bq, bcount);
        }
        srp_reduce(ctx, d_partial, P, d_force, d_torque);
        out_finish(ctx, force, d_force, n_att * 24);
        out_finish(ctx, torque, d_torque, n_att * 24);
        if (facet_power) out_finish(ctx, facet_power, d_facet, n_att * s->n_tris * 8);
        check_device_error(ctx, "crt_srp");
    }();
}

extern "C" int crt_srp(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att, double* force,
                       double* torque, double* facet_power) {
    if (!s || !desc) return CRT_ERR_INVALID;
    return crt_guard(s->ctx, [&] { srp_run(s->ctx, s, desc, quats, n_att, force, torque, facet_power); });
}

// ---------------------------------------------------------------- allocation-free variant
// crt_srp_static: the same force / torque computation with every piece of scratch (work counter,
// attitude table, per-chunk FP64 partial sums, staging of host outputs) in the file-scope device
// array below, so a call performs no device allocation.  It serves callers that must not allocate
// device memory after start-up: flight-dynamics or attitude-control loops with a fixed memory
// budget, and code that runs while another component owns the CUDA allocator.  Every GPU that loads
// the library holds this array until the process exits.
#define CRT_SRP_STATIC_BYTES (16u << 20)          // 16 MiB per device
#define CRT_SRP_STATIC_MAX_ATT 4096u              // attitudes per call
static __device__ __align__(256) unsigned char g_srp_static_scratch[CRT_SRP_STATIC_BYTES];

namespace {

constexpr size_t SS_COUNTER = 0;                                  // work counter (zeroed per launch)
constexpr size_t SS_ATT = 256;                                    // SrpAtt table
constexpr size_t SS_OUT = SS_ATT + sizeof(SrpAtt) * CRT_SRP_STATIC_MAX_ATT;    // force | torque staging
constexpr size_t SS_PART = (SS_OUT + 48ull * CRT_SRP_STATIC_MAX_ATT + 255) & ~size_t(255);
constexpr size_t SS_PART_BYTES = CRT_SRP_STATIC_BYTES - SS_PART;

std::mutex g_static_mu;
void* g_static_ptr[256] = {};

// Device address of the scratch array on the current device; resolved once per device.
void* static_scratch(int device) {
    CRT_CHECK(device >= 0 && device < 256, CRT_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[device]) {
        void* p = nullptr;
        CRT_CUDA(cudaGetSymbolAddress(&p, g_srp_static_scratch));
        g_static_ptr[device] = p;
    }
    return g_static_ptr[device];
}

}  // namespace

extern "C" int crt_srp_static(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att,
                              double* force, double* torque) {
    if (!s || !desc) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n_att == 0 || (quats && force && torque), CRT_ERR_INVALID, "null buffer");
        CRT_CHECK(n_att <= CRT_SRP_STATIC_MAX_ATT, CRT_ERR_INVALID,
                  "crt_srp_static: at most 4096 attitudes per call (static scratch limit)");
        CRT_CHECK(desc->grid > 0 && desc->grid <= 32768, CRT_ERR_INVALID, "grid must be in [1, 32768]");
        CRT_CHECK(desc->c > 0 && std::isfinite(desc->flux), CRT_ERR_INVALID, "bad flux or speed of light");
        CRT_CHECK(desc->num_bounces <= 16, CRT_ERR_INVALID, "at most 16 specular bounces");
        CRT_CHECK(!is_device_ptr(quats), CRT_ERR_INVALID, "crt_srp_static reads the quaternions from host memory");
        const uint32_t G = desc->grid;
        const uint32_t tiles = ((G + 7) / 8) * ((G + 3) / 4);
        const uint32_t gpa = (tiles + CHUNK - 1) / CHUNK;
        CRT_CHECK((size_t)gpa * 48 <= SS_PART_BYTES, CRT_ERR_INVALID,
                  "crt_srp_static: grid too large for the 16 MiB static scratch (one attitude's partial sums "
                  "must fit; grid <= 11585)");
        if (!n_att) return;
        CRT_CUDA(cudaSetDevice(ctx->device));
        char* base = (char*)static_scratch(ctx->device);
        uint32_t* queue = (uint32_t*)(base + SS_COUNTER);
        SrpAtt* d_att = (SrpAtt*)(base + SS_ATT);
        double* d_out = (double*)(base + SS_OUT);
        double* d_partial = (double*)(base + SS_PART);
        cudaStream_t st = ctx->stream;

        const double sl = std::sqrt(desc->sun_dir_inertial[0] * desc->sun_dir_inertial[0] +
                                    desc->sun_dir_inertial[1] * desc->sun_dir_inertial[1] +
                                    desc->sun_dir_inertial[2] * desc->sun_dir_inertial[2]);
        CRT_CHECK(sl > 0 && std::isfinite(sl), CRT_ERR_INVALID, "sun direction must be a non-zero vector");
        const double si[3] = {desc->sun_dir_inertial[0] / sl, desc->sun_dir_inertial[1] / sl,
                              desc->sun_dir_inertial[2] / sl};
        double ctr[3], ext2 = 0;
        for (int k = 0; k < 3; ++k) {
            ctr[k] = 0.5 * ((double)s->bounds[k] + (double)s->bounds[3 + k]);
            const double e = (double)s->bounds[3 + k] - (double)s->bounds[k];
            ext2 += e * e;
        }
        const double Rb = 0.5 * std::sqrt(ext2);
        const double h = 2.0 * Rb / G;
        // attitude table: computed on the host in chunks held on the stack, copied into the scratch
        SrpAtt chunk[64];
        for (size_t a0 = 0; a0 < n_att; a0 += 64) {
            const size_t na = std::min<size_t>(64, n_att - a0);
            for (size_t j = 0; j < na; ++j) {
                const double* q = quats + 4 * (a0 + j);
                double w = q[0], x = q[1], y = q[2], z = q[3];
                const double qn = std::sqrt(w * w + x * x + y * y + z * z);
                CRT_CHECK(qn > 0 && std::isfinite(qn), CRT_ERR_INVALID, "attitude quaternion must be non-zero");
                w /= qn; x /= qn; y /= qn; z /= qn;
                const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                                     2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                                     2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
                double sb[3];
                for (int k = 0; k < 3; ++k) sb[k] = R[k] * si[0] + R[3 + k] * si[1] + R[6 + k] * si[2];
                double ax[3] = {1, 0, 0};
                if (std::fabs(sb[0]) >= 0.9) { ax[0] = 0; ax[1] = 1; }
                double e1[3] = {sb[1] * ax[2] - sb[2] * ax[1], sb[2] * ax[0] - sb[0] * ax[2],
                                sb[0] * ax[1] - sb[1] * ax[0]};
                const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
                for (int k = 0; k < 3; ++k) e1[k] /= l1;
                const double e2[3] = {sb[1] * e1[2] - sb[2] * e1[1], sb[2] * e1[0] - sb[0] * e1[2],
                                      sb[0] * e1[1] - sb[1] * e1[0]};
                for (int k = 0; k < 3; ++k) {
                    const double o0 = ctr[k] + sb[k] * (2.0 * Rb + 1.0) + e1[k] * (-Rb + 0.5 * h) + e2[k] * (-Rb + 0.5 * h);
                    chunk[j].org[k] = (float)o0;
                    chunk[j].du[k] = (float)(e1[k] * h);
                    chunk[j].dv[k] = (float)(e2[k] * h);
                    chunk[j].dir[k] = (float)(-sb[k]);
                }
                chunk[j].E0 = (float)(desc->flux * h * h);
                chunk[j].pad = 0.f;
            }
            CRT_CUDA(cudaMemcpyAsync(d_att + a0, chunk, sizeof(SrpAtt) * na, cudaMemcpyHostToDevice, st));
            CRT_CUDA(cudaStreamSynchronize(st));   // the stack chunk is reused for the next attitudes
        }
        const bool host_out = !is_device_ptr(force) || !is_device_ptr(torque);
        double* f_out = host_out ? d_out : force;
        double* t_out = host_out ? d_out + 3 * CRT_SRP_STATIC_MAX_ATT : torque;
        const size_t att_per_launch = std::max<size_t>(1, std::min<size_t>(n_att, SS_PART_BYTES / (48ull * gpa)));
        const size_t smem = (size_t)CRT_STACK_SMEM * CRT_TRACE_BLOCK * sizeof(uint2);
        const int grid = occupancy_grid(ctx, ctx->counting ? (const void*)k_srp<true> : (const void*)k_srp<false>,
                                        CRT_TRACE_BLOCK, smem);
        const SceneView sv = scene_view(s);
        for (size_t a0 = 0; a0 < n_att; a0 += att_per_launch) {
            const size_t na = std::min(att_per_launch, n_att - a0);
            SrpArgs A;
            A.att = d_att + a0;
            A.G = G;
            A.tiles = tiles;
            A.grabs_per_att = gpa;
            A.chunk = CHUNK;
            A.n_att = (uint32_t)na;
            A.inv_c = (float)(1.0 / desc->c);
            for (int k = 0; k < 3; ++k) A.cm[k] = (float)desc->center_of_mass[k];
            A.nb = desc->num_bounces;
            A.partial = d_partial;
            A.facet = nullptr;
            A.n_tris = (uint32_t)s->n_tris;
            CRT_CUDA(cudaMemsetAsync(queue, 0, sizeof(uint32_t), st));   // the counter must start at zero
            if (ctx->counting)
                k_srp<true><<<grid, CRT_TRACE_BLOCK, smem, st>>>(sv, A, queue, ctx->d_error, ctx->d_counters);
            else
                k_srp<false><<<grid, CRT_TRACE_BLOCK, smem, st>>>(sv, A, queue, ctx->d_error, ctx->d_counters);
            check_launch(ctx, "k_srp");
            k_srp_reduce<<<(uint32_t)na, 256, 0, st>>>(d_partial, gpa, f_out + 3 * a0, t_out + 3 * a0);
            check_launch(ctx, "k_srp_reduce");
        }
        if (host_out) {
            CRT_CUDA(cudaMemcpyAsync(force, f_out, n_att * 24, cudaMemcpyDeviceToHost, st));
            CRT_CUDA(cudaMemcpyAsync(torque, t_out, n_att * 24, cudaMemcpyDeviceToHost, st));
            check_device_error(ctx, "crt_srp_static");
        }
    });
}
