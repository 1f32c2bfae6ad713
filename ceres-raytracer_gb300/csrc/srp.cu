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
// into per-ray hits, then k_srp_shade; see the section below); crt_srp_static runs the same stages
// with its scratch in a static device array.  Per-attitude totals are summed from per-block partial
// sums in a fixed order (bitwise reproducible); facet powers are summed per facet within a warp (FP32,
// at most 32 terms) and added with FP64 atomics (reproducible up to the order of additions); warps
// whose rays all missed skip that step.
#include "common.cuh"
#include "srp.cuh"
#include "trace.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

// Per-attitude totals from the partial sums of its blocks, in a fixed order: thread t of a 256-thread
// block adds blocks t, t + 256, t + 512, ... in increasing order, then a shared-memory tree sums the
// 256 thread totals.  k_srp_reduce does both for whole attitudes; k_srp_fold runs the first step over
// the blocks of one wave (a part of one attitude) into a running per-thread total and k_srp_tree the
// second, so an attitude summed wave by wave gets the same additions in the same order.
constexpr uint32_t SRP_REDUCE_THREADS = 256;

__device__ __forceinline__ void srp_tree_store(double (*sh)[6], const double acc[6], double* __restrict__ force,
                                               double* __restrict__ torque) {
    for (int k = 0; k < 6; ++k) sh[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int s = SRP_REDUCE_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 6; ++k) sh[threadIdx.x][k] += sh[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            force[k] = sh[0][k];
            torque[k] = sh[0][3 + k];
        }
    }
}

// one block per attitude
__global__ void __launch_bounds__(SRP_REDUCE_THREADS) k_srp_reduce(const double* __restrict__ partial,
                                                                  uint32_t blocks_per_att, double* __restrict__ force,
                                                                  double* __restrict__ torque) {
    __shared__ double sh[SRP_REDUCE_THREADS][6];
    const uint32_t a = blockIdx.x;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t g = threadIdx.x; g < blocks_per_att; g += SRP_REDUCE_THREADS)
        for (int k = 0; k < 6; ++k) acc[k] += partial[6ull * ((size_t)a * blocks_per_att + g) + k];
    srp_tree_store(sh, acc, force + 3ull * a, torque + 3ull * a);
}

// blocks [block0, block0 + nblk) of one attitude, whose partials start at `partial`, into the
// running thread totals `run` (SRP_REDUCE_THREADS x 6, zeroed before the attitude's first wave)
__global__ void __launch_bounds__(SRP_REDUCE_THREADS) k_srp_fold(const double* __restrict__ partial, uint64_t block0,
                                                                uint32_t nblk, double* __restrict__ run) {
    double acc[6];
    for (int k = 0; k < 6; ++k) acc[k] = run[6 * threadIdx.x + k];
    uint64_t g = block0 + ((threadIdx.x + SRP_REDUCE_THREADS - block0 % SRP_REDUCE_THREADS) % SRP_REDUCE_THREADS);
    for (; g < block0 + nblk; g += SRP_REDUCE_THREADS)
        for (int k = 0; k < 6; ++k) acc[k] += partial[6ull * (g - block0) + k];
    for (int k = 0; k < 6; ++k) run[6 * threadIdx.x + k] = acc[k];
}

__global__ void __launch_bounds__(SRP_REDUCE_THREADS) k_srp_tree(const double* __restrict__ run,
                                                                double* __restrict__ force,
                                                                double* __restrict__ torque) {
    __shared__ double sh[SRP_REDUCE_THREADS][6];
    double acc[6];
    for (int k = 0; k < 6; ++k) acc[k] = run[6 * threadIdx.x + k];
    srp_tree_store(sh, acc, force, torque);
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
    double* partial;          // 6 per block of SRP_BLOCK_ITEMS items (the request's block index - block0)
    uint64_t block0;
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
__device__ __forceinline__ void srp_shade(const SceneView& sv, const SrpWave& W, const SrpShadeArgs& A) {
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
    const size_t slot = (size_t)(W.i0 / SRP_BLOCK_ITEMS + blockIdx.x - A.block0) * 6;
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

template <bool FIRST>
__global__ void __launch_bounds__(SRP_SHADE_THREADS) k_srp_shade(SceneView sv, SrpWave W, SrpShadeArgs A) {
    srp_shade<FIRST>(sv, W, A);
}

// the same, for the range of a device stage descriptor (blocks past its items, or segments past its
// request's, return at once: the condition is uniform over the block)
template <bool FIRST>
__global__ void __launch_bounds__(SRP_SHADE_THREADS) k_srp_shade_dev(const SrpStage* __restrict__ S, uint32_t seg,
                                                                    uint32_t* q_out, uint32_t* q_count) {
    const uint32_t n = S->n, nb = S->nb;
    if (seg > nb || blockIdx.x * SRP_BLOCK_ITEMS >= n) return;
    SrpShadeArgs A;
    A.n_items = n;
    A.seg = seg;
    A.nb = nb;
    A.inv_c = S->inv_c;
    for (int k = 0; k < 3; ++k) A.cm[k] = S->cm[k];
    A.partial = S->partial;
    A.block0 = 0;
    A.facet = nullptr;
    A.n_tris = S->n_tris;
    A.q_out = q_out;
    A.q_count = q_count;
    const SceneView sv = S->sv;
    const SrpWave W = S->W;
    srp_shade<FIRST>(sv, W, A);
}

// continuing rays of a device stage descriptor's range
struct SrpBounceJobDev {
    const SrpStage* S;
    const uint32_t* q;
    struct Item {
        uint32_t i;
    };
    __device__ __forceinline__ SceneView view(const SceneView&, const Item&) const { return S->sv; }
    __device__ bool ray(uint32_t k, TRay& r, Item& it) const {
        const uint32_t i = q[k];
        const float4 o = S->W.st_o[i], d = S->W.st_d[i];
        r.o = f3(o.x, o.y, o.z);
        r.d = f3(d.x, d.y, d.z);
        r.tmin = 0.f;
        r.tmax = 3.402823466e38f;
        r.skip = __float_as_uint(d.w);
        it.i = i;
        return true;
    }
    __device__ void write(const SceneView&, uint32_t, const TRay&, const THit& h, const Item& it) const {
        S->W.hit[it.i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    }
};

}  // namespace

void srp_frame(crt_scene* s, const crt_srp_desc* desc, SrpPlan& P, SrpFrame& F) {
    CRT_CHECK(desc->grid > 0 && desc->grid <= 32768, CRT_ERR_INVALID, "grid must be in [1, 32768]");
    CRT_CHECK(desc->c > 0 && std::isfinite(desc->flux), CRT_ERR_INVALID, "bad flux or speed of light");
    CRT_CHECK(desc->num_bounces <= 16, CRT_ERR_INVALID, "at most 16 specular bounces");
    const double sl = std::sqrt(desc->sun_dir_inertial[0] * desc->sun_dir_inertial[0] +
                                desc->sun_dir_inertial[1] * desc->sun_dir_inertial[1] +
                                desc->sun_dir_inertial[2] * desc->sun_dir_inertial[2]);
    CRT_CHECK(sl > 0 && std::isfinite(sl), CRT_ERR_INVALID, "sun direction must be a non-zero vector");
    for (int k = 0; k < 3; ++k) F.si[k] = desc->sun_dir_inertial[k] / sl;
    // body-frame box of the scene
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = s->bounds[k];
        hi[k] = s->bounds[3 + k];
        F.ctr[k] = 0.5 * (lo[k] + hi[k]);
    }
    F.Rb = 0.5 * std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                           (hi[2] - lo[2]) * (hi[2] - lo[2]));
    const uint32_t G = desc->grid;
    F.h = 2.0 * F.Rb / G;
    F.E0 = desc->flux * F.h * F.h;
    P.G = G;
    P.tiles_x = (G + 7) / 8;
    P.tiles = P.tiles_x * ((G + 3) / 4);
    P.ipa = ((uint64_t)P.tiles * 32 + SRP_BLOCK_ITEMS - 1) / SRP_BLOCK_ITEMS * SRP_BLOCK_ITEMS;
    P.blocks_per_att = P.ipa / SRP_BLOCK_ITEMS;
    P.natt = 0;
    P.total = 0;
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

void srp_set_attitudes(SrpPlan& P, size_t n_att) {
    CRT_CHECK(P.blocks_per_att * n_att < (1ull << 31), CRT_ERR_INVALID, "too many rays in one call");
    P.natt = n_att;
    P.total = P.ipa * n_att;
}

void srp_attitude(const SrpFrame& F, const double q[4], SrpAtt& out) {
    double w = q[0], x = q[1], y = q[2], z = q[3];
    const double qn = std::sqrt(w * w + x * x + y * y + z * z);
    CRT_CHECK(qn > 0 && std::isfinite(qn), CRT_ERR_INVALID, "attitude quaternion must be non-zero");
    w /= qn; x /= qn; y /= qn; z /= qn;
    // R(q) maps body vectors into the inertial frame; s_b = R^T s_i
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
    const double* si = F.si;
    double sb[3];
    for (int k = 0; k < 3; ++k) sb[k] = R[k] * si[0] + R[3 + k] * si[1] + R[6 + k] * si[2];
    // grid basis perpendicular to s_b (same construction as the oracle)
    double ax[3] = {1, 0, 0};
    if (std::fabs(sb[0]) >= 0.9) { ax[0] = 0; ax[1] = 1; }
    double e1[3] = {sb[1] * ax[2] - sb[2] * ax[1], sb[2] * ax[0] - sb[0] * ax[2], sb[0] * ax[1] - sb[1] * ax[0]};
    const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int k = 0; k < 3; ++k) e1[k] /= l1;
    const double e2[3] = {sb[1] * e1[2] - sb[2] * e1[1], sb[2] * e1[0] - sb[0] * e1[2], sb[0] * e1[1] - sb[1] * e1[0]};
    const double Rb = F.Rb, h = F.h;
    for (int k = 0; k < 3; ++k) {
        const double o0 = F.ctr[k] + sb[k] * (2.0 * Rb + 1.0) + e1[k] * (-Rb + 0.5 * h) + e2[k] * (-Rb + 0.5 * h);
        out.org[k] = (float)o0;
        out.du[k] = (float)(e1[k] * h);
        out.dv[k] = (float)(e2[k] * h);
        out.dir[k] = (float)(-sb[k]);
    }
    out.E0 = (float)F.E0;
    out.pad = 0.f;
}

void srp_plan(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att, SrpPlan& P) {
    CRT_CHECK(n_att == 0 || quats, CRT_ERR_INVALID, "null buffer");
    SrpFrame F;
    srp_frame(s, desc, P, F);
    std::vector<double> hq(4 * n_att);
    if (n_att && is_device_ptr(quats)) {
        CRT_CUDA(cudaMemcpy(hq.data(), quats, 32 * n_att, cudaMemcpyDeviceToHost));
    } else {
        std::copy(quats, quats + 4 * n_att, hq.begin());
    }
    P.att.resize(n_att);
    for (size_t a = 0; a < n_att; ++a) srp_attitude(F, hq.data() + 4 * a, P.att[a]);
    srp_set_attitudes(P, n_att);
}

uint64_t srp_wave_items(const SrpPlan& P, uint64_t cap, uint64_t i0) {
    const uint64_t att_per_wave = P.ipa <= cap ? cap / P.ipa : 0;
    return att_per_wave ? std::min<uint64_t>(att_per_wave * P.ipa, P.total - i0)
                        : std::min<uint64_t>(cap, P.ipa - i0 % P.ipa);
}

SrpWave srp_wave(const SrpPlan& P, const SrpAtt* d_att, char* state, uint64_t cap, uint64_t i0, uint64_t n,
                 int layout_nb) {
    const uint32_t nb = layout_nb < 0 ? P.nb : (uint32_t)layout_nb;
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
    W.hitmask = (uint32_t*)(state + srp_mask_offset(cap, nb));
    W.st_o = nb ? (float4*)(state + cap * 16) : nullptr;
    W.st_d = nb ? (float4*)(state + cap * 32) : nullptr;
    W.alive = nb ? (uint8_t*)(state + cap * 48) : nullptr;
    return W;
}

void srp_wave_stages(crt_context* ctx, const SceneView& sv, const SrpWave& W, uint32_t n, const SrpPlan& P,
                     double* partial, double* facet, uint32_t n_tris, uint32_t* bq, uint32_t* bcount,
                     uint64_t partial_block0, uint32_t* trace_queue) {
    cudaStream_t st = ctx->stream;
    SrpShadeArgs A;
    A.n_items = n;
    A.nb = P.nb;
    A.inv_c = P.inv_c;
    for (int k = 0; k < 3; ++k) A.cm[k] = P.cm[k];
    A.partial = partial;
    A.block0 = partial_block0;
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
            launch_trace<false>(ctx, sv, J, n, bcount + ((seg - 1) & 1), trace_queue);
            k_srp_shade<false><<<nblk, SRP_SHADE_THREADS, 0, st>>>(sv, W, A);
        }
        check_launch(ctx, "k_srp_shade");
    }
}

SrpStage srp_stage(const SceneView& sv, const SrpWave& W, uint32_t n, const SrpPlan& P, double* partial,
                   uint32_t n_tris) {
    SrpStage S;
    std::memset(&S, 0, sizeof(S));
    S.sv = sv;
    S.W = W;
    S.partial = partial;
    S.n = n;
    S.nb = P.nb;
    S.n_tris = n_tris;
    S.inv_c = P.inv_c;
    for (int k = 0; k < 3; ++k) S.cm[k] = P.cm[k];
    return S;
}

void srp_wave_stages_dev(crt_context* ctx, const SrpStage* d_stage, uint32_t n_max, uint32_t nb_max, uint32_t* bq,
                         uint32_t* bcount, uint32_t* trace_queue) {
    cudaStream_t st = ctx->stream;
    const uint32_t nblk = std::max<uint32_t>(1, (n_max + SRP_BLOCK_ITEMS - 1) / SRP_BLOCK_ITEMS);
    for (uint32_t seg = 0; seg <= nb_max; ++seg) {
        uint32_t* q_count = bcount + (seg & 1);   // filled by this segment's shade
        if (seg < nb_max) CRT_CUDA(cudaMemsetAsync(q_count, 0, sizeof(uint32_t), st));
        if (seg == 0) {
            k_srp_shade_dev<true><<<nblk, SRP_SHADE_THREADS, 0, st>>>(d_stage, 0, bq, q_count);
        } else {
            SrpBounceJobDev J;
            J.S = d_stage;
            J.q = bq;
            launch_trace<false>(ctx, SceneView{}, J, n_max, bcount + ((seg - 1) & 1), trace_queue);
            k_srp_shade_dev<false><<<nblk, SRP_SHADE_THREADS, 0, st>>>(d_stage, seg, bq, q_count);
        }
        check_launch(ctx, "k_srp_shade");
    }
}

void srp_reduce(crt_context* ctx, const double* partial, const SrpPlan& P, double* force, double* torque) {
    if (!P.n_att()) return;
    k_srp_reduce<<<(uint32_t)P.n_att(), SRP_REDUCE_THREADS, 0, ctx->stream>>>(partial, (uint32_t)P.blocks_per_att,
                                                                             force, torque);
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
// crt_srp_static: the same force and torque as crt_srp, from the same wavefront stages, with every
// piece of scratch in the file-scope device array below, so that a call allocates no memory.  It
// serves callers that must not allocate device memory once they run: flight-dynamics or attitude
// loops that evaluate radiation pressure every integration step under a fixed memory budget, and
// components embedded in a host application that owns the CUDA allocator.  Every GPU that loads the
// library holds this array until the process exits.
//
// Layout: work counters, the attitude table and the staging of host outputs, then the state of one
// wave of at most SS_WAVE items (per-item hits and continuation rays, hit mask, continuation queue)
// and the partial sums of that wave's blocks.  Waves hold whole attitudes when an attitude has at
// most SS_WAVE items (their totals are reduced right after the wave); a larger attitude runs as
// several waves whose block sums are folded into running per-thread totals (k_srp_fold) and summed
// by k_srp_tree after its last wave.  Either way every addition happens in the order crt_srp uses,
// so the results are bitwise equal to crt_srp's.
#define CRT_SRP_STATIC_BYTES (64u << 20)          // 64 MiB per device
#define CRT_SRP_STATIC_MAX_ATT 4096u              // attitudes per call
static __device__ __align__(256) unsigned char g_srp_static_scratch[CRT_SRP_STATIC_BYTES];

namespace {

constexpr uint64_t SS_WAVE = 1u << 20;                            // items per wave
constexpr size_t ss_align(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t SS_QUEUE = 0;                                    // trace work counter
constexpr size_t SS_BCOUNT = 128;                                 // 2 continuation-queue counters
constexpr size_t SS_ATT = 256;                                    // SrpAtt table
constexpr size_t SS_OUT = ss_align(SS_ATT + sizeof(SrpAtt) * CRT_SRP_STATIC_MAX_ATT);   // force | torque staging
constexpr size_t SS_RUN = ss_align(SS_OUT + 48ull * CRT_SRP_STATIC_MAX_ATT);          // running totals 256 x 6
constexpr size_t SS_PART = ss_align(SS_RUN + 6ull * 8 * SRP_REDUCE_THREADS);          // one wave's block sums
constexpr size_t SS_BQ = ss_align(SS_PART + 48ull * (SS_WAVE / SRP_BLOCK_ITEMS));      // continuation queue
constexpr size_t SS_STATE = ss_align(SS_BQ + 4ull * SS_WAVE + 256);                   // wave state
static_assert(SS_WAVE % SRP_BLOCK_ITEMS == 0, "waves hold whole reduction blocks");

std::mutex g_static_mu;
void* g_static_ptr[256] = {};

// Device address of the scratch array on `device` (which must be current); resolved once per device.
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

// One output: written on the device directly, or staged in the scratch and copied to host memory.
struct StaticOut {
    double* user;
    double* dev;
    bool host;
};

}  // namespace

extern "C" int crt_srp_static(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att,
                              double* force, double* torque) {
    if (!s || !desc) return CRT_ERR_INVALID;
    crt_context* ctx = s->ctx;
    return crt_guard(ctx, [&] {
        CRT_CHECK(n_att == 0 || (quats && force && torque), CRT_ERR_INVALID, "null buffer");
        CRT_CHECK(n_att <= CRT_SRP_STATIC_MAX_ATT, CRT_ERR_INVALID,
                  "crt_srp_static: at most 4096 attitudes per call (static scratch limit)");
        SrpPlan P;   // its attitude table stays empty: the attitudes go to the static array
        SrpFrame F;
        srp_frame(s, desc, P, F);
        static_assert(srp_state_bytes(SS_WAVE, 1) <= CRT_SRP_STATIC_BYTES - SS_STATE, "static scratch too small");
        if (!n_att) return;
        CRT_CUDA(cudaSetDevice(ctx->device));
        char* base = (char*)static_scratch(ctx->device);
        uint32_t* queue = (uint32_t*)(base + SS_QUEUE);
        uint32_t* bcount = (uint32_t*)(base + SS_BCOUNT);
        SrpAtt* d_att = (SrpAtt*)(base + SS_ATT);
        double* run = (double*)(base + SS_RUN);
        double* d_partial = (double*)(base + SS_PART);
        uint32_t* bq = (uint32_t*)(base + SS_BQ);
        char* state = base + SS_STATE;
        cudaStream_t st = ctx->stream;

        // attitude table: computed on the host in chunks held on the stack, copied into the scratch;
        // quaternions in device memory are read back chunk by chunk
        const bool dev_q = is_device_ptr(quats);
        for (size_t a0 = 0; a0 < n_att; a0 += 64) {
            const size_t na = std::min<size_t>(64, n_att - a0);
            double qh[4 * 64];
            SrpAtt chunk[64];
            if (dev_q) CRT_CUDA(cudaMemcpy(qh, quats + 4 * a0, 32 * na, cudaMemcpyDeviceToHost));
            else std::copy(quats + 4 * a0, quats + 4 * (a0 + na), qh);
            for (size_t j = 0; j < na; ++j) srp_attitude(F, qh + 4 * j, chunk[j]);
            CRT_CUDA(cudaMemcpyAsync(d_att + a0, chunk, sizeof(SrpAtt) * na, cudaMemcpyHostToDevice, st));
            CRT_CUDA(cudaStreamSynchronize(st));   // the stack chunk is reused for the next attitudes
        }
        StaticOut out[2] = {{force, nullptr, !is_device_ptr(force)}, {torque, nullptr, !is_device_ptr(torque)}};
        for (int k = 0; k < 2; ++k)
            out[k].dev = out[k].host ? (double*)(base + SS_OUT) + 3 * CRT_SRP_STATIC_MAX_ATT * k : out[k].user;

        const SceneView sv = scene_view(s);
        // whole attitudes per wave when they fit, else one attitude over several waves
        const size_t att_per_wave = P.ipa <= SS_WAVE ? (size_t)(SS_WAVE / P.ipa) : 1;
        for (size_t a0 = 0; a0 < n_att; a0 += att_per_wave) {
            const size_t na = std::min(att_per_wave, n_att - a0);
            SrpPlan G = P;   // the group of attitudes [a0, a0 + na) as a request of its own
            srp_set_attitudes(G, na);
            const bool split = G.total > SS_WAVE;
            if (split) CRT_CUDA(cudaMemsetAsync(run, 0, 6 * 8 * SRP_REDUCE_THREADS, st));
            for (uint64_t i0 = 0; i0 < G.total;) {
                const uint32_t n = (uint32_t)srp_wave_items(G, SS_WAVE, i0);
                const SrpWave W = srp_wave(G, d_att + a0, state, SS_WAVE, i0, n);
                SrpPrimaryJob J;
                J.W = W;
                CRT_CUDA(cudaMemsetAsync(W.hitmask, 0, srp_mask_bytes(n), st));
                launch_trace<false>(ctx, sv, J, n, nullptr, queue);
                // block sums of this wave only: slot = (block of the attitude group) - (wave's first block)
                const uint64_t block0 = i0 / SRP_BLOCK_ITEMS;
                srp_wave_stages(ctx, sv, W, n, G, d_partial, nullptr, (uint32_t)s->n_tris, bq, bcount, block0, queue);
                if (split) {
                    k_srp_fold<<<1, SRP_REDUCE_THREADS, 0, st>>>(d_partial, block0, n / SRP_BLOCK_ITEMS, run);
                    check_launch(ctx, "k_srp_fold");
                }
                i0 += n;
            }
            if (split) {
                k_srp_tree<<<1, SRP_REDUCE_THREADS, 0, st>>>(run, out[0].dev + 3 * a0, out[1].dev + 3 * a0);
                check_launch(ctx, "k_srp_tree");
            } else {
                srp_reduce(ctx, d_partial, G, out[0].dev + 3 * a0, out[1].dev + 3 * a0);
            }
        }
        for (int k = 0; k < 2; ++k)
            if (out[k].host)
                CRT_CUDA(cudaMemcpyAsync(out[k].user, out[k].dev, n_att * 24, cudaMemcpyDeviceToHost, st));
        check_device_error(ctx, "crt_srp_static");
    });
}
