// Solar radiation pressure: the sun-ray grid items shared by crt_srp (srp.cu) and the batched
// wavefront (render.cu, SRP requests riding in a wave's primary trace), and the host stages both run.
//
// Items are (attitude, 8 x 4 tile, lane) with each attitude's items padded to SRP_BLOCK_ITEMS.  A
// wave is a range of one request's items aligned to SRP_BLOCK_ITEMS: whole attitudes, or a part of
// one attitude.  Force and torque are summed per block of SRP_BLOCK_ITEMS items into a partial slot
// indexed by the block's place in the request (not in the wave), in a fixed order, so the totals do
// not depend on how the items are cut into waves.
#pragma once

#include "common.cuh"
#include "trace.cuh"

#include <vector>

constexpr uint32_t SRP_BLOCK_ITEMS = 1024;

struct SrpAtt {
    float org[3];   // centre of cell (0, 0)
    float du[3];    // step to the next cell in x
    float dv[3];    // step to the next cell in y
    float dir[3];   // -s_b
    float E0;       // flux * cell area
    float pad;
};

struct SrpWave {
    const SrpAtt* att;
    uint32_t G, tiles_x, tiles;
    uint32_t items_per_att;   // multiple of SRP_BLOCK_ITEMS
    uint64_t i0;              // first item of the wave
    uint32_t a0, r0;          // i0 = a0 * items_per_att + r0
    uint32_t multi;           // the wave holds whole attitudes (r0 == 0) rather than part of one
    float box_lo[3], box_hi[3];   // scene box, enlarged (srp_plan): rays that miss it are not traced
    float4* hit;              // per wave item: t, u, v, slot (primary segment: written for hits only)
    uint32_t* hitmask;        // primary segment: one bit per wave item that hit (zeroed before the trace)
    float4* st_o;             // continuing ray: origin, power
    float4* st_d;             // continuing ray: direction, triangle it leaves
    uint8_t* alive;           // continuing ray present
};

// attitude of wave item i (32-bit arithmetic: a wave is whole attitudes or a part of one)
__device__ __forceinline__ uint32_t srp_att(const SrpWave& W, uint32_t i, uint32_t& local) {
    if (W.multi) {
        const uint32_t q = i / W.items_per_att;
        local = i - q * W.items_per_att;
        return W.a0 + q;
    }
    local = W.r0 + i;
    return W.a0;
}

__device__ __forceinline__ bool srp_item(const SrpWave& W, uint32_t i, uint32_t& a, uint32_t& px, uint32_t& py) {
    uint32_t local;
    a = srp_att(W, i, local);
    const uint32_t tile = local >> 5, lane = local & 31u;
    if (tile >= W.tiles) return false;
    px = (tile % W.tiles_x) * 8u + (lane & 7u);
    py = (tile / W.tiles_x) * 4u + (lane >> 3);
    return px < W.G && py < W.G;
}

// sun ray of wave item i: 1 to trace, 0 for a padding item, 2 for a ray that misses the enlarged
// scene box and so every triangle (resolved as a miss without a traversal: most of a grid around a
// spacecraft, whose 8-wide root test costs ~10x this one); the job-contract values of k_trace
__device__ __forceinline__ int srp_primary_ray(const SrpWave& W, uint32_t i, TRay& r) {
    uint32_t a, px, py;
    if (!srp_item(W, i, a, px, py)) return 0;
    const SrpAtt& P = W.att[a];
    r.o = f3(P.org[0] + px * P.du[0] + py * P.dv[0], P.org[1] + px * P.du[1] + py * P.dv[1],
             P.org[2] + px * P.du[2] + py * P.dv[2]);
    r.d = f3(P.dir[0], P.dir[1], P.dir[2]);
    r.tmin = 0.f;
    r.tmax = 3.402823466e38f;
    const float ix = safe_rcp(r.d.x), iy = safe_rcp(r.d.y), iz = safe_rcp(r.d.z);
    const float x0 = (W.box_lo[0] - r.o.x) * ix, x1 = (W.box_hi[0] - r.o.x) * ix;
    const float y0 = (W.box_lo[1] - r.o.y) * iy, y1 = (W.box_hi[1] - r.o.y) * iy;
    const float z0 = (W.box_lo[2] - r.o.z) * iz, z1 = (W.box_hi[2] - r.o.z) * iz;
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.f));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
    return tn <= tf ? 1 : 2;
}

// One request's attitude table and item geometry (host side)
struct SrpPlan {
    std::vector<SrpAtt> att;
    uint32_t G = 0, tiles_x = 0, tiles = 0;
    uint32_t nb = 0;                  // specular segments actually traced (0 when no entity reflects)
    uint64_t ipa = 0;                 // items per attitude (multiple of SRP_BLOCK_ITEMS)
    uint64_t total = 0;               // ipa * attitudes
    uint64_t blocks_per_att = 0;
    float inv_c = 0.f, cm[3] = {0.f, 0.f, 0.f};
    float box_lo[3] = {0.f, 0.f, 0.f}, box_hi[3] = {0.f, 0.f, 0.f};   // scene box + 1e-4 extent + 1e-5
    size_t natt = 0;                  // attitudes (att holds their table unless the caller keeps it)
    size_t n_att() const { return natt; }
};

// The attitude-independent frame of a request: unit sun direction (inertial), grid centre and
// half size, cell size and ray power.  srp_attitude turns one quaternion into its grid of rays.
struct SrpFrame {
    double si[3];
    double ctr[3];
    double Rb, h, E0;
};

// One wave's SRP range as the stage kernels read it from device memory (a batched wave's descriptor):
// the launches of a wave stay the same from wave to wave, so the wave can be replayed as one CUDA
// graph; the range they work on, and its request's constants, come from here.
struct SrpStage {
    SceneView sv;        // the request's scene
    SrpWave W;           // the range's items and per-item state
    double* partial;     // the request's partial sums (slot = block of the request)
    uint32_t n;          // items in the range (0: the wave has none)
    uint32_t nb;         // specular segments of the request
    uint32_t n_tris;
    float inv_c;
    float cm[3];
    uint32_t pad;
};

// Per-wave SRP state for waves of at most `cap` items: hits (16 B per item), continuation state when
// there are specular segments (33 B per item), then the primary segment's hit mask (1 bit per item).
constexpr size_t srp_mask_offset(uint64_t cap, uint32_t nb) {
    return ((size_t)cap * (nb ? 49 : 16) + 255) & ~size_t(255);
}
constexpr size_t srp_state_bytes(uint64_t cap, uint32_t nb) {
    return srp_mask_offset(cap, nb) + ((((size_t)cap + 31) / 32 * 4 + 255) & ~size_t(255)) + 256;
}
inline size_t srp_mask_bytes(uint64_t n) { return ((size_t)n + 31) / 32 * 4; }

// Primary-segment result of wave item i: hits are stored and flagged in the mask; misses leave both
__device__ __forceinline__ void srp_store_primary(const SrpWave& W, uint32_t i, const THit& h) {
    if (h.slot == CRT_MISS) return;
    W.hit[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
    atomicOr(W.hitmask + (i >> 5), 1u << (i & 31u));
}

// Validates an SRP request and builds its plan; quaternions may be host or device memory.  Throws
// CrtError.
void srp_plan(crt_scene* s, const crt_srp_desc* desc, const double* quats, size_t n_att, SrpPlan& P);
// The parts of srp_plan that need no attitude: validates desc and fills every field of P but the
// attitude table and count (natt = total = 0), and the frame F.  Allocates nothing.  Throws CrtError.
void srp_frame(crt_scene* s, const crt_srp_desc* desc, SrpPlan& P, SrpFrame& F);
// Sets P's attitude count (natt, total); throws when the call holds too many rays.
void srp_set_attitudes(SrpPlan& P, size_t n_att);
// Ray grid of one attitude (unit quaternion w, x, y, z rotating body vectors into the inertial
// frame; normalised here).  Throws CrtError for a zero or non-finite quaternion.
void srp_attitude(const SrpFrame& F, const double q[4], SrpAtt& out);
// Wave descriptor over `state` (room for `cap` items) for items [i0, i0 + n) of the request
// (d_att: its attitude table on the device)
// (state laid out for `layout_nb` specular segments, default P.nb: requests sharing one state buffer
// use the largest)
SrpWave srp_wave(const SrpPlan& P, const SrpAtt* d_att, char* state, uint64_t cap, uint64_t i0, uint64_t n,
                 int layout_nb = -1);
// Largest wave at most `cap` items long that starts at item i0: whole attitudes when one fits,
// else the rest of the current attitude
uint64_t srp_wave_items(const SrpPlan& P, uint64_t cap, uint64_t i0);
// After the primary segment's hits are in W.hit: its shade, then the specular segments (trace of
// the compacted continuation queue + shade).  bq: room for n entries; bcount: 2 counters.  Block b
// of the wave sums into partial slot W.i0 / SRP_BLOCK_ITEMS + b - partial_block0 (0: the request's
// whole partial array; the wave's first block: an array holding this wave's blocks only).
// trace_queue: work counter of the continuation traces (null: the context's scratch counter).
void srp_wave_stages(crt_context* ctx, const SceneView& sv, const SrpWave& W, uint32_t n, const SrpPlan& P,
                     double* partial, double* facet, uint32_t n_tris, uint32_t* bq, uint32_t* bcount,
                     uint64_t partial_block0 = 0, uint32_t* trace_queue = nullptr);
// The stage descriptor of items [W.i0, W.i0 + n) of a request (plan P, partial sums `partial`)
SrpStage srp_stage(const SceneView& sv, const SrpWave& W, uint32_t n, const SrpPlan& P, double* partial,
                   uint32_t n_tris);
// srp_wave_stages for the range in d_stage (device memory, filled before the launches run): launches
// nb_max specular segments over n_max items; segments and blocks beyond the range's own do nothing.
// No argument depends on the range, so the launches can be captured once and replayed per wave.
void srp_wave_stages_dev(crt_context* ctx, const SrpStage* d_stage, uint32_t n_max, uint32_t nb_max, uint32_t* bq,
                         uint32_t* bcount, uint32_t* trace_queue);
// Per-attitude force and torque from the request's partial sums (device outputs)
void srp_reduce(crt_context* ctx, const double* partial, const SrpPlan& P, double* force, double* torque);
