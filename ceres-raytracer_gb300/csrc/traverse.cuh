// Traversal of the 8-wide compressed BVH (device code).
//
// Semantics follow SingleRayTraverser (lib/bvh/single_ray_traverser.hpp:68-126) with
// Closest/AnyPrimitiveIntersector: every triangle whose test passes shrinks tmax (closest hit) or
// ends the traversal (any hit).  Leaves are intersected as soon as their parent node is visited
// (the reference's "eager" leaves); internal children are visited nearest-first by the octant
// order fixed at build time.  Node groups (base index, hit bits, slot mask) live on a per-thread
// stack whose first STACK_SMEM entries are in shared memory and the rest in local memory.
#pragma once

#include "common.cuh"

#ifndef CRT_STACK_SMEM
#define CRT_STACK_SMEM 8
#endif
#define CRT_STACK_TOTAL 64   // > wide-tree depth bound (binary depth <= 62 with index tie-breaks)

struct SceneView {
    const WideNode* __restrict__ nodes;
    const float4* __restrict__ tris;
    const uint32_t* __restrict__ leaf_prim;
    const float4* __restrict__ leaf_vn;
    const uint32_t* __restrict__ leaf_entity;
    const EntityDev* __restrict__ entities;
    uint32_t n_tris;
};

struct TravStats {
    uint32_t nodes, tris;
};

// 32768 + (byte k of w) as an exact float: the byte lands in bits 8..15 of the mantissa of 2^15
// (result bytes {0x00, w_k, 0x00, 0x47}).  Plane distances are then fma(32768 + b, s, a - 32768 s):
// one PRMT and one FFMA per plane, with the node-constant offset folded into a - 32768 s.  Its
// rounding adds at most 2^-24 (|a| + 2^15 |s|), i.e. the size of the existing rounding of a plus
// 0.002 quantum, well inside the build's one-quantum slack on every child box.
__device__ __forceinline__ float byte_f15(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x47000000u, 0x7404u | ((uint32_t)k << 4)));
}

// barycentrics of a hit from tri_test's weights
__device__ __forceinline__ THit normalized(THit h, float det) {
    const float inv = 1.0f / det;
    h.u *= inv;
    h.v *= inv;
    return h;
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ THit traverse(const SceneView& sv, TRay ray, uint2* __restrict__ sstack, int sstride,
                                         TravStats& st, uint32_t* __restrict__ err) {
    THit hit;
    hit.slot = CRT_MISS;
    hit.t = hit.u = hit.v = 0.f;
    // octant from the sign bits, as NodeIntersector does with std::signbit (node_intersectors.hpp:25-30):
    // -0.0 counts as negative, consistent with safe_rcp(-0.0) < 0
    const uint32_t oct = (__float_as_uint(ray.d.x) >> 31) | ((__float_as_uint(ray.d.y) >> 31) << 1) |
                         ((__float_as_uint(ray.d.z) >> 31) << 2);
    const float3 idir = f3(safe_rcp(ray.d.x), safe_rcp(ray.d.y), safe_rcp(ray.d.z));
    TShear shear = make_shear(ray.d);
    shear.ox = shear_proj(ray.o, shear.bx);
    shear.oy = shear_proj(ray.o, shear.by);
    uint2 lstack[CRT_STACK_TOTAL - CRT_STACK_SMEM];
    int sp = 0;
    // root = slot 0 of a virtual parent whose children start at node 0
    uint2 ngroup = make_uint2(0u, (1u << (24u + oct)) | 1u);
    float hit_det = 1.0f;   // weight sum of the hit's barycentrics (tri_test)
    uint2 tgroup = make_uint2(0u, 0u);
    while (true) {
        // ---- leaf triangles of the last visited node
        while (tgroup.y) {
            const int b = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1;
            const uint32_t slot = tgroup.x + (uint32_t)b;
            if (slot == ray.skip) continue;
            const float4* tp = sv.tris + 3ull * slot;
            const float4 a = __ldg(tp), bb = __ldg(tp + 1), c = __ldg(tp + 2);
            if (COUNT) st.tris++;
            float t, wv, ww, det;
            if (tri_test(a, bb, c, ray, shear, t, wv, ww, det)) {
                hit.t = t;
                hit.u = wv;
                hit.v = ww;
                hit_det = det;
                hit.slot = slot;
                if (ANY) return normalized(hit, hit_det);
                ray.tmax = t;
            }
        }
        // ---- next internal node
        if (ngroup.y <= 0x00FFFFFFu) {
            if (sp == 0) break;
            --sp;
            ngroup = sp < CRT_STACK_SMEM ? sstack[sp * sstride] : lstack[sp - CRT_STACK_SMEM];
        }
        const uint32_t bit = 31u - __clz(ngroup.y);
        const uint32_t cslot = (bit - 24u) ^ oct;
        const uint32_t pmask = ngroup.y & 0xFFu;
        const uint32_t node = ngroup.x + __popc(pmask & ((1u << cslot) - 1u));
        ngroup.y &= ~(1u << bit);
        if (ngroup.y > 0x00FFFFFFu) {
            if (sp < CRT_STACK_SMEM) sstack[sp * sstride] = ngroup;
            else if (sp < CRT_STACK_TOTAL) lstack[sp - CRT_STACK_SMEM] = ngroup;
            else {
                atomicOr(err, (uint32_t)DEVERR_STACK_OVERFLOW);
                return normalized(hit, hit_det);
            }
            ++sp;
        }
        // ---- visit: test the 8 quantised child boxes
        const float4* np = reinterpret_cast<const float4*>(sv.nodes + node);
        const float4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
        if (COUNT) st.nodes++;
        const uint32_t ew = __float_as_uint(w0.w);
        const float sx = __uint_as_float((uint32_t)(((int)(int8_t)(ew & 0xFF) + 127) << 23)) * idir.x;
        const float sy = __uint_as_float((uint32_t)(((int)(int8_t)((ew >> 8) & 0xFF) + 127) << 23)) * idir.y;
        const float sz = __uint_as_float((uint32_t)(((int)(int8_t)((ew >> 16) & 0xFF) + 127) << 23)) * idir.z;
        const float ax = fmaf(-32768.0f, sx, (w0.x - ray.o.x) * idir.x);
        const float ay = fmaf(-32768.0f, sy, (w0.y - ray.o.y) * idir.y);
        const float az = fmaf(-32768.0f, sz, (w0.z - ray.o.z) * idir.z);
        const uint32_t imask = ew >> 24;
        // entry / exit planes per axis depend on the ray octant
        uint32_t xlo0 = __float_as_uint(w2.x), xlo1 = __float_as_uint(w2.y);
        uint32_t ylo0 = __float_as_uint(w2.z), ylo1 = __float_as_uint(w2.w);
        uint32_t zlo0 = __float_as_uint(w3.x), zlo1 = __float_as_uint(w3.y);
        uint32_t xhi0 = __float_as_uint(w3.z), xhi1 = __float_as_uint(w3.w);
        uint32_t yhi0 = __float_as_uint(w4.x), yhi1 = __float_as_uint(w4.y);
        uint32_t zhi0 = __float_as_uint(w4.z), zhi1 = __float_as_uint(w4.w);
        if (oct & 1u) { uint32_t t0 = xlo0, t1 = xlo1; xlo0 = xhi0; xlo1 = xhi1; xhi0 = t0; xhi1 = t1; }
        if (oct & 2u) { uint32_t t0 = ylo0, t1 = ylo1; ylo0 = yhi0; ylo1 = yhi1; yhi0 = t0; yhi1 = t1; }
        if (oct & 4u) { uint32_t t0 = zlo0, t1 = zlo1; zlo0 = zhi0; zlo1 = zhi1; zhi0 = t0; zhi1 = t1; }
        const uint32_t meta0 = __float_as_uint(w1.z), meta1 = __float_as_uint(w1.w);
        uint32_t hitmask = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int k = c & 3;
            const uint32_t xl = c < 4 ? xlo0 : xlo1, xh = c < 4 ? xhi0 : xhi1;
            const uint32_t yl = c < 4 ? ylo0 : ylo1, yh = c < 4 ? yhi0 : yhi1;
            const uint32_t zl = c < 4 ? zlo0 : zlo1, zh = c < 4 ? zhi0 : zhi1;
            const float tx0 = fmaf(byte_f15(xl, k), sx, ax), tx1 = fmaf(byte_f15(xh, k), sx, ax);
            const float ty0 = fmaf(byte_f15(yl, k), sy, ay), ty1 = fmaf(byte_f15(yh, k), sy, ay);
            const float tz0 = fmaf(byte_f15(zl, k), sz, az), tz1 = fmaf(byte_f15(zh, k), sz, az);
            const float tmin = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, ray.tmin));
            const float tmax = fminf(fminf(tx1, ty1), fminf(tz1, ray.tmax));
            if (tmin <= tmax) {
                const uint32_t meta = ((c < 4 ? meta0 : meta1) >> (8 * k)) & 0xFFu;
                uint32_t shift = meta & 31u;
                if ((imask >> c) & 1u) shift ^= oct;
                hitmask |= (meta >> 5) << shift;
            }
        }
        ngroup = make_uint2(__float_as_uint(w1.x), (hitmask & 0xFF000000u) | imask);
        tgroup = make_uint2(__float_as_uint(w1.y), hitmask & 0x00FFFFFFu);
    }
    return normalized(hit, hit_det);
}
