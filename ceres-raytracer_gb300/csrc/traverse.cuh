// Traversal of the 8-wide compressed BVH (device code).
//
// Semantics follow SingleRayTraverser (lib/bvh/single_ray_traverser.hpp:68-126) with
// Closest/AnyPrimitiveIntersector: every triangle whose test passes shrinks tmax (closest hit) or
// ends the traversal (any hit).  Leaves are intersected as soon as their parent node is visited
// (the reference's "eager" leaves); internal children are visited nearest-first by the octant
// order fixed at build time.  Node groups (base index, hit bits, slot mask) live on a per-thread
// stack whose first STACK_SMEM entries are in shared memory and the rest in local memory.  The
// triangle test is watertight (tri_test); the child-box test reads the node's planes as halves
// (WideNode), so the ray octant picks each axis's entry / exit row by address.
#pragma once

#include "common.cuh"
#include <cuda_fp16.h>

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

// barycentrics of a hit from tri_test's weights
__device__ __forceinline__ THit normalized(THit h, float det) {
    const float inv = 1.0f / det;
    h.u *= inv;
    h.v *= inv;
    return h;
}

// Plane c (0..3) of half a row (4 halves 256 + q / 4) as an exact float (one half-to-float
// conversion).  Plane distances are then fma(256 + q / 4, 4 s, a - 1024 s) with s = quantum / d: one
// conversion and one FFMA per plane, the node-constant offset folded into a - 1024 s, whose rounding
// adds at most 2^-24 (|a| + 2^10 |s|), well inside the build's one-quantum slack on every child box.
__device__ __forceinline__ float half_at2(const float2 r, int c) {
    const float w = (c >> 1) == 0 ? r.x : r.y;
    const __half2 h = *reinterpret_cast<const __half2*>(&w);
    return (c & 1) ? __high2float(h) : __low2float(h);
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
    // rows of the entry planes per axis (lo rows 2..4, hi rows 5..7; a negative direction enters at hi)
    const int offx = (oct & 1u) ? 3 : 0, offy = (oct & 2u) ? 3 : 0, offz = (oct & 4u) ? 3 : 0;
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
        const float4 w0 = __ldg(np), w1 = __ldg(np + 1);
        if (COUNT) st.nodes++;
        const uint32_t ew = __float_as_uint(w0.w);
        // 4 x quantum x 1/d per axis (the planes are stored as 256 + q / 4)
        const float sx4 = __uint_as_float((uint32_t)(((int)(int8_t)(ew & 0xFF) + 129) << 23)) * idir.x;
        const float sy4 = __uint_as_float((uint32_t)(((int)(int8_t)((ew >> 8) & 0xFF) + 129) << 23)) * idir.y;
        const float sz4 = __uint_as_float((uint32_t)(((int)(int8_t)((ew >> 16) & 0xFF) + 129) << 23)) * idir.z;
        const float ax = fmaf(-256.0f, sx4, (w0.x - ray.o.x) * idir.x);
        const float ay = fmaf(-256.0f, sy4, (w0.y - ray.o.y) * idir.y);
        const float az = fmaf(-256.0f, sz4, (w0.z - ray.o.z) * idir.z);
        const uint32_t imask = ew >> 24;
        const uint32_t meta0 = __float_as_uint(w1.z), meta1 = __float_as_uint(w1.w);
        // entry / exit planes per axis by the ray octant: the lo / hi rows swap by address; each half
        // of a row (children 0-3, 4-7) is loaded when its children are tested
        const float2* rp = reinterpret_cast<const float2*>(np);
        uint32_t hitmask = 0;
#pragma unroll
        for (int hlf = 0; hlf < 2; ++hlf) {
            const float2 xl = __ldg(rp + 2 * (2 + offx) + hlf), xh = __ldg(rp + 2 * (5 - offx) + hlf);
            const float2 yl = __ldg(rp + 2 * (3 + offy) + hlf), yh = __ldg(rp + 2 * (6 - offy) + hlf);
            const float2 zl = __ldg(rp + 2 * (4 + offz) + hlf), zh = __ldg(rp + 2 * (7 - offz) + hlf);
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                const int c = 4 * hlf + cc;
                const int k = c & 3;
                const float tx0 = fmaf(half_at2(xl, cc), sx4, ax), tx1 = fmaf(half_at2(xh, cc), sx4, ax);
                const float ty0 = fmaf(half_at2(yl, cc), sy4, ay), ty1 = fmaf(half_at2(yh, cc), sy4, ay);
                const float tz0 = fmaf(half_at2(zl, cc), sz4, az), tz1 = fmaf(half_at2(zh, cc), sz4, az);
                const float tmin = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, ray.tmin));
                const float tmax = fminf(fminf(tx1, ty1), fminf(tz1, ray.tmax));
                if (tmin <= tmax) {
                    const uint32_t meta = ((c < 4 ? meta0 : meta1) >> (8 * k)) & 0xFFu;
                    uint32_t shift = meta & 31u;
                    if ((imask >> c) & 1u) shift ^= oct;
                    hitmask |= (meta >> 5) << shift;
                }
            }
        }
        ngroup = make_uint2(__float_as_uint(w1.x), (hitmask & 0xFF000000u) | imask);
        tgroup = make_uint2(__float_as_uint(w1.y), hitmask & 0x00FFFFFFu);
    }
    return normalized(hit, hit_det);
}
