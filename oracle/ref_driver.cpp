// Driver around the reference's own headers (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/build_ref.py against the unmodified ceres-raytracer sources (include paths
// lib/, src/, src/crt/) into oracle/_ref/.  It exposes per-ray results the reference's Python
// module does not return: the closest-hit primitive index with t, u, v
// (bvh::ClosestPrimitiveIntersector, lib/bvh/primitive_intersectors.hpp:33-54), any-hit
// occlusion (AnyPrimitiveIntersector :58-76), and the float radiance of the path tracer before
// the uint8 quantisation (src/crt/do_render.hpp:65-116 calling unidirectional,
// src/crt/path_tracing/unidirectional.hpp:24-96).  Scenes are assembled exactly as
// BodyFixedGroup does (src/crt/rendering_body_fixed/body_fixed_group.hpp:45-89, ids 1..n as in
// src/pybind.cpp:107-127).  Used here only to produce the committed golden fixtures.
#include "crt/cameras/camera.hpp"
#include "crt/cameras/simple_camera.hpp"
#include "crt/lidars/lidar.hpp"
#include "crt/lidars/simple_lidar.hpp"
#include "crt/lights/light.hpp"
#include "crt/lights/point_light.hpp"
#include "crt/lights/area_light.hpp"
#include "crt/rendering_body_fixed/body_fixed_entity.hpp"
#include "crt/rendering_body_fixed/body_fixed_group.hpp"
#include "crt/rendering_dynamic/entity.hpp"
#include "crt/passes.hpp"

#include <cstring>
#include <limits>

using S = double;
using V3 = bvh::Vector3<S>;

struct RefScene {
    std::vector<Entity<S>*> ents;
    BodyFixedGroup<S>* group;
};

static void set_rot(RigidBody<S>& rb, const double* r) {
    S R[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = r[3 * i + j];
    rb.set_rotation(R);
}

extern "C" {

void* ref_scene_create(int n, const char** paths, const int* smooth, const double* colors, const double* scales,
                       const double* positions, const double* rotations) {
    auto* rs = new RefScene();
    for (int i = 0; i < n; ++i) {
        Color c(0);
        c[0] = (float)colors[3 * i]; c[1] = (float)colors[3 * i + 1]; c[2] = (float)colors[3 * i + 2];
        auto* e = new Entity<S>(paths[i], "obj", smooth[i] != 0, c);
        e->set_scale(scales[i]);
        e->set_position(V3(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]));
        set_rot(*e, rotations + 9 * i);
        e->set_id((uint32_t)(i + 1));
        rs->ents.push_back(e);
    }
    rs->group = new BodyFixedGroup<S>(rs->ents);
    return rs;
}

void ref_scene_destroy(void* h) {
    auto* rs = (RefScene*)h;
    delete rs->group;
    for (auto* e : rs->ents) delete e;
    delete rs;
}

size_t ref_num_tris(void* h) { return ((RefScene*)h)->group->triangles.size(); }

// p0, e1, e2, n, vn0, vn1, vn2 (21 doubles per triangle) in scene order
void ref_tris(void* h, double* out) {
    auto& tris = ((RefScene*)h)->group->triangles;
    for (size_t i = 0; i < tris.size(); ++i) {
        const auto& t = tris[i];
        const V3* v[7] = {&t.p0, &t.e1, &t.e2, &t.n, &t.vn0, &t.vn1, &t.vn2};
        for (int k = 0; k < 7; ++k)
            for (int c = 0; c < 3; ++c) out[21 * i + 3 * k + c] = (*v[k])[c];
    }
}

// rays: 8 doubles each (origin, direction, tmin, tmax)
void ref_trace_closest(void* h, const double* rays, size_t n, int64_t* prim, double* t, double* u, double* v) {
    auto* g = ((RefScene*)h)->group;
    auto* tri_data = g->triangles.data();
    bvh::ClosestPrimitiveIntersector<bvh::Bvh<S>, bvh::Triangle<S>, false> closest(g->bvh_cache, tri_data);
    bvh::SingleRayTraverser<bvh::Bvh<S>> trav(g->bvh_cache);
    for (size_t i = 0; i < n; ++i) {
        const double* q = rays + 8 * i;
        bvh::Ray<S> r(V3(q[0], q[1], q[2]), V3(q[3], q[4], q[5]), q[6], q[7]);
        auto hit = trav.traverse(r, closest);
        if (hit) {
            prim[i] = (int64_t)hit->primitive_index;
            t[i] = hit->intersection.t; u[i] = hit->intersection.u; v[i] = hit->intersection.v;
        } else {
            prim[i] = -1; t[i] = u[i] = v[i] = 0;
        }
    }
}

void ref_trace_any(void* h, const double* rays, size_t n, uint8_t* occluded) {
    auto* g = ((RefScene*)h)->group;
    auto* tri_data = g->triangles.data();
    bvh::AnyPrimitiveIntersector<bvh::Bvh<S>, bvh::Triangle<S>, false> any(g->bvh_cache, tri_data);
    bvh::SingleRayTraverser<bvh::Bvh<S>> trav(g->bvh_cache);
    for (size_t i = 0; i < n; ++i) {
        const double* q = rays + 8 * i;
        bvh::Ray<S> r(V3(q[0], q[1], q[2]), V3(q[3], q[4], q[5]), q[6], q[7]);
        occluded[i] = trav.traverse(r, any) ? 1 : 0;
    }
}

// Float radiance of the reference path tracer (single thread, deterministic under ref_shim.h).
// lights: per light 1 type (0 point, 1 area) + intensity + position[3] + rotation[9] + size[2] = 16 doubles.
// out: W*H*3 floats (running mean as do_render keeps it), out_m2: per-pixel sum of squared sample
// deviations (Welford) so the caller can form a Monte-Carlo standard error.
void ref_render(void* h, double focal, const double* res, const double* sensor, int z_positive, const double* cam_pos,
                const double* cam_rot, int n_lights, const double* lights, int min_samples, int max_samples,
                double noise_threshold, int num_bounces, float* out, float* out_m2) {
    auto* g = ((RefScene*)h)->group;
    S r2[2] = {res[0], res[1]}, s2[2] = {sensor[0], sensor[1]};
    std::unique_ptr<Camera<S>> cam = std::make_unique<SimpleCamera<S>>(focal, r2, s2, z_positive != 0);
    cam->set_position(V3(cam_pos[0], cam_pos[1], cam_pos[2]));
    set_rot(*cam, cam_rot);
    std::vector<std::unique_ptr<Light<S>>> ls;
    for (int l = 0; l < n_lights; ++l) {
        const double* q = lights + 16 * l;
        if (q[0] == 0) {
            auto pl = std::make_unique<PointLight<S>>(q[1]);
            pl->set_position(V3(q[2], q[3], q[4]));
            ls.push_back(std::move(pl));
        } else {
            S sz[2] = {q[14], q[15]};
            auto al = std::make_unique<AreaLight<S>>(q[1], sz);
            al->set_position(V3(q[2], q[3], q[4]));
            set_rot(*al, q + 5);
            ls.push_back(std::move(al));
        }
    }
    auto* tri_data = g->triangles.data();
    bvh::ClosestPrimitiveIntersector<bvh::Bvh<S>, bvh::Triangle<S>, false> closest(g->bvh_cache, tri_data);
    bvh::AnyPrimitiveIntersector<bvh::Bvh<S>, bvh::Triangle<S>, false> any(g->bvh_cache, tri_data);
    bvh::SingleRayTraverser<bvh::Bvh<S>> trav(g->bvh_cache);
    size_t W = (size_t)floor(res[0]), H = (size_t)floor(res[1]);
    std::minstd_rand eng(12345);
    std::uniform_real_distribution<S> distr(-0.5, 0.5);
    for (size_t j = 0; j < H; ++j)
        for (size_t i = 0; i < W; ++i) {
            Color pix(0);
            Color m2(0);
            for (int sample = 1; sample < max_samples + 1; ++sample) {
                auto a = distr(eng), b = distr(eng);
                bvh::Ray<S> ray = max_samples == 1 ? cam->pixel_to_ray(i, j) : cam->pixel_to_ray(i + a, j + b);
                Color L = unidirectional(ls, tri_data, closest, any, trav, ray, num_bounces);
                auto d = (L - pix) * (1.0f / sample);
                Color before = pix;
                pix += d;
                for (int c = 0; c < 3; ++c) m2[c] += (L[c] - before[c]) * (L[c] - pix[c]);
                if (sample >= min_samples && bvh::length(d) < noise_threshold) break;
            }
            for (int c = 0; c < 3; ++c) {
                out[3 * (j * W + i) + c] = pix[c];
                if (out_m2) out_m2[3 * (j * W + i) + c] = m2[c];
            }
        }
}

}  // extern "C"
