/* CPU oracle for the CRT ray-query path.  TEST INFRASTRUCTURE ONLY (see crt_oracle.h).
 *
 * FP64 restatement of the reference code paths; every function cites the reference
 * file:line it follows (paths relative to the ceres-raytracer source tree).  Compiled with
 * -ffp-contract=off so that products and sums round exactly as written, which is also how the
 * reference rounds when built without -march=native.
 *
 * The BVH here is a binned-SAH binary tree.  Closest-hit and any-hit results do not depend on
 * the tree (only the order in which exact ties are met does), so a different builder than the
 * reference's SweepSahBuilder (lib/bvh/sweep_sah_builder.hpp:43) yields the same answers; the
 * traversal itself restates SingleRayTraverser (lib/bvh/single_ray_traverser.hpp:68-126).
 */
#include "crt_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y, z; } v3;
static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
/* bvh::dot (lib/bvh/vector.hpp:133-139): left-to-right sum */
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* bvh::cross (vector.hpp:161-169) */
static inline v3 cross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline double length(v3 a) { return sqrt(dot(a, a)); }
/* bvh::normalize (vector.hpp:147-152): multiply by the reciprocal length */
static inline v3 normalize(v3 a) { double inv = 1.0 / length(a); return scl(a, inv); }
static inline double comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

/* transform.hpp:22-28 rotate(): R * v */
static inline v3 rotate(v3 v, const double* R) {
    return mk(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
              R[6] * v.x + R[7] * v.y + R[8] * v.z);
}
/* simple_camera.hpp:72-75: R^T * v */
static inline v3 rotate_t(v3 v, const double* R) {
    return mk(R[0] * v.x + R[3] * v.y + R[6] * v.z, R[1] * v.x + R[4] * v.y + R[7] * v.z,
              R[2] * v.x + R[5] * v.y + R[8] * v.z);
}

/* bvh::Triangle<double> (lib/bvh/triangle.hpp:21-60): p0, e1 = p0 - p1, e2 = p2 - p0,
 * n = cross(e1, e2) (left-handed, i.e. inward for counter-clockwise outward meshes). */
typedef struct { v3 p0, e1, e2, n, vn0, vn1, vn2; } tri_t;

static inline void tri_set(tri_t* t, v3 p0, v3 p1, v3 p2) {  /* update_vertices, triangle.hpp:50-55 */
    t->p0 = p0;
    t->e1 = sub(p0, p1);
    t->e2 = sub(p2, p0);
    t->n = cross(t->e1, t->e2);
}
static inline v3 tri_p1(const tri_t* t) { return sub(t->p0, t->e1); }  /* triangle.hpp:81 */
static inline v3 tri_p2(const tri_t* t) { return add(t->p0, t->e2); }  /* triangle.hpp:82 */

typedef struct {   /* Bvh<double>::Node (lib/bvh/bvh.hpp:26-31): siblings adjacent, root at 0 */
    double b[6];   /* xmin, xmax, ymin, ymax, zmin, zmax */
    uint32_t count; /* 0 => inner node */
    uint32_t first; /* first child (inner) or first index into prim_idx (leaf) */
} node_t;

typedef struct { uint32_t smooth; uint32_t id; float color[3]; double rho_s, rho_d; } ent_t;

struct oracle_scene {
    size_t n;
    tri_t* tris;
    uint32_t* tri_ent;
    ent_t* ents;
    uint32_t n_ents;
    node_t* nodes;
    size_t n_nodes;
    uint32_t* prim_idx;
    double* flat;   /* p0, e1, e2, n per triangle for the test harness */
};

/* ------------------------------------------------------------------ scene assembly
 * render.hpp:21-31 / body_fixed_group.hpp:47-56: per entity copy its triangles, then
 * resize_triangles, rotate_triangles, translate_triangles (transform.hpp:43-85), then append. */
static void transform_entity(const oracle_entity* e, tri_t* out) {
    for (size_t i = 0; i < e->n_tris; ++i) {
        const float* q = e->tri_xyz + 9 * i;
        tri_t t;
        tri_set(&t, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
        if (e->tri_vn) {
            const double* n = e->tri_vn + 9 * i;
            t.vn0 = mk(n[0], n[1], n[2]);
            t.vn1 = mk(n[3], n[4], n[5]);
            t.vn2 = mk(n[6], n[7], n[8]);
        } else {
            t.vn0 = t.vn1 = t.vn2 = mk(0, 0, 0);
        }
        /* resize_triangles (transform.hpp:43-54) */
        v3 p0 = scl(t.p0, e->scale), p1 = scl(tri_p1(&t), e->scale), p2 = scl(tri_p2(&t), e->scale);
        tri_set(&t, p0, p1, p2);
        /* rotate_triangles (transform.hpp:67-84) */
        p0 = rotate(t.p0, e->rotation);
        p1 = rotate(tri_p1(&t), e->rotation);
        p2 = rotate(tri_p2(&t), e->rotation);
        t.vn0 = rotate(t.vn0, e->rotation);
        t.vn1 = rotate(t.vn1, e->rotation);
        t.vn2 = rotate(t.vn2, e->rotation);
        tri_set(&t, p0, p1, p2);
        /* translate_triangles (transform.hpp:56-65) */
        v3 pos = mk(e->position[0], e->position[1], e->position[2]);
        p0 = add(t.p0, pos);
        p1 = add(tri_p1(&t), pos);
        p2 = add(tri_p2(&t), pos);
        tri_set(&t, p0, p1, p2);
        out[i] = t;
    }
}

/* ------------------------------------------------------------------ binned SAH builder */
typedef struct { double lo[3], hi[3]; } aabb;
static inline void aabb_empty(aabb* b) {
    for (int k = 0; k < 3; ++k) { b->lo[k] = DBL_MAX; b->hi[k] = -DBL_MAX; }
}
static inline void aabb_grow(aabb* b, const aabb* o) {
    for (int k = 0; k < 3; ++k) {
        if (o->lo[k] < b->lo[k]) b->lo[k] = o->lo[k];
        if (o->hi[k] > b->hi[k]) b->hi[k] = o->hi[k];
    }
}
static inline double aabb_half_area(const aabb* b) {
    double dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.0;
    return dx * dy + dy * dz + dz * dx;
}

typedef struct {
    aabb* box;
    double* cen;  /* 3 per triangle */
    uint32_t* idx;
    node_t* nodes;
    size_t next; /* node allocator */
} builder_t;

#define NBINS 32
#define MAX_LEAF 16

static size_t alloc_pair(builder_t* B) {
    size_t r;
#pragma omp atomic capture
    { r = B->next; B->next += 2; }
    return r;
}

static void build_rec(builder_t* B, size_t node, uint32_t begin, uint32_t end, int depth) {
    aabb nb, cb;
    aabb_empty(&nb);
    aabb_empty(&cb);
    for (uint32_t i = begin; i < end; ++i) {
        uint32_t p = B->idx[i];
        aabb_grow(&nb, &B->box[p]);
        aabb c;
        for (int k = 0; k < 3; ++k) c.lo[k] = c.hi[k] = B->cen[3 * p + k];
        aabb_grow(&cb, &c);
    }
    node_t* N = &B->nodes[node];
    N->b[0] = nb.lo[0]; N->b[1] = nb.hi[0]; N->b[2] = nb.lo[1];
    N->b[3] = nb.hi[1]; N->b[4] = nb.lo[2]; N->b[5] = nb.hi[2];
    uint32_t count = end - begin;
    int best_axis = -1;
    double best_cost = DBL_MAX;
    int best_bin = 0;
    if (count > 2 && depth < 60) {
        for (int ax = 0; ax < 3; ++ax) {
            double lo = cb.lo[ax], ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0)) continue;
            aabb bb[NBINS];
            uint32_t bc[NBINS];
            for (int k = 0; k < NBINS; ++k) { aabb_empty(&bb[k]); bc[k] = 0; }
            double s = NBINS / ext;
            for (uint32_t i = begin; i < end; ++i) {
                uint32_t p = B->idx[i];
                int k = (int)((B->cen[3 * p + ax] - lo) * s);
                if (k >= NBINS) k = NBINS - 1;
                if (k < 0) k = 0;
                aabb_grow(&bb[k], &B->box[p]);
                bc[k]++;
            }
            double right_area[NBINS];
            uint32_t right_count[NBINS];
            aabb acc;
            aabb_empty(&acc);
            uint32_t c = 0;
            for (int k = NBINS - 1; k > 0; --k) {
                aabb_grow(&acc, &bb[k]);
                c += bc[k];
                right_area[k] = aabb_half_area(&acc);
                right_count[k] = c;
            }
            aabb_empty(&acc);
            c = 0;
            for (int k = 0; k < NBINS - 1; ++k) {
                aabb_grow(&acc, &bb[k]);
                c += bc[k];
                if (c == 0 || right_count[k + 1] == 0) continue;
                double cost = aabb_half_area(&acc) * c + right_area[k + 1] * right_count[k + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = k; }
            }
        }
    }
    /* leaf when SAH prefers it (traversal cost 1, sah_based_algorithm.hpp:11-17) and it is small enough */
    double leaf_cost = aabb_half_area(&nb) * (count - 1.0);
    int make_leaf = count <= 2 || (best_axis < 0 && count <= MAX_LEAF) ||
                    (best_axis >= 0 && best_cost >= leaf_cost && count <= MAX_LEAF);
    if (make_leaf || depth >= 60) {
        N->count = count;
        N->first = begin;
        return;
    }
    uint32_t mid;
    if (best_axis >= 0) {
        double lo = cb.lo[best_axis], s = NBINS / (cb.hi[best_axis] - cb.lo[best_axis]);
        uint32_t i = begin, j = end;
        while (i < j) {
            uint32_t p = B->idx[i];
            int k = (int)((B->cen[3 * p + best_axis] - lo) * s);
            if (k >= NBINS) k = NBINS - 1;
            if (k < 0) k = 0;
            if (k <= best_bin) ++i;
            else { uint32_t tmp = B->idx[--j]; B->idx[j] = B->idx[i]; B->idx[i] = tmp; }
        }
        mid = i;
        if (mid == begin || mid == end) mid = begin + count / 2;
    } else {
        mid = begin + count / 2;  /* all centroids coincide: median split */
    }
    size_t first = alloc_pair(B);
    N->count = 0;
    N->first = (uint32_t)first;
    if (count > 4096) {
#pragma omp task
        build_rec(B, first, begin, mid, depth + 1);
#pragma omp task
        build_rec(B, first + 1, mid, end, depth + 1);
#pragma omp taskwait
    } else {
        build_rec(B, first, begin, mid, depth + 1);
        build_rec(B, first + 1, mid, end, depth + 1);
    }
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

oracle_scene* oracle_scene_create(const oracle_entity* ents, uint32_t n_ents, int nthreads) {
    set_threads(nthreads);
    oracle_scene* s = (oracle_scene*)calloc(1, sizeof(oracle_scene));
    size_t n = 0;
    for (uint32_t e = 0; e < n_ents; ++e) n += ents[e].n_tris;
    s->n = n;
    s->tris = (tri_t*)malloc(sizeof(tri_t) * (n ? n : 1));
    s->tri_ent = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    s->ents = (ent_t*)malloc(sizeof(ent_t) * (n_ents ? n_ents : 1));
    s->n_ents = n_ents;
    size_t off = 0;
    for (uint32_t e = 0; e < n_ents; ++e) {
        transform_entity(&ents[e], s->tris + off);
        for (size_t i = 0; i < ents[e].n_tris; ++i) s->tri_ent[off + i] = e;
        s->ents[e].smooth = (uint32_t)ents[e].smooth_shading;
        s->ents[e].id = ents[e].id;
        memcpy(s->ents[e].color, ents[e].color, sizeof(float) * 3);
        s->ents[e].rho_s = ents[e].rho_s;
        s->ents[e].rho_d = ents[e].rho_d;
        off += ents[e].n_tris;
    }
    s->flat = (double*)malloc(sizeof(double) * 12 * (n ? n : 1));
    for (size_t i = 0; i < n; ++i) {
        const tri_t* t = &s->tris[i];
        double* f = s->flat + 12 * i;
        f[0] = t->p0.x; f[1] = t->p0.y; f[2] = t->p0.z;
        f[3] = t->e1.x; f[4] = t->e1.y; f[5] = t->e1.z;
        f[6] = t->e2.x; f[7] = t->e2.y; f[8] = t->e2.z;
        f[9] = t->n.x; f[10] = t->n.y; f[11] = t->n.z;
    }
    /* compute_bounding_boxes_and_centers (lib/bvh/utilities.hpp:162-173; centre = triangle.hpp:91-93) */
    builder_t B;
    B.box = (aabb*)malloc(sizeof(aabb) * (n ? n : 1));
    B.cen = (double*)malloc(sizeof(double) * 3 * (n ? n : 1));
    B.idx = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        const tri_t* t = &s->tris[i];
        v3 p[3] = {t->p0, tri_p1(t), tri_p2(t)};
        for (int k = 0; k < 3; ++k) {
            double a = comp(p[0], k), b = comp(p[1], k), c = comp(p[2], k);
            B.box[i].lo[k] = fmin(a, fmin(b, c));
            B.box[i].hi[k] = fmax(a, fmax(b, c));
        }
        v3 c = scl(add(add(p[0], p[1]), p[2]), 1.0 / 3.0);
        B.cen[3 * i] = c.x; B.cen[3 * i + 1] = c.y; B.cen[3 * i + 2] = c.z;
        B.idx[i] = (uint32_t)i;
    }
    B.nodes = (node_t*)calloc(2 * (n ? n : 1) + 1, sizeof(node_t));
    B.next = 1;
    if (n) {
#pragma omp parallel
#pragma omp single
        build_rec(&B, 0, 0, (uint32_t)n, 0);
    }
    s->nodes = B.nodes;
    s->n_nodes = B.next;
    s->prim_idx = B.idx;
    free(B.box);
    free(B.cen);
    return s;
}

void oracle_scene_destroy(oracle_scene* s) {
    if (!s) return;
    free(s->tris); free(s->tri_ent); free(s->ents); free(s->nodes); free(s->prim_idx); free(s->flat);
    free(s);
}
size_t oracle_scene_num_tris(const oracle_scene* s) { return s->n; }
size_t oracle_scene_num_nodes(const oracle_scene* s) { return s->n_nodes; }
const double* oracle_scene_tris(const oracle_scene* s) { return s->flat; }

/* ------------------------------------------------------------------ intersection */
typedef struct { v3 o, d; double tmin, tmax; } ray_t;

/* Triangle::intersect (triangle.hpp:140-160): NaN-rejecting barycentric test, inclusive t range */
static inline int tri_intersect(const tri_t* tr, const ray_t* r, double* t, double* u, double* v) {
    v3 c = sub(tr->p0, r->o);
    v3 rr = cross(r->d, c);
    double inv_det = 1.0 / dot(tr->n, r->d);
    double uu = dot(rr, tr->e2) * inv_det;
    double vv = dot(rr, tr->e1) * inv_det;
    double ww = 1.0 - uu - vv;
    if (uu >= 0 && vv >= 0 && ww >= 0) {
        double tt = dot(tr->n, c) * inv_det;
        if (tt >= r->tmin && tt <= r->tmax) { *t = tt; *u = uu; *v = vv; return 1; }
    }
    return 0;
}

/* Vector::safe_inverse (vector.hpp:75-80) */
static inline double safe_inv(double x) {
    const double eps = DBL_EPSILON;
    return 1.0 / (fabs(x) < eps ? copysign(eps, x) : x);
}

typedef struct { int oct[3]; v3 inv, so; } nisect_t;  /* FastNodeIntersector (node_intersectors.hpp:83-103) */
static inline void nisect_init(nisect_t* ni, const ray_t* r) {
    ni->oct[0] = signbit(r->d.x) != 0;
    ni->oct[1] = signbit(r->d.y) != 0;
    ni->oct[2] = signbit(r->d.z) != 0;
    ni->inv = mk(safe_inv(r->d.x), safe_inv(r->d.y), safe_inv(r->d.z));
    ni->so = mk(-r->o.x * ni->inv.x, -r->o.y * ni->inv.y, -r->o.z * ni->inv.z);
}
/* robust_min / robust_max (utilities.hpp:59-85) */
static inline double rmin(double x, double y) { return x < y ? x : y; }
static inline double rmax(double x, double y) { return x > y ? x : y; }
/* NodeIntersector::intersect (node_intersectors.hpp:35-47) */
static inline void node_isect(const nisect_t* ni, const node_t* nd, const ray_t* r, double* entry, double* exit) {
    double ex = nd->b[0 + ni->oct[0]] * ni->inv.x + ni->so.x;
    double ey = nd->b[2 + ni->oct[1]] * ni->inv.y + ni->so.y;
    double ez = nd->b[4 + ni->oct[2]] * ni->inv.z + ni->so.z;
    double xx = nd->b[1 - ni->oct[0]] * ni->inv.x + ni->so.x;
    double xy = nd->b[3 - ni->oct[1]] * ni->inv.y + ni->so.y;
    double xz = nd->b[5 - ni->oct[2]] * ni->inv.z + ni->so.z;
    *entry = rmax(ex, rmax(ey, rmax(ez, r->tmin)));
    *exit = rmin(xx, rmin(xy, rmin(xz, r->tmax)));
}

typedef struct { int64_t prim; double t, u, v; } hit_t;

/* intersect_leaf (single_ray_traverser.hpp:40-59) with Closest/AnyPrimitiveIntersector
 * (primitive_intersectors.hpp:33-76): index through prim_idx, shrink tmax on every hit. */
static inline int leaf(const oracle_scene* s, const node_t* nd, ray_t* r, hit_t* best, int any) {
    for (uint32_t i = nd->first; i < nd->first + nd->count; ++i) {
        uint32_t p = s->prim_idx[i];
        double t, u, v;
        if (tri_intersect(&s->tris[p], r, &t, &u, &v)) {
            best->prim = p; best->t = t; best->u = u; best->v = v;
            if (any) return 1;
            r->tmax = t;
        }
    }
    return 0;
}

/* SingleRayTraverser::intersect (single_ray_traverser.hpp:68-126): eager leaves, near child first,
 * 64-entry stack. Returns 1 when something was hit. */
static int traverse(const oracle_scene* s, ray_t r, hit_t* best, int any) {
    best->prim = -1;
    if (s->n == 0) return 0;
    const node_t* nodes = s->nodes;
    if (nodes[0].count) { leaf(s, &nodes[0], &r, best, any); return best->prim >= 0; }
    nisect_t ni;
    nisect_init(&ni, &r);
    uint32_t stack[64];
    int sp = 0;
    const node_t* left = &nodes[nodes[0].first];
    while (1) {
        const node_t* right = left + 1;
        double le, lx, re, rx;
        node_isect(&ni, left, &r, &le, &lx);
        node_isect(&ni, right, &r, &re, &rx);
        if (le <= lx) {
            if (left->count) {
                if (leaf(s, left, &r, best, any) && any) break;
                left = NULL;
            }
        } else left = NULL;
        if (re <= rx) {
            if (right->count) {
                if (leaf(s, right, &r, best, any) && any) break;
                right = NULL;
            }
        } else right = NULL;
        if (left) {
            if (right) {
                if (le > re) { const node_t* tmp = left; left = right; right = tmp; }
                if (sp < 64) stack[sp++] = right->first;
            }
            left = &nodes[left->first];
        } else if (right) {
            left = &nodes[right->first];
        } else {
            if (sp == 0) break;
            left = &nodes[stack[--sp]];
        }
    }
    return best->prim >= 0;
}

static inline ray_t ray_from(const double* q) {
    ray_t r;
    r.o = mk(q[0], q[1], q[2]);
    r.d = mk(q[3], q[4], q[5]);
    r.tmin = q[6];
    r.tmax = q[7];
    return r;
}

void oracle_trace_closest(const oracle_scene* s, const double* rays, size_t n, int64_t* prim, double* t,
                          double* u, double* v, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        hit_t h;
        traverse(s, ray_from(rays + 8 * i), &h, 0);
        prim[i] = h.prim;
        if (t) t[i] = h.prim >= 0 ? h.t : 0;
        if (u) u[i] = h.prim >= 0 ? h.u : 0;
        if (v) v[i] = h.prim >= 0 ? h.v : 0;
    }
}

void oracle_trace_any(const oracle_scene* s, const double* rays, size_t n, uint8_t* occluded, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        hit_t h;
        occluded[i] = (uint8_t)traverse(s, ray_from(rays + 8 * i), &h, 1);
    }
}

/* ------------------------------------------------------------------ cameras and passes */
/* SimpleCamera ctor + pixel_to_ray (cameras/simple_camera.hpp:14-27, 61-81) */
static inline ray_t camera_ray(const oracle_camera* c, double u, double v) {
    double cx = c->resolution[0] / 2.0, cy = c->resolution[1] / 2.0;
    double sx = c->resolution[0] / c->sensor_size[0], sy = c->resolution[1] / c->sensor_size[1];
    v3 d = normalize(mk((-cx + u) / sx, (cy - v) / sy, c->z_positive ? c->focal_length : -c->focal_length));
    ray_t r;
    r.d = rotate_t(d, c->rotation);
    r.o = mk(c->position[0], c->position[1], c->position[2]);
    r.tmin = 0.0;
    r.tmax = DBL_MAX;
    return r;
}

static inline uint32_t width_of(const oracle_camera* c) { return (uint32_t)floor(c->resolution[0]); }

void oracle_camera_rays(const oracle_camera* cam, uint32_t row0, uint32_t row1, double* rays) {
    uint32_t W = width_of(cam);
    for (uint32_t j = row0; j < row1; ++j)
        for (uint32_t i = 0; i < W; ++i) {
            ray_t r = camera_ray(cam, i, j);
            double* q = rays + 8 * ((size_t)(j - row0) * W + i);
            q[0] = r.o.x; q[1] = r.o.y; q[2] = r.o.z;
            q[3] = r.d.x; q[4] = r.d.y; q[5] = r.d.z;
            q[6] = r.tmin; q[7] = r.tmax;
        }
}

/* hit point u*p1 + v*p2 + (1-u-v)*p0 (passes.hpp:53, do_lidar.hpp:53) */
static inline v3 hit_point(const tri_t* t, double u, double v) {
    return add(add(scl(tri_p1(t), u), scl(tri_p2(t), v)), scl(t->p0, 1.0 - u - v));
}
/* shading normal (passes.hpp:179, unidirectional.hpp:45-52) */
static inline v3 shading_normal(const oracle_scene* s, int64_t p, double u, double v) {
    const tri_t* t = &s->tris[p];
    if (s->ents[s->tri_ent[p]].smooth)
        return normalize(add(add(scl(t->vn1, u), scl(t->vn2, v)), scl(t->vn0, 1.0 - u - v)));
    return normalize(t->n);
}

/* get_inetersections / get_instances / get_normals (passes.hpp:14-198) fused over one traversal */
void oracle_passes(const oracle_scene* s, const oracle_camera* cam, uint32_t row0, uint32_t row1, double* xyz,
                   uint32_t* ids, double* normals, int64_t* prim, int nthreads) {
    set_threads(nthreads);
    uint32_t W = width_of(cam);
    long long total = (long long)(row1 - row0) * W;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long k = 0; k < total; ++k) {
        uint32_t j = row0 + (uint32_t)(k / W), i = (uint32_t)(k % W);
        hit_t h;
        int hit = traverse(s, camera_ray(cam, i, j), &h, 0);
        v3 x = mk(0, 0, 0), nn = mk(0, 0, 0);
        uint32_t id = 0;
        if (hit) {
            x = hit_point(&s->tris[h.prim], h.u, h.v);
            nn = shading_normal(s, h.prim, h.u, h.v);
            id = s->ents[s->tri_ent[h.prim]].id;
        }
        if (xyz) { xyz[3 * k] = x.x; xyz[3 * k + 1] = x.y; xyz[3 * k + 2] = x.z; }
        if (normals) { normals[3 * k] = nn.x; normals[3 * k + 1] = nn.y; normals[3 * k + 2] = nn.z; }
        if (ids) ids[k] = id;
        if (prim) prim[k] = hit ? h.prim : -1;
    }
}

/* SimpleLidar::batch_cast_rays (lidars/simple_lidar.hpp:66-96) + do_batch_lidar (do_lidar.hpp:80-155):
 * one boresight ray per pose, range = |hit - position|, 0 on a miss. */
void oracle_lidar_batch(const oracle_scene* s, const double* positions, const double* rotations, size_t n,
                        int z_positive, double* range, int64_t* prim, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        ray_t r;
        r.o = mk(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]);
        r.d = rotate_t(normalize(mk(0, 0, z_positive ? 1.0 : -1.0)), rotations + 9 * i);
        r.tmin = 0.0;
        r.tmax = DBL_MAX;
        hit_t h;
        int hit = traverse(s, r, &h, 0);
        range[i] = hit ? length(sub(hit_point(&s->tris[h.prim], h.u, h.v), r.o)) : 0.0;
        if (prim) prim[i] = hit ? h.prim : -1;
    }
}

/* ------------------------------------------------------------------ Philox4x32-10
 * Counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as easy as
 * 1, 2, 3" (SC'11): ten rounds of two 32x32->64 multiplies with a Weyl-sequence key schedule. */
void oracle_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
static inline double unif24(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }

/* draw two uniforms for (pixel, sample, bounce, purpose) */
static inline void rng2(const oracle_render_params* p, uint32_t pixel, uint32_t sample, uint32_t bounce,
                        uint32_t purpose, double* a, double* b) {
    uint32_t o[4];
    oracle_philox(pixel, sample, (bounce << 8) | purpose, p->request, (uint32_t)p->seed, (uint32_t)(p->seed >> 32), o);
    *a = unif24(o[0]);
    *b = unif24(o[1]);
}

/* ------------------------------------------------------------------ path tracer */
typedef struct { float r, g, b; } col_t;

/* cosine_importance (materials/brdfs.hpp:18-42): Malley's method about a left-handed normal */
static v3 cosine_importance(v3 n, double r1, double r2) {
    double r = sqrt(r1);
    double theta = r2 * 2 * 3.1415926;
    double x = -r * cos(theta);
    double y = -r * sin(theta);
    double z = -sqrt(fmax(0.0, 1.0 - x * x - y * y));
    v3 nx;
    if (fabs(n.x) > fabs(n.y)) nx = scl(mk(n.z, 0.0, -n.x), 1.0 / sqrt(n.x * n.x + n.z * n.z));
    else nx = scl(mk(0, n.z, -n.y), 1.0 / sqrt(n.y * n.y + n.z * n.z));
    v3 ny = cross(n, nx);
    return add(add(scl(nx, x), scl(ny, y)), scl(n, z));
}

/* unidirectional (path_tracing/unidirectional.hpp:24-96) with lights PointLight
 * (lights/point_light.hpp:32-39) and AreaLight (lights/area_light.hpp:54-72) and
 * ColoredLambertianMaterial (materials/material.hpp:91-111). */
static col_t trace_path(const oracle_scene* s, const oracle_light* L, uint32_t nl, const oracle_render_params* p,
                        ray_t ray, uint32_t pixel, uint32_t sample) {
    col_t path = {0, 0, 0};
    float w0 = (float)(2 * M_PI);
    col_t weight = {w0, w0, w0};
    hit_t h;
    int hit = traverse(s, ray, &h, 0);
    for (int bounce = 0; bounce < p->num_bounces; ++bounce) {
        if (!hit) break;
        const tri_t* tr = &s->tris[h.prim];
        const ent_t* en = &s->ents[s->tri_ent[h.prim]];
        double u = h.u, v = h.v;
        v3 normal = normalize(tr->n);
        v3 sn = en->smooth ? normalize(add(add(scl(tr->vn1, u), scl(tr->vn2, v)), scl(tr->vn0, 1.0 - u - v))) : normal;
        v3 x = hit_point(tr, u, v);
        x = sub(x, scl(normal, 0.0001));
        col_t lr = {0, 0, 0};
        for (uint32_t l = 0; l < nl; ++l) {
            ray_t sr;
            double inten;
            v3 lp = mk(L[l].position[0], L[l].position[1], L[l].position[2]);
            if (L[l].type == 1) {
                double a, b;
                rng2(p, pixel, sample, (uint32_t)bounce, 2 + l, &a, &b);
                double xc = L[l].size[0] * a - L[l].size[0] / 2;
                double yc = L[l].size[1] * b - L[l].size[1] / 2;
                v3 sp = add(rotate(mk(xc, yc, 0.0), L[l].rotation), lp);  /* transform(), transform.hpp:30-40 */
                sr.d = normalize(sub(sp, x));
                sr.tmax = length(sub(sp, x));
                inten = L[l].intensity / dot(sub(x, sp), sub(x, sp));
            } else {
                sr.d = normalize(sub(lp, x));
                sr.tmax = length(sub(lp, x));
                inten = fmin(L[l].intensity / dot(sub(x, lp), sub(x, lp)), 10000.0);
            }
            sr.o = x;
            sr.tmin = 0.0;
            hit_t sh;
            col_t c = {0, 0, 0};
            if (!traverse(s, sr, &sh, 1)) {       /* illumination (unidirectional.hpp:12-21) */
                float ldn = (float)(-dot(sr.d, sn));
                c.r = en->color[0] * ldn; c.g = en->color[1] * ldn; c.b = en->color[2] * ldn;
            }
            float fi = (float)inten;
            lr.r += c.r * fi; lr.g += c.g * fi; lr.b += c.b * fi;
        }
        if (bounce >= 1) {
            lr.r = fminf(fmaxf(lr.r, 0.f), 1.f);
            lr.g = fminf(fmaxf(lr.g, 0.f), 1.f);
            lr.b = fminf(fmaxf(lr.b, 0.f), 1.f);
        }
        path.r += lr.r * weight.r; path.g += lr.g * weight.g; path.b += lr.b * weight.b;
        if (bounce == p->num_bounces - 1) break;
        double r1, r2;
        rng2(p, pixel, sample, (uint32_t)bounce, 1, &r1, &r2);
        v3 nd = cosine_importance(sn, r1, r2);
        float bc = (float)(1 - r1);
        ray.o = x;
        ray.d = nd;
        ray.tmin = 0.0;
        ray.tmax = DBL_MAX;
        hit = traverse(s, ray, &h, 0);
        weight.r *= bc; weight.g *= bc; weight.b *= bc;
    }
    return path;
}

/* do_render (do_render.hpp:65-134): jittered samples, running mean, adaptive stop, u8 quantise */
void oracle_render(const oracle_scene* s, const oracle_camera* cam, const oracle_light* lights, uint32_t n_lights,
                   const oracle_render_params* p, uint32_t row0, uint32_t row1, float* radiance, uint8_t* rgba8,
                   uint32_t* samples_taken, double* m2, int nthreads) {
    set_threads(nthreads);
    uint32_t W = width_of(cam);
    long long total = (long long)(row1 - row0) * W;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long k = 0; k < total; ++k) {
        uint32_t j = row0 + (uint32_t)(k / W), i = (uint32_t)(k % W);
        uint32_t pixel = j * W + i;
        col_t pix = {0, 0, 0};
        double wm[3] = {0, 0, 0}, wm2[3] = {0, 0, 0};   /* Welford mean / M2 of the samples (test statistics) */
        int sample;
        int taken = 0;
        for (sample = 1; sample < p->max_samples + 1; ++sample) {
            ray_t ray;
            if (p->max_samples == 1) ray = camera_ray(cam, i, j);
            else {
                double a, b;
                rng2(p, pixel, (uint32_t)(sample - 1), 0, 0, &a, &b);
                ray = camera_ray(cam, i + (a - 0.5), j + (b - 0.5));
            }
            col_t L = trace_path(s, lights, n_lights, p, ray, pixel, (uint32_t)(sample - 1));
            taken = sample;
            const double lv[3] = {L.r, L.g, L.b};
            for (int c = 0; c < 3; ++c) {
                double dl = lv[c] - wm[c];
                wm[c] += dl / sample;
                wm2[c] += dl * (lv[c] - wm[c]);
            }
            float inv = 1.0f / sample;
            col_t d = {(L.r - pix.r) * inv, (L.g - pix.g) * inv, (L.b - pix.b) * inv};
            pix.r += d.r; pix.g += d.g; pix.b += d.b;
            if (sample >= p->min_samples) {
                double noise = sqrtf(d.r * d.r + d.g * d.g + d.b * d.b);
                if (noise < p->noise_threshold) break;
            }
        }
        float px[4] = {pix.r, pix.g, pix.b, 1.0f};
        for (int c = 0; c < 4; ++c) {
            if (radiance) radiance[4 * k + c] = px[c];
            if (rgba8) {
                float q = px[c] * 256;
                q = q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q);
                rgba8[4 * k + c] = (uint8_t)q;
            }
        }
        if (samples_taken) samples_taken[k] = (uint32_t)taken;
        if (m2) for (int c = 0; c < 3; ++c) m2[3 * k + c] = wm2[c];
    }
}

/* ------------------------------------------------------------------ radiation pressure
 * No counterpart in the reference (README.md:9 names the feature only).  Flat-plate model
 * (Montenbruck & Gill, Satellite Orbits, sec. 3.4): a ray of power E along d hitting a facet
 * whose normal n faces the ray (cos = -d.n) transfers force (E/c)[(1-rs) d - (2 rs cos + 2/3 rd) n];
 * the facet absorbs (1-rs-rd) E; the specular part continues along the mirror direction with
 * power rs E for up to num_bounces further segments.  Facets are two-sided. */
void oracle_srp(const oracle_scene* s, const oracle_srp_params* p, uint32_t row0, uint32_t row1, double* force,
                double* torque, double* facet_power, int nthreads) {
    set_threads(nthreads);
    v3 sd = normalize(mk(p->sun_dir[0], p->sun_dir[1], p->sun_dir[2]));
    /* grid basis perpendicular to the sun direction */
    v3 a = fabs(sd.x) < 0.9 ? mk(1, 0, 0) : mk(0, 1, 0);
    v3 e1 = normalize(cross(sd, a));
    v3 e2 = cross(sd, e1);
    double h = 2.0 * p->half_extent / p->grid;
    double E0 = p->flux * h * h;
    v3 ctr = mk(p->center[0], p->center[1], p->center[2]);
    v3 cm = mk(p->center_of_mass[0], p->center_of_mass[1], p->center_of_mass[2]);
    v3 org0 = add(ctr, scl(sd, 2.0 * p->half_extent + 1.0));
    double eps = 1e-5 * 2.0 * p->half_extent;
    double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
    long long total = (long long)(row1 - row0) * p->grid;
#pragma omp parallel
    {
        double f[3] = {0, 0, 0}, t[3] = {0, 0, 0};
#pragma omp for schedule(dynamic, 256)
        for (long long k = 0; k < total; ++k) {
            uint32_t j = row0 + (uint32_t)(k / p->grid), i = (uint32_t)(k % p->grid);
            ray_t r;
            r.o = add(org0, add(scl(e1, -p->half_extent + (i + 0.5) * h), scl(e2, -p->half_extent + (j + 0.5) * h)));
            r.d = scl(sd, -1.0);
            r.tmin = 0.0;
            r.tmax = DBL_MAX;
            double E = E0;
            for (uint32_t seg = 0; seg <= p->num_bounces; ++seg) {
                hit_t hh;
                if (!traverse(s, r, &hh, 0)) break;
                const tri_t* tr = &s->tris[hh.prim];
                const ent_t* en = &s->ents[s->tri_ent[hh.prim]];
                v3 n = scl(normalize(tr->n), -1.0);        /* outward for counter-clockwise meshes */
                if (dot(r.d, n) > 0) n = scl(n, -1.0);      /* two-sided: face the incoming ray */
                double cs = -dot(r.d, n);
                double rs = en->rho_s, rd = en->rho_d;
                double k1 = (E / p->c) * (1.0 - rs), k2 = (E / p->c) * (2.0 * rs * cs + (2.0 / 3.0) * rd);
                v3 df = sub(scl(r.d, k1), scl(n, k2));
                v3 x = hit_point(tr, hh.u, hh.v);
                v3 dt = cross(sub(x, cm), df);
                f[0] += df.x; f[1] += df.y; f[2] += df.z;
                t[0] += dt.x; t[1] += dt.y; t[2] += dt.z;
                if (facet_power) {
                    double pw = (1.0 - rs - rd) * E;
#pragma omp atomic
                    facet_power[hh.prim] += pw;
                }
                if (!(rs > 0)) break;
                v3 rdir = sub(r.d, scl(n, 2.0 * dot(r.d, n)));
                r.o = add(x, scl(n, eps));
                r.d = rdir;
                r.tmin = 0.0;
                r.tmax = DBL_MAX;
                E *= rs;
            }
        }
#pragma omp critical
        {
            for (int c = 0; c < 3; ++c) { F[c] += f[c]; T[c] += t[c]; }
        }
    }
    for (int c = 0; c < 3; ++c) { force[c] = F[c]; torque[c] = T[c]; }
}
