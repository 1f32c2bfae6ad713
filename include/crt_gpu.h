/* crt_gpu.h -- C ABI of the GB300 ray-query library (libcrt_gpu.so).
 *
 * This is the drop-in boundary for the ray-query hot path of ceres-raytracer (CRT v0.6a4): BVH
 * construction, closest-hit and any-hit traversal with ray/triangle intersection, and the
 * integrators built on them (primary-ray passes, LiDAR, unidirectional path tracing, solar
 * radiation pressure).  The reference implements this path as C++ templates behind its pybind11
 * module `_crt` (src/pybind.cpp); each entry point below cites the reference function it replaces.
 *
 * Conventions
 *  - Every function returns an int status: CRT_OK (0) or a negative CRT_ERR_* code;
 *    crt_context_last_error() returns the message of the last failure on that context.
 *  - Plain pointers and sizes only.  Input and output buffers may live in host memory or in device
 *    memory of the context's GPU: the library inspects each pointer and copies host buffers itself.
 *    Calls are synchronous with respect to host buffers; device-buffer outputs are ordered on the
 *    context stream (see crt_context_set_stream).
 *  - Geometry is FP32 on the device; camera, LiDAR, light and body-frame inputs are FP64 as in the
 *    reference and are reduced to FP32 rays once per request on the host.  Radiation-pressure sums
 *    are FP64.  The FP32 triangle test is watertight: no ray passes between two triangles that
 *    share an edge (its vertices transformed once, so they are bit-identical in both triangles).
 *  - Host outputs of renders, passes, LiDAR and ray traces in page-locked memory (crt_host_alloc)
 *    are written by the kernels in place; other host outputs are staged in device memory and
 *    copied back.
 *  - A context (and every scene created on it) must not be used from two threads at once.
 */
#ifndef CRT_GPU_H
#define CRT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRT_ABI_VERSION 3

enum {
    CRT_OK = 0,
    CRT_ERR_INVALID = -1,   /* bad argument, shape or state                              */
    CRT_ERR_CUDA = -2,      /* CUDA runtime error (message in crt_context_last_error)     */
    CRT_ERR_OOM = -3,       /* device or host allocation failed / over the memory budget  */
    CRT_ERR_TIMEOUT = -4,   /* a bounded device wait or a host deadline expired           */
    CRT_ERR_IO = -5,        /* file could not be read                                     */
    CRT_ERR_DEVICE = -6,    /* a device-side check failed (e.g. traversal stack overflow) */
    CRT_ERR_NO_DEVICE = -7  /* no CUDA device / the library was built for another GPU      */
};

#define CRT_MISS 0xFFFFFFFFu   /* primitive index reported for a ray that hits nothing */

typedef struct crt_context crt_context;
typedef struct crt_scene crt_scene;
typedef struct crt_mesh crt_mesh;

/* A ray: bvh::Ray (lib/bvh/ray.hpp:10-23) in FP32, 32 bytes.  Hits are accepted for
 * tmin <= t <= tmax (inclusive, lib/bvh/triangle.hpp:155). */
typedef struct {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} crt_ray;

/* Closest hit: ClosestPrimitiveIntersector::Result (lib/bvh/primitive_intersectors.hpp:37-42), 16 bytes.
 * prim is the index into the scene's triangle list (entities concatenated in order, each entity's
 * triangles in file order), or CRT_MISS. */
typedef struct {
    float t, u, v;
    uint32_t prim;
} crt_hit;

/* One entity placed in a scene: Entity (src/crt/rendering_dynamic/entity.hpp:21-86) with its pose.
 * The library applies resize -> rotate -> translate in FP64 as transform.hpp:43-85 does. */
typedef struct {
    const float* tri_xyz;     /* n_tris * 9: p0, p1, p2 (host or device memory) */
    const float* tri_vn;      /* n_tris * 9 vertex normals, or NULL (only used with smooth shading) */
    size_t n_tris;
    double scale;
    double position[3];
    double rotation[9];       /* row-major 3x3 */
    float color[3];           /* ColoredLambertianMaterial colour (entity.hpp:52) */
    int smooth_shading;
    uint32_t id;              /* instance id reported by the instance pass */
    float rho_s, rho_d;       /* specular / diffuse reflectivity (radiation pressure only) */
} crt_entity_desc;

/* SimpleCamera (src/crt/cameras/simple_camera.hpp:14-81) */
typedef struct {
    double position[3];
    double rotation[9];       /* row-major; directions go to the world frame through its transpose */
    double focal_length;
    double resolution[2];
    double sensor_size[2];
    int z_positive;
} crt_camera_desc;

/* PointLight (lights/point_light.hpp) when type == 0, AreaLight (lights/area_light.hpp) when 1 */
typedef struct {
    int type;
    double intensity;
    double position[3];
    double rotation[9];
    double size[2];
} crt_light_desc;

/* Arguments of BodyFixedGroup.render (src/pybind.cpp:467-498) plus the random stream identity. */
typedef struct {
    int min_samples;
    int max_samples;
    double noise_threshold;
    int num_bounces;
    uint64_t seed;            /* Philox key; results do not depend on how requests are batched */
    uint32_t request;         /* Philox counter word distinguishing requests with the same seed */
} crt_render_params;

/* LiDAR beam grid (extension of SimpleLidar, lidars/simple_lidar.hpp:42-64, to nx * ny beams).
 * Beam (i, j) points along normalize(tan_x[i], tan_y[j], +-1) in the sensor frame with
 * tan_x[i] = tan(-half_x + (i + 0.5) * 2 half_x / nx) (same for y), i.e. angles uniform over
 * [-half, half]; the world direction is R^T of that, as for the reference boresight. */
typedef struct {
    double position[3];
    double rotation[9];
    int z_positive;
    uint32_t nx, ny;
    double half_angle_x, half_angle_y;   /* radians */
} crt_lidar_grid_desc;

/* Solar radiation pressure over a parallel sun-ray grid (no counterpart in the reference). */
typedef struct {
    double sun_dir_inertial[3];   /* unit vector toward the sun in the inertial frame */
    double flux;                  /* W / m^2 at the body */
    double c;                     /* m / s */
    double center_of_mass[3];     /* body frame */
    uint32_t grid;                /* grid x grid rays per attitude, 1..32768 */
    uint32_t num_bounces;         /* specular continuation segments after the primary hit */
} crt_srp_desc;

/* One request of a batch (crt_batch).  kind selects which fields are used. */
enum { CRT_REQUEST_RENDER = 0, CRT_REQUEST_LIDAR = 1 };
typedef struct {
    int kind;
    crt_scene* scene;                     /* resident scene (requests of a batch may use different ones) */
    /* CRT_REQUEST_RENDER: as crt_render */
    const crt_camera_desc* camera;
    const crt_light_desc* lights;
    uint32_t n_lights;
    const crt_render_params* params;
    uint8_t* rgba8;                       /* [H][W][4] or NULL */
    float* radiance;                      /* [H][W][4] or NULL */
    /* CRT_REQUEST_LIDAR: as crt_lidar_grid */
    const crt_lidar_grid_desc* lidar;
    double* range;                        /* [ny][nx] */
    uint32_t* prim;                       /* [ny][nx] or NULL */
} crt_request;

typedef struct {
    size_t waves;                         /* wavefront waves executed */
    uint64_t render_paths;                /* camera paths (pixels x samples) */
    uint64_t lidar_beams;
} crt_batch_stats;

/* Tuning knobs of the persistent kernels and the batched wavefront (chosen by the autotuner). */
typedef struct {
    uint32_t queue_chunk;                 /* max 32-ray groups per atomic grab (1..8), guided by the work left */
    uint32_t wave_paths;                  /* camera paths per wave (>= 65536) */
    int use_graphs;                       /* replay batched waves as CUDA graphs */
    int build_sah;                        /* scenes built afterwards: binned-SAH tree (1, default) or
                                             Karras radix tree over the Morton order (0, faster build) */
    float collapse_tri_cost;              /* scenes built afterwards: cost of a triangle test relative to
                                             an 8-wide node test in the 8-wide collapse (default 0.15,
                                             best for coherent rays; ~0.5 suits multi-bounce path
                                             tracing); 0.01 .. 10 */
    uint32_t treelet_passes;              /* scenes built afterwards: passes of treelet restructuring over
                                             the binary tree before the 8-wide collapse (default 1; 0 .. 8;
                                             0 skips the optimisation: faster build) */
} crt_tuning;

typedef struct {
    size_t n_tris;
    size_t n_nodes;           /* 8-wide compressed nodes */
    size_t n_entities;
    uint32_t depth;           /* levels of the 8-wide tree */
    double build_ms;          /* device time of the last build */
    size_t device_bytes;      /* resident bytes held by the scene */
    float bounds[6];          /* xmin, ymin, zmin, xmax, ymax, zmax */
} crt_scene_stats;

typedef struct {
    uint64_t rays;            /* rays traversed by counting-mode kernels */
    uint64_t nodes;           /* 8-wide nodes fetched */
    uint64_t tris;            /* triangles tested */
    uint64_t launches;        /* kernels launched by the library on this context (always counted) */
    uint64_t resolved;        /* rays answered without a traversal (counting mode): SRP sun rays that
                                 miss the scene box, shadow rays stopped by the surface they leave */
} crt_counters;

/* ---------------------------------------------------------------- context */
int crt_context_create(int device, crt_context** out);
int crt_context_destroy(crt_context* ctx);
/* Order all work of this context on `stream` (a cudaStream_t); NULL restores the context's own. */
int crt_context_set_stream(crt_context* ctx, void* stream);
void* crt_context_get_stream(crt_context* ctx);
int crt_context_synchronize(crt_context* ctx);
/* Counting mode: traversal kernels also count node fetches and triangle tests (slower). */
int crt_context_set_counting(crt_context* ctx, int enabled);
int crt_context_get_counters(crt_context* ctx, crt_counters* out);
int crt_context_reset_counters(crt_context* ctx);
int crt_context_set_tuning(crt_context* ctx, const crt_tuning* tuning);
int crt_context_get_tuning(const crt_context* ctx, crt_tuning* out);
const char* crt_context_last_error(const crt_context* ctx);
const char* crt_status_string(int status);
int crt_abi_version(void);

/* ---------------------------------------------------------------- meshes (host) */
/* obj::load_from_file (lib/model_loaders/obj.hpp:59-127): `v` lines via strtof, `f` lines
 * fan-triangulated, negative indices allowed, vertex normals = normalised sums of left-handed face
 * normals.  Used by Entity's constructor (entity.hpp:31-41). */
int crt_mesh_load_obj(const char* path, crt_mesh** out);
size_t crt_mesh_num_tris(const crt_mesh* mesh);
const float* crt_mesh_xyz(const crt_mesh* mesh);       /* n_tris * 9 */
const float* crt_mesh_normals(const crt_mesh* mesh);   /* n_tris * 9 */
void crt_mesh_destroy(crt_mesh* mesh);

/* ---------------------------------------------------------------- scenes */
/* Upload, transform and build the device-resident BVH: replaces the scene assembly and BVH build of
 * BodyFixedGroup (rendering_body_fixed/body_fixed_group.hpp:45-89) and of the per-call rebuild in
 * rendering_dynamic/render.hpp:14-66 (SweepSahBuilder + ParallelReinsertionOptimizer +
 * NodeLayoutOptimizer, lib/bvh/sweep_sah_builder.hpp:43).  The GPU builder is Morton / LBVH /
 * 8-wide collapse; results of queries do not depend on the tree. */
int crt_scene_create(crt_context* ctx, const crt_entity_desc* entities, uint32_t n_entities, crt_scene** out);
int crt_scene_destroy(crt_scene* scene);
int crt_scene_get_stats(const crt_scene* scene, crt_scene_stats* out);

/* ---------------------------------------------------------------- ray queries */
/* SingleRayTraverser::traverse + ClosestPrimitiveIntersector (lib/bvh/single_ray_traverser.hpp:145,
 * primitive_intersectors.hpp:33-54). */
int crt_trace_closest(crt_scene* scene, const crt_ray* rays, size_t n, crt_hit* hits);
/* SingleRayTraverser::traverse + AnyPrimitiveIntersector (primitive_intersectors.hpp:58-76). */
int crt_trace_any(crt_scene* scene, const crt_ray* rays, size_t n, uint8_t* occluded);

/* ---------------------------------------------------------------- integrators */
/* get_inetersections / get_instances / get_normals (src/crt/passes.hpp:14-198), fused over one
 * traversal per pixel; any output may be NULL.  xyz and normals are [H][W][3] doubles, ids [H][W]. */
int crt_passes(crt_scene* scene, const crt_camera_desc* camera, double* xyz, uint32_t* ids, double* normals);
/* do_batch_lidar (src/crt/do_lidar.hpp:80-155) with SimpleLidar::batch_cast_rays
 * (lidars/simple_lidar.hpp:66-96): one boresight ray per pose, range = |hit - position|, 0 on a
 * miss.  positions n*3, rotations n*9 (row-major per pose).  prim may be NULL. */
int crt_lidar_batch(crt_scene* scene, const double* positions, const double* rotations, size_t n,
                    int z_positive, double* range, uint32_t* prim);
/* nx * ny beam grid from one pose; range and prim are [ny][nx]; prim may be NULL. */
int crt_lidar_grid(crt_scene* scene, const crt_lidar_grid_desc* desc, double* range, uint32_t* prim);
/* do_render (src/crt/do_render.hpp:28-141) with unidirectional (path_tracing/unidirectional.hpp:24-96):
 * rgba8 is [H][W][4] (clamp(v*256, 0, 255)), radiance (optional) the float RGBA before quantisation. */
int crt_render(crt_scene* scene, const crt_camera_desc* camera, const crt_light_desc* lights, uint32_t n_lights,
               const crt_render_params* params, uint8_t* rgba8, float* radiance);
/* Many render and LiDAR requests in one set of persistent launches: do_render / do_batch_lidar
 * called once per request in the reference become one wavefront over every request's rays (one
 * shared ray queue per stage).  Each request's outputs are identical to its own crt_render /
 * crt_lidar_grid call: random streams are keyed by (seed, request) and pixels consume their samples
 * in order.  Requests with adaptive sampling (noise_threshold > 0, min < max) advance one sample
 * per wave after their first min_samples. */
int crt_batch(crt_context* ctx, const crt_request* requests, size_t n, crt_batch_stats* stats);
/* Solar radiation pressure for n_att attitudes (unit quaternions w,x,y,z rotating body vectors into the
 * inertial frame).  force and torque are n_att*3 in the body frame (N, N m); facet_power (optional)
 * is n_att * n_tris absorbed power per triangle (W).  No reference counterpart (README.md:9). */
int crt_srp(crt_scene* scene, const crt_srp_desc* desc, const double* quaternions, size_t n_att, double* force,
            double* torque, double* facet_power);
/* Allocation-free variant of crt_srp (no counterpart in the reference): the same force and torque,
 * bit for bit, from the same wavefront stages, with all scratch (work counters, attitude table, one
 * wave's ray state and block sums, staging of host outputs) in one 64 MiB file-scope device array
 * instead of device allocations.  It is for callers that must not allocate device memory once they
 * run: flight-dynamics or attitude loops that evaluate radiation pressure every integration step
 * under a fixed memory budget, and components embedded in an application that owns the CUDA
 * allocator.  Limits: n_att <= 4096 per call (larger counts are refused with CRT_ERR_INVALID and a
 * message naming the static scratch); grid <= 32768 as for crt_srp; no per-facet output.
 * Quaternions, force and torque may each be host or device memory.  The first call on a device
 * resolves the array's device address (cudaGetSymbolAddress) and should come before any stream
 * capture.  Every call shares the array and keeps the previous call's contents: calls that overlap
 * on the GPU (other streams or contexts of the same device) race.  Every GPU that loads the library
 * keeps the 64 MiB until the process exits. */
int crt_srp_static(crt_scene* scene, const crt_srp_desc* desc, const double* quaternions, size_t n_att,
                   double* force, double* torque);

/* Read bandwidth of the context's GPU (no counterpart in the reference; a measurement aid for the
 * roofline of the traversal kernels): reads the `bytes` (>= 16) of the 16-byte aligned device buffer
 * `buf` `reps` times with 16-byte loads that bypass L1 and returns the mean device time of one pass
 * in ms (CUDA events on the context stream, after one untimed pass).  A buffer well inside the L2
 * cache measures L2 read bandwidth, one much larger than L2 measures HBM read bandwidth. */
int crt_measure_read(crt_context* ctx, const void* buf, size_t bytes, uint32_t reps, double* ms_per_pass);

/* Page-locked host memory for outputs (no counterpart in the reference): device-to-host copies
 * into such buffers run at the full host link rate instead of through a pageable bounce buffer.
 * The pybind11 module hands its result arrays out of a pool of these. */
int crt_host_alloc(size_t bytes, void** out);
int crt_host_free(void* ptr);

/* ---------------------------------------------------------------- serving
 * A request loop over resident scenes (no counterpart in the reference, which renders one camera per
 * call), with continuous batching: requests are submitted from any thread and queued; each of
 * `lanes` lanes (own stream, own wave engine) admits them in arrival order while their device state
 * fits its budget, and runs one wavefront wave at a time over all of its resident requests,
 * shortest remaining work first; an SRP query's sun rays ride in the waves' primary traces, one range
 * of its items per wave (as in crt_batch_mixed).  A request that arrives while others are on the GPU joins the next
 * wave and leaves when its own last wave is done.  Results equal the same requests run alone. */
typedef struct crt_server crt_server;
enum { CRT_REQUEST_SRP = 2 };
typedef struct {
    uint32_t lanes;                       /* concurrent lanes, 1..8 */
    size_t lane_budget_bytes;             /* device memory per lane: one wave's path buffers + request state */
    uint32_t max_batch;                   /* resident requests per lane */
    uint32_t count_rays;                  /* 1: lanes run the counting build (crt_server_stats.rays) */
    uint32_t wave_paths;                  /* camera paths per wave (0: 4194304; >= 65536) */
} crt_server_config;
typedef struct {
    crt_request base;                     /* kind RENDER or LIDAR: as for crt_batch; kind SRP: below */
    const crt_srp_desc* srp;
    const double* quaternions;            /* n_att * 4, host memory */
    size_t n_att;
    double* force;                        /* n_att * 3 */
    double* torque;                       /* n_att * 3 */
} crt_server_request;
/* Mixed batch (no counterpart in the reference, which renders one camera per call and names SRP only
 * in its README): render, LiDAR and SRP requests in one call, given as crt_server_request (kind SRP:
 * srp / quaternions / n_att / force / torque; quaternions and outputs host or device memory).  The
 * SRP requests' sun rays ride in the waves' primary trace launches beside the camera paths and LiDAR
 * beams (one shared ray queue), each wave carrying a range of one SRP request's items, and that
 * range's shade and specular segments follow in the same wave.  Render and LiDAR results equal
 * crt_batch's; force and torque equal crt_srp's bit for bit (partial sums are kept per block of the
 * request's items, whatever the waves).  Waves that carry SRP items are launched one by one (no
 * CUDA-graph replay). */
int crt_batch_mixed(crt_context* ctx, const crt_server_request* requests, size_t n, crt_batch_stats* stats);

typedef struct {
    int status;                           /* CRT_OK or the failure of the wave that ran it */
    double submit_s, start_s, end_s;      /* steady-clock seconds: submitted, admitted, completed */
    uint32_t batch_size;                  /* requests resident in the lane during its last wave */
} crt_server_result;
typedef struct {
    uint64_t submitted, completed, batches, failed;   /* batches: waves run */
    uint64_t rays;                        /* rays of completed batches, traversed or resolved without a
                                             traversal (count_rays only) */
    double busy_s;                        /* summed lane time */
} crt_server_stats;

/* Lanes own their contexts.  Requests name scenes built on any context of the same device (the
 * lanes only read a scene's arrays), so the caller can keep using those scenes directly; scenes
 * must outlive every request that names them. */
int crt_server_create(int device, const crt_server_config* config, crt_server** out);
/* Stops the lanes after the queued requests finish. */
int crt_server_destroy(crt_server* server);
/* Copies the request's descriptors; outputs must stay valid until the request completes.  Rejects
 * malformed requests at once (CRT_ERR_INVALID); crt_server_last_error then holds the reason. */
int crt_server_submit(crt_server* server, const crt_server_request* request, uint64_t* ticket);
/* Message of the calling thread's last failed crt_server_submit. */
const char* crt_server_last_error(void);
/* Waits up to timeout_s (negative: forever) for a ticket; CRT_ERR_TIMEOUT when it has not finished.
 * A ticket's result is collected once: CRT_ERR_INVALID for a ticket never issued or already collected. */
int crt_server_wait(crt_server* server, uint64_t ticket, double timeout_s, crt_server_result* out);
int crt_server_get_stats(crt_server* server, crt_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif
