/* CPU oracle for the CRT ray-query path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference (ceres-navigation/ceres-raytracer v0.6a4)
 * algorithms on the ray-query path.  The CUDA library is tested against it: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.  Nothing in the
 * product links or calls it.
 *
 * Pinning: tests/golden/ holds fixtures produced by the reference itself (compiled from its own
 * sources by oracle/build_ref.py); tests/test_oracle_golden.py checks this oracle against them.
 * The radiation-pressure integrator has no counterpart in the reference, so its parity is
 * unpinned (analytic known answers only).
 */
#ifndef CRT_ORACLE_H
#define CRT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One entity placed in a scene (rendering_dynamic/entity.hpp:21-86 + its pose). */
typedef struct {
    const float* tri_xyz;   /* n_tris * 9: p0, p1, p2 as loaded (float32, obj.hpp:78-80) */
    const double* tri_vn;   /* n_tris * 9 vertex normals (obj.hpp:108-114) or NULL (zeros) */
    size_t n_tris;
    double scale;
    double position[3];
    double rotation[9];     /* row-major */
    float color[3];
    int smooth_shading;
    uint32_t id;
    double rho_s, rho_d;    /* specular / diffuse coefficients (radiation pressure only) */
} oracle_entity;

typedef struct oracle_scene oracle_scene;

typedef struct {
    double position[3];
    double rotation[9];
    double focal_length;
    double resolution[2];
    double sensor_size[2];
    int z_positive;
} oracle_camera;

typedef struct {
    int type;               /* 0 = PointLight, 1 = AreaLight */
    double intensity;
    double position[3];
    double rotation[9];
    double size[2];
} oracle_light;

typedef struct {
    int min_samples, max_samples;
    double noise_threshold;
    int num_bounces;
    uint64_t seed;
    uint32_t request;
} oracle_render_params;

typedef struct {
    double sun_dir[3];      /* unit vector from the body toward the sun, body frame */
    double flux;            /* W / m^2 */
    double c;               /* speed of light, m / s */
    double center[3];       /* centre of the ray grid (body frame) */
    double half_extent;     /* half side of the square ray grid */
    double center_of_mass[3];
    uint32_t grid;          /* grid x grid rays */
    uint32_t num_bounces;   /* specular continuation segments after the primary hit */
} oracle_srp_params;

oracle_scene* oracle_scene_create(const oracle_entity* ents, uint32_t n_ents, int nthreads);
void oracle_scene_destroy(oracle_scene* s);
size_t oracle_scene_num_tris(const oracle_scene* s);
size_t oracle_scene_num_nodes(const oracle_scene* s);
/* transformed FP64 triangle data: p0, e1, e2, n (12 doubles per triangle) */
const double* oracle_scene_tris(const oracle_scene* s);

/* rays: n * 8 doubles (ox, oy, oz, dx, dy, dz, tmin, tmax) */
void oracle_trace_closest(const oracle_scene* s, const double* rays, size_t n, int64_t* prim,
                          double* t, double* u, double* v, int nthreads);
void oracle_trace_any(const oracle_scene* s, const double* rays, size_t n, uint8_t* occluded, int nthreads);

/* camera rays for pixels of rows [row0, row1): n*8 doubles, pixel (i, j) at index (j-row0)*W + i */
void oracle_camera_rays(const oracle_camera* cam, uint32_t row0, uint32_t row1, double* rays);

/* primary-ray passes over rows [row0, row1) (passes.hpp); any output may be NULL */
void oracle_passes(const oracle_scene* s, const oracle_camera* cam, uint32_t row0, uint32_t row1,
                   double* xyz, uint32_t* ids, double* normals, int64_t* prim, int nthreads);

/* per-pose boresight lidar (do_lidar.hpp:80-155): one range per pose, 0 on miss */
void oracle_lidar_batch(const oracle_scene* s, const double* positions, const double* rotations, size_t n,
                        int z_positive, double* range, int64_t* prim, int nthreads);

/* unidirectional path tracer over rows [row0, row1): radiance n*4 floats, rgba8 n*4 bytes; m2 (may be
 * NULL) n*3 Welford sums of squared deviations of each pixel's path samples (FP64), for statistics */
void oracle_render(const oracle_scene* s, const oracle_camera* cam, const oracle_light* lights, uint32_t n_lights,
                   const oracle_render_params* p, uint32_t row0, uint32_t row1, float* radiance,
                   uint8_t* rgba8, uint32_t* samples_taken, double* m2, int nthreads);

/* radiation pressure for one attitude (sun direction already in the body frame) over grid rows
 * [row0, row1): force[3], torque[3] (N, N m), facet_power[n_tris] (W, accumulated, caller zeroes) */
void oracle_srp(const oracle_scene* s, const oracle_srp_params* p, uint32_t row0, uint32_t row1,
                double* force, double* torque, double* facet_power, int nthreads);

/* Philox4x32-10 counter-based generator shared with the CUDA library */
void oracle_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
