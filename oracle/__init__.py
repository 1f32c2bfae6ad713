"""CPU oracle for the CRT ray-query path -- TEST INFRASTRUCTURE ONLY.

ctypes binding of oracle/libcrt_oracle.so (FP64 C restatement of the reference path, see
crt_oracle.c).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package; the product never does.  Parity of the ray-query functions is pinned against fixtures
produced by the reference itself (tests/golden/); the radiation-pressure integrator has no
reference counterpart and its parity is unpinned (analytic known answers only).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcrt_oracle.so")

c_double_p = ctypes.POINTER(ctypes.c_double)


class Entity(ctypes.Structure):
    _fields_ = [("tri_xyz", ctypes.c_void_p), ("tri_vn", ctypes.c_void_p), ("n_tris", ctypes.c_size_t),
                ("scale", ctypes.c_double), ("position", ctypes.c_double * 3), ("rotation", ctypes.c_double * 9),
                ("color", ctypes.c_float * 3), ("smooth_shading", ctypes.c_int), ("id", ctypes.c_uint32),
                ("rho_s", ctypes.c_double), ("rho_d", ctypes.c_double)]


class Camera(ctypes.Structure):
    _fields_ = [("position", ctypes.c_double * 3), ("rotation", ctypes.c_double * 9),
                ("focal_length", ctypes.c_double), ("resolution", ctypes.c_double * 2),
                ("sensor_size", ctypes.c_double * 2), ("z_positive", ctypes.c_int)]


class Light(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("intensity", ctypes.c_double), ("position", ctypes.c_double * 3),
                ("rotation", ctypes.c_double * 9), ("size", ctypes.c_double * 2)]


class RenderParams(ctypes.Structure):
    _fields_ = [("min_samples", ctypes.c_int), ("max_samples", ctypes.c_int), ("noise_threshold", ctypes.c_double),
                ("num_bounces", ctypes.c_int), ("seed", ctypes.c_uint64), ("request", ctypes.c_uint32)]


class SrpParams(ctypes.Structure):
    _fields_ = [("sun_dir", ctypes.c_double * 3), ("flux", ctypes.c_double), ("c", ctypes.c_double),
                ("center", ctypes.c_double * 3), ("half_extent", ctypes.c_double),
                ("center_of_mass", ctypes.c_double * 3), ("grid", ctypes.c_uint32), ("num_bounces", ctypes.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, sz, i32, u32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32
        L.oracle_scene_create.argtypes = [vp, u32, i32]
        L.oracle_scene_create.restype = vp
        L.oracle_scene_destroy.argtypes = [vp]
        L.oracle_scene_num_tris.argtypes = [vp]
        L.oracle_scene_num_tris.restype = sz
        L.oracle_scene_num_nodes.argtypes = [vp]
        L.oracle_scene_num_nodes.restype = sz
        L.oracle_scene_tris.argtypes = [vp]
        L.oracle_scene_tris.restype = vp
        L.oracle_trace_closest.argtypes = [vp, vp, sz, vp, vp, vp, vp, i32]
        L.oracle_trace_any.argtypes = [vp, vp, sz, vp, i32]
        L.oracle_camera_rays.argtypes = [vp, u32, u32, vp]
        L.oracle_passes.argtypes = [vp, vp, u32, u32, vp, vp, vp, vp, i32]
        L.oracle_lidar_batch.argtypes = [vp, vp, vp, sz, i32, vp, vp, i32]
        L.oracle_render.argtypes = [vp, vp, vp, u32, vp, u32, u32, vp, vp, vp, vp, i32]
        L.oracle_srp.argtypes = [vp, vp, u32, u32, vp, vp, vp, i32]
        L.oracle_philox.argtypes = [u32, u32, u32, u32, u32, u32, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def make_camera(cam):
    c = Camera()
    c.position[:] = [float(x) for x in np.asarray(cam["position"], dtype=np.float64).ravel()]
    c.rotation[:] = [float(x) for x in np.asarray(cam["rotation"], dtype=np.float64).ravel()]
    c.focal_length = float(cam["focal_length"])
    c.resolution[:] = [float(x) for x in cam["resolution"]]
    c.sensor_size[:] = [float(x) for x in cam["sensor_size"]]
    c.z_positive = int(bool(cam.get("z_positive", False)))
    return c


def make_lights(lights):
    arr = (Light * max(1, len(lights)))()
    for i, l in enumerate(lights):
        arr[i].type = 1 if l["type"] == "area" else 0
        arr[i].intensity = float(l["intensity"])
        arr[i].position[:] = [float(x) for x in np.asarray(l["position"], dtype=np.float64).ravel()]
        arr[i].rotation[:] = [float(x) for x in np.asarray(l.get("rotation", np.eye(3)), dtype=np.float64).ravel()]
        sz = l.get("size", [0.0, 0.0])
        arr[i].size[:] = [float(sz[0]), float(sz[1])]
    return arr


class Scene:
    """FP64 oracle scene built from entity specs (crt_gb300.scenes.EntitySpec-like objects)."""

    def __init__(self, entities, nthreads=0, ids=None):
        self.nthreads = nthreads
        L = lib()
        self._keep = []
        arr = (Entity * len(entities))()
        for i, e in enumerate(entities):
            xyz = np.ascontiguousarray(e.mesh.soup(), dtype=np.float32)
            vn = np.ascontiguousarray(e.mesh.soup_normals(), dtype=np.float64)
            self._keep += [xyz, vn]
            arr[i].tri_xyz = xyz.ctypes.data
            arr[i].tri_vn = vn.ctypes.data
            arr[i].n_tris = xyz.shape[0]
            arr[i].scale = float(e.scale)
            arr[i].position[:] = [float(x) for x in np.asarray(e.position, dtype=np.float64).ravel()]
            arr[i].rotation[:] = [float(x) for x in np.asarray(e.rotation, dtype=np.float64).ravel()]
            arr[i].color[:] = [float(x) for x in e.color]
            arr[i].smooth_shading = int(bool(e.smooth))
            arr[i].id = (i + 1) if ids is None else ids[i]
            arr[i].rho_s = float(getattr(e, "rho_s", 0.0))
            arr[i].rho_d = float(getattr(e, "rho_d", 0.0))
        self.h = L.oracle_scene_create(arr, len(entities), nthreads)
        self._keep = None
        self.n_tris = L.oracle_scene_num_tris(self.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_scene_destroy(self.h)
            self.h = None

    def tris(self):
        p = lib().oracle_scene_tris(self.h)
        return np.ctypeslib.as_array((ctypes.c_double * (12 * self.n_tris)).from_address(p)).reshape(-1, 12).copy()

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        prim = np.empty(n, np.int64)
        t, u, v = np.empty(n), np.empty(n), np.empty(n)
        lib().oracle_trace_closest(self.h, _ptr(rays), n, _ptr(prim), _ptr(t), _ptr(u), _ptr(v), self.nthreads)
        return prim, t, u, v

    def trace_any(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        occ = np.empty(rays.shape[0], np.uint8)
        lib().oracle_trace_any(self.h, _ptr(rays), rays.shape[0], _ptr(occ), self.nthreads)
        return occ

    def passes(self, cam, row0=0, row1=None):
        c = make_camera(cam)
        W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
        row1 = H if row1 is None else row1
        n = (row1 - row0) * W
        xyz, nrm = np.empty((n, 3)), np.empty((n, 3))
        ids, prim = np.empty(n, np.uint32), np.empty(n, np.int64)
        lib().oracle_passes(self.h, ctypes.byref(c), row0, row1, _ptr(xyz), _ptr(ids), _ptr(nrm), _ptr(prim),
                            self.nthreads)
        shp = (row1 - row0, W)
        return xyz.reshape(shp + (3,)), ids.reshape(shp), nrm.reshape(shp + (3,)), prim.reshape(shp)

    def lidar_batch(self, positions, rotations, z_positive=False):
        positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        rotations = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        n = positions.shape[0]
        rng, prim = np.empty(n), np.empty(n, np.int64)
        lib().oracle_lidar_batch(self.h, _ptr(positions), _ptr(rotations), n, int(z_positive), _ptr(rng),
                                 _ptr(prim), self.nthreads)
        return rng, prim

    def render(self, cam, lights, min_samples=1, max_samples=1, noise_threshold=1.0, num_bounces=1, seed=0,
               request=0, row0=0, row1=None, with_m2=False):
        """(radiance [h, w, 4] f32, rgba8 [h, w, 4], samples taken [h, w]) and, with_m2, the Welford
        M2 [h, w, 3] (FP64) of each pixel's path samples: the sample variance is M2 / (n - 1)."""
        c = make_camera(cam)
        L = make_lights(lights)
        p = RenderParams(int(min_samples), int(max_samples), float(noise_threshold), int(num_bounces), int(seed),
                         int(request))
        W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
        row1 = H if row1 is None else row1
        n = (row1 - row0) * W
        rad = np.empty((n, 4), np.float32)
        u8 = np.empty((n, 4), np.uint8)
        taken = np.empty(n, np.uint32)
        m2 = np.empty((n, 3)) if with_m2 else None
        lib().oracle_render(self.h, ctypes.byref(c), L, len(lights), ctypes.byref(p), row0, row1, _ptr(rad), _ptr(u8),
                            _ptr(taken), _ptr(m2), self.nthreads)
        shp = (row1 - row0, W)
        out = rad.reshape(shp + (4,)), u8.reshape(shp + (4,)), taken.reshape(shp)
        return out + (m2.reshape(shp + (3,)),) if with_m2 else out

    def srp(self, params, row0=0, row1=None, facet_power=None):
        row1 = params.grid if row1 is None else row1
        f, t = np.zeros(3), np.zeros(3)
        if facet_power is None:
            facet_power = np.zeros(self.n_tris)
        lib().oracle_srp(self.h, ctypes.byref(params), row0, row1, _ptr(f), _ptr(t), _ptr(facet_power), self.nthreads)
        return f, t, facet_power


def camera_rays(cam, row0=0, row1=None):
    c = make_camera(cam)
    W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
    row1 = H if row1 is None else row1
    rays = np.empty(((row1 - row0) * W, 8))
    lib().oracle_camera_rays(ctypes.byref(c), row0, row1, _ptr(rays))
    return rays


def philox(c0, c1, c2, c3, k0, k1):
    out = np.empty(4, np.uint32)
    lib().oracle_philox(c0, c1, c2, c3, k0, k1, _ptr(out))
    return out
