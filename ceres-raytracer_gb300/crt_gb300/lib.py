"""ctypes binding of libcrt_gpu.so: every entry point declared in include/crt_gpu.h.

This is the raw C ABI as a foreign caller sees it (plain pointers and sizes).  Arrays may be
numpy arrays (host memory) or torch CUDA tensors (device memory); the library detects which.
Raises `CrtError` for any non-zero status.  There is no CPU fallback: loading fails loudly when
the shared library is missing, and every compute call needs a GB300.
"""
import ctypes
import os

import numpy as np

from . import PKG_DIR

LIB_PATH = os.path.join(PKG_DIR, "libcrt_gpu.so")

CRT_OK = 0
CRT_MISS = 0xFFFFFFFF

vp = ctypes.c_void_p
sz = ctypes.c_size_t
u32 = ctypes.c_uint32
i32 = ctypes.c_int
dbl = ctypes.c_double


class CrtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class EntityDesc(ctypes.Structure):
    _fields_ = [("tri_xyz", vp), ("tri_vn", vp), ("n_tris", sz), ("scale", dbl), ("position", dbl * 3),
                ("rotation", dbl * 9), ("color", ctypes.c_float * 3), ("smooth_shading", i32), ("id", u32),
                ("rho_s", ctypes.c_float), ("rho_d", ctypes.c_float)]


class CameraDesc(ctypes.Structure):
    _fields_ = [("position", dbl * 3), ("rotation", dbl * 9), ("focal_length", dbl), ("resolution", dbl * 2),
                ("sensor_size", dbl * 2), ("z_positive", i32)]


class LightDesc(ctypes.Structure):
    _fields_ = [("type", i32), ("intensity", dbl), ("position", dbl * 3), ("rotation", dbl * 9), ("size", dbl * 2)]


class RenderParams(ctypes.Structure):
    _fields_ = [("min_samples", i32), ("max_samples", i32), ("noise_threshold", dbl), ("num_bounces", i32),
                ("seed", ctypes.c_uint64), ("request", u32)]


class LidarGridDesc(ctypes.Structure):
    _fields_ = [("position", dbl * 3), ("rotation", dbl * 9), ("z_positive", i32), ("nx", u32), ("ny", u32),
                ("half_angle_x", dbl), ("half_angle_y", dbl)]


class SrpDesc(ctypes.Structure):
    _fields_ = [("sun_dir_inertial", dbl * 3), ("flux", dbl), ("c", dbl), ("center_of_mass", dbl * 3),
                ("grid", u32), ("num_bounces", u32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", i32), ("scene", vp), ("camera", ctypes.POINTER(CameraDesc)), ("lights", vp),
                ("n_lights", u32), ("params", ctypes.POINTER(RenderParams)), ("rgba8", vp), ("radiance", vp),
                ("lidar", ctypes.POINTER(LidarGridDesc)), ("range", vp), ("prim", vp)]


class BatchStats(ctypes.Structure):
    _fields_ = [("waves", sz), ("render_paths", ctypes.c_uint64), ("lidar_beams", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    _fields_ = [("queue_chunk", u32), ("wave_paths", u32), ("use_graphs", i32), ("build_sah", i32),
                ("collapse_tri_cost", ctypes.c_float), ("treelet_passes", u32)]


REQUEST_RENDER, REQUEST_LIDAR, REQUEST_SRP = 0, 1, 2


class ServerConfig(ctypes.Structure):
    _fields_ = [("lanes", u32), ("lane_budget_bytes", sz), ("max_batch", u32), ("count_rays", u32),
                ("wave_paths", u32)]


class ServerRequest(ctypes.Structure):
    _fields_ = [("base", Request), ("srp", ctypes.POINTER(SrpDesc)), ("quaternions", vp), ("n_att", sz),
                ("force", vp), ("torque", vp)]


class ServerResult(ctypes.Structure):
    _fields_ = [("status", i32), ("submit_s", dbl), ("start_s", dbl), ("end_s", dbl), ("batch_size", u32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("rays", ctypes.c_uint64), ("busy_s", dbl)]


class SceneStats(ctypes.Structure):
    _fields_ = [("n_tris", sz), ("n_nodes", sz), ("n_entities", sz), ("depth", u32), ("build_ms", dbl),
                ("device_bytes", sz), ("bounds", ctypes.c_float * 6)]


class Counters(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("nodes", ctypes.c_uint64), ("tris", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("resolved", ctypes.c_uint64)]


RAY_DTYPE = np.dtype([("o", np.float32, 3), ("tmin", np.float32), ("d", np.float32, 3), ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim", np.uint32)])

# name -> (argtypes, restype)
SIGNATURES = {
    "crt_abi_version": ([], i32),
    "crt_status_string": ([i32], ctypes.c_char_p),
    "crt_context_create": ([i32, ctypes.POINTER(vp)], i32),
    "crt_context_destroy": ([vp], i32),
    "crt_context_set_stream": ([vp, vp], i32),
    "crt_context_get_stream": ([vp], vp),
    "crt_context_synchronize": ([vp], i32),
    "crt_measure_read": ([vp, vp, sz, u32, ctypes.POINTER(dbl)], i32),
    "crt_context_set_counting": ([vp, i32], i32),
    "crt_context_get_counters": ([vp, ctypes.POINTER(Counters)], i32),
    "crt_context_reset_counters": ([vp], i32),
    "crt_context_last_error": ([vp], ctypes.c_char_p),
    "crt_mesh_load_obj": ([ctypes.c_char_p, ctypes.POINTER(vp)], i32),
    "crt_mesh_num_tris": ([vp], sz),
    "crt_mesh_xyz": ([vp], vp),
    "crt_mesh_normals": ([vp], vp),
    "crt_mesh_destroy": ([vp], None),
    "crt_scene_create": ([vp, vp, u32, ctypes.POINTER(vp)], i32),
    "crt_scene_destroy": ([vp], i32),
    "crt_scene_get_stats": ([vp, ctypes.POINTER(SceneStats)], i32),
    "crt_trace_closest": ([vp, vp, sz, vp], i32),
    "crt_trace_any": ([vp, vp, sz, vp], i32),
    "crt_passes": ([vp, ctypes.POINTER(CameraDesc), vp, vp, vp], i32),
    "crt_lidar_batch": ([vp, vp, vp, sz, i32, vp, vp], i32),
    "crt_lidar_grid": ([vp, ctypes.POINTER(LidarGridDesc), vp, vp], i32),
    "crt_render": ([vp, ctypes.POINTER(CameraDesc), vp, u32, ctypes.POINTER(RenderParams), vp, vp], i32),
    "crt_srp": ([vp, ctypes.POINTER(SrpDesc), vp, sz, vp, vp, vp], i32),
    "crt_srp_static": ([vp, ctypes.POINTER(SrpDesc), vp, sz, vp, vp], i32),
    "crt_batch": ([vp, vp, sz, ctypes.POINTER(BatchStats)], i32),
    "crt_batch_mixed": ([vp, vp, sz, ctypes.POINTER(BatchStats)], i32),
    "crt_context_set_tuning": ([vp, ctypes.POINTER(Tuning)], i32),
    "crt_context_get_tuning": ([vp, ctypes.POINTER(Tuning)], i32),
    "crt_host_alloc": ([sz, ctypes.POINTER(vp)], i32),
    "crt_host_free": ([vp], i32),
    "crt_server_create": ([i32, ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)], i32),
    "crt_server_destroy": ([vp], i32),
    "crt_server_last_error": ([], ctypes.c_char_p),
    "crt_server_submit": ([vp, ctypes.POINTER(ServerRequest), ctypes.POINTER(ctypes.c_uint64)], i32),
    "crt_server_wait": ([vp, ctypes.c_uint64, dbl, ctypes.POINTER(ServerResult)], i32),
    "crt_server_get_stats": ([vp, ctypes.POINTER(ServerStats)], i32),
}

_lib = None


def load():
    """Load libcrt_gpu.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: build the CUDA library first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def ptr(a):
    """Data pointer of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def fill_camera(cam):
    c = CameraDesc()
    c.position[:] = [float(x) for x in np.asarray(cam["position"], dtype=np.float64).ravel()]
    c.rotation[:] = [float(x) for x in np.asarray(cam["rotation"], dtype=np.float64).ravel()]
    c.focal_length = float(cam["focal_length"])
    c.resolution[:] = [float(x) for x in cam["resolution"]]
    c.sensor_size[:] = [float(x) for x in cam["sensor_size"]]
    c.z_positive = int(bool(cam.get("z_positive", False)))
    return c


def fill_srp_request(q, sr, outputs, keep):
    """Fills the SRP fields of a ServerRequest from a request dict ({"sun_dir", "quaternions", "grid",
    "num_bounces", "flux", "c", "center_of_mass"}); returns the (force, torque) outputs."""
    d = SrpDesc()
    d.sun_dir_inertial[:] = [float(x) for x in q["sun_dir"]]
    d.flux, d.c = float(q.get("flux", 1361.0)), float(q.get("c", 299792458.0))
    d.center_of_mass[:] = [float(x) for x in q.get("center_of_mass", (0.0, 0.0, 0.0))]
    d.grid, d.num_bounces = int(q["grid"]), int(q.get("num_bounces", 2))
    quats = np.ascontiguousarray(q["quaternions"], dtype=np.float64).reshape(-1, 4)
    out = outputs or (np.empty((len(quats), 3)), np.empty((len(quats), 3)))
    keep += [d, quats]
    sr.base.kind = REQUEST_SRP
    sr.base.scene = q["scene"].h
    sr.srp, sr.quaternions, sr.n_att = ctypes.pointer(d), quats.ctypes.data, len(quats)
    sr.force, sr.torque = ptr(out[0]), ptr(out[1])
    return out


def fill_lights(lights):
    arr = (LightDesc * max(1, len(lights)))()
    for i, l in enumerate(lights):
        arr[i].type = 1 if l["type"] == "area" else 0
        arr[i].intensity = float(l["intensity"])
        arr[i].position[:] = [float(x) for x in np.asarray(l["position"], dtype=np.float64).ravel()]
        arr[i].rotation[:] = [float(x) for x in np.asarray(l.get("rotation", np.eye(3)), dtype=np.float64).ravel()]
        s = l.get("size", [0.0, 0.0])
        arr[i].size[:] = [float(s[0]), float(s[1])]
    return arr


class Context:
    """Owns a crt_context; scenes created from it are destroyed before it (the C ABI requires
    scenes to be released before their context)."""

    def __init__(self, device=0):
        import weakref
        self.L = load()
        self._scenes = weakref.WeakSet()
        self.h = None
        h = vp()
        self._check(self.L.crt_context_create(device, ctypes.byref(h)), None)
        self.h = h

    def _check(self, rc, h=-1):
        if rc != CRT_OK:
            hh = self.h if h == -1 else h
            msg = self.L.crt_context_last_error(hh).decode() if hh else self.L.crt_status_string(rc).decode()
            raise CrtError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            for s in list(self._scenes):
                s.close()
            self.L.crt_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        self._check(self.L.crt_context_set_stream(self.h, stream_handle))

    def stream_handle(self):
        """cudaStream_t of the context (an integer), e.g. for torch.cuda.ExternalStream."""
        return self.L.crt_context_get_stream(self.h) or 0

    def synchronize(self):
        self._check(self.L.crt_context_synchronize(self.h))

    def measure_read(self, buf, reps=20):
        """Mean device time (ms) of one streaming read of a device buffer (a torch tensor or a pointer
        with .nbytes): crt_measure_read."""
        ms = dbl()
        nbytes = buf.numel() * buf.element_size() if hasattr(buf, "numel") else buf.nbytes
        self._check(self.L.crt_measure_read(self.h, ptr(buf), nbytes, int(reps), ctypes.byref(ms)))
        return ms.value

    def set_counting(self, on):
        self._check(self.L.crt_context_set_counting(self.h, int(bool(on))))

    def counters(self):
        c = Counters()
        self._check(self.L.crt_context_get_counters(self.h, ctypes.byref(c)))
        # rays: traversed; resolved: answered without a traversal; answered: both
        return dict(rays=c.rays, nodes=c.nodes, tris=c.tris, launches=c.launches, resolved=c.resolved,
                    answered=c.rays + c.resolved)

    def reset_counters(self):
        self._check(self.L.crt_context_reset_counters(self.h))

    def scene(self, entities):
        return Scene(self, entities)

    def set_tuning(self, queue_chunk=1, wave_paths=1 << 23, use_graphs=True, build_sah=True, collapse_tri_cost=0.15,
                   treelet_passes=1):
        t = Tuning(int(queue_chunk), int(wave_paths), int(bool(use_graphs)), int(bool(build_sah)),
                   float(collapse_tri_cost), int(treelet_passes))
        self._check(self.L.crt_context_set_tuning(self.h, ctypes.byref(t)))

    def get_tuning(self):
        t = Tuning()
        self._check(self.L.crt_context_get_tuning(self.h, ctypes.byref(t)))
        return dict(queue_chunk=t.queue_chunk, wave_paths=t.wave_paths, use_graphs=bool(t.use_graphs),
                    build_sah=bool(t.build_sah), collapse_tri_cost=round(float(t.collapse_tri_cost), 4),
                    treelet_passes=int(t.treelet_passes))

    def batch(self, requests, outputs=None):
        """Run render / LiDAR / SRP requests in one batch.  Each request is a dict:
        {"kind": "render", "scene": Scene, "camera": cam, "lights": [...], "min_samples", "max_samples",
         "noise_threshold", "num_bounces", "seed", "request", "radiance": bool}
        {"kind": "lidar", "scene": Scene, "position", "rotation", "nx", "ny", "half_x", "half_y", "z_positive"}
        {"kind": "srp", "scene": Scene, "sun_dir", "quaternions", "grid", "num_bounces", "flux", "c",
         "center_of_mass"}
        Render / LiDAR only: crt_batch; with SRP requests: crt_batch_mixed (their sun rays share the waves'
        primary traces).  Returns (outputs, stats): outputs[i] = (rgba, radiance), (range, prim) or
        (force, torque)."""
        n = len(requests)
        mixed = any(q["kind"] == "srp" for q in requests)
        sarr = (ServerRequest * max(1, n))() if mixed else None
        arr = None if mixed else (Request * max(1, n))()
        keep, outs = [], []
        for i, q in enumerate(requests):
            r = sarr[i].base if mixed else arr[i]
            r.scene = q["scene"].h
            given = outputs[i] if outputs is not None else None
            if q["kind"] == "render":
                cam = q["camera"]
                W, H = int(np.floor(cam["resolution"][0])), int(np.floor(cam["resolution"][1]))
                c = fill_camera(cam)
                L = fill_lights(q.get("lights", []))
                p = RenderParams(int(q.get("min_samples", 1)), int(q.get("max_samples", 1)),
                                 float(q.get("noise_threshold", 1.0)), int(q.get("num_bounces", 1)),
                                 int(q.get("seed", 0)), int(q.get("request", 0)))
                rgba, rad = given if given is not None else (
                    np.empty((H, W, 4), np.uint8), np.empty((H, W, 4), np.float32) if q.get("radiance") else None)
                keep += [c, L, p]
                r.kind = REQUEST_RENDER
                r.camera = ctypes.pointer(c)
                r.lights = ctypes.cast(L, vp)
                r.n_lights = len(q.get("lights", []))
                r.params = ctypes.pointer(p)
                r.rgba8 = ptr(rgba)
                r.radiance = ptr(rad)
                outs.append((rgba, rad))
            elif q["kind"] == "srp":
                outs.append(fill_srp_request(q, sarr[i], given, keep))
            else:
                g = LidarGridDesc()
                g.position[:] = [float(x) for x in np.asarray(q["position"], dtype=np.float64).ravel()]
                g.rotation[:] = [float(x) for x in np.asarray(q["rotation"], dtype=np.float64).ravel()]
                g.z_positive = int(bool(q.get("z_positive", False)))
                g.nx, g.ny = int(q["nx"]), int(q["ny"])
                g.half_angle_x, g.half_angle_y = float(q["half_x"]), float(q["half_y"])
                rng, prim = given if given is not None else (np.empty((g.ny, g.nx)), np.empty((g.ny, g.nx), np.uint32))
                keep.append(g)
                r.kind = REQUEST_LIDAR
                r.lidar = ctypes.pointer(g)
                r.range = ptr(rng)
                r.prim = ptr(prim)
                outs.append((rng, prim))
        st = BatchStats()
        if mixed:
            self._check(self.L.crt_batch_mixed(self.h, sarr, n, ctypes.byref(st)))
        else:
            self._check(self.L.crt_batch(self.h, arr, n, ctypes.byref(st)))
        del keep
        return outs, dict(waves=st.waves, render_paths=st.render_paths, lidar_beams=st.lidar_beams)


class Scene:
    """Device-resident scene built from entity specs (objects with mesh/color/smooth/scale/position/
    rotation/rho_s/rho_d attributes, e.g. crt_gb300.scenes.EntitySpec)."""

    def __init__(self, ctx, entities, ids=None):
        self.ctx = ctx
        L = ctx.L
        arr = (EntityDesc * max(1, len(entities)))()
        keep = []
        for i, e in enumerate(entities):
            xyz = np.ascontiguousarray(e.mesh.soup(), dtype=np.float32)
            vn = np.ascontiguousarray(e.mesh.soup_normals(), dtype=np.float32) if e.smooth else None
            keep += [xyz, vn]
            arr[i].tri_xyz = xyz.ctypes.data
            arr[i].tri_vn = vn.ctypes.data if vn is not None else None
            arr[i].n_tris = xyz.shape[0]
            arr[i].scale = float(e.scale)
            arr[i].position[:] = [float(x) for x in np.asarray(e.position, dtype=np.float64).ravel()]
            arr[i].rotation[:] = [float(x) for x in np.asarray(e.rotation, dtype=np.float64).ravel()]
            arr[i].color[:] = [float(x) for x in e.color]
            arr[i].smooth_shading = int(bool(e.smooth))
            arr[i].id = (i + 1) if ids is None else int(ids[i])
            arr[i].rho_s = float(getattr(e, "rho_s", 0.0))
            arr[i].rho_d = float(getattr(e, "rho_d", 0.0))
        h = vp()
        self.h = None
        ctx._check(L.crt_scene_create(ctx.h, arr, len(entities), ctypes.byref(h)))
        self.h = h
        ctx._scenes.add(self)
        del keep

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.ctx.L.crt_scene_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        s = SceneStats()
        self.ctx._check(self.ctx.L.crt_scene_get_stats(self.h, ctypes.byref(s)))
        return dict(n_tris=s.n_tris, n_nodes=s.n_nodes, n_entities=s.n_entities, depth=s.depth, build_ms=s.build_ms,
                    device_bytes=s.device_bytes, bounds=list(s.bounds))

    def trace_closest(self, rays, out=None):
        """rays: structured RAY_DTYPE array (or [n, 8] float32); returns HIT_DTYPE array."""
        rays = np.ascontiguousarray(rays).view(RAY_DTYPE).reshape(-1) if not hasattr(rays, "data_ptr") else rays
        n = rays.shape[0]
        if out is None:
            out = np.empty(n, HIT_DTYPE)
        self.ctx._check(self.ctx.L.crt_trace_closest(self.h, ptr(rays), n, ptr(out)))
        return out

    def trace_any(self, rays, out=None):
        rays = np.ascontiguousarray(rays).view(RAY_DTYPE).reshape(-1) if not hasattr(rays, "data_ptr") else rays
        n = rays.shape[0]
        if out is None:
            out = np.empty(n, np.uint8)
        self.ctx._check(self.ctx.L.crt_trace_any(self.h, ptr(rays), n, ptr(out)))
        return out

    def passes(self, cam, xyz=True, ids=True, normals=True):
        c = fill_camera(cam)
        W, H = int(np.floor(cam["resolution"][0])), int(np.floor(cam["resolution"][1]))
        def out(a, shape, dtype=np.float64):   # True: allocate; False / None: skip; else caller buffer
            return np.empty(shape, dtype) if a is True else (None if a is None or a is False else a)
        ox = out(xyz, (H, W, 3))
        oi = out(ids, (H, W), np.uint32)
        on = out(normals, (H, W, 3))
        self.ctx._check(self.ctx.L.crt_passes(self.h, ctypes.byref(c), ptr(ox), ptr(oi), ptr(on)))
        return ox, oi, on

    def lidar_batch(self, positions, rotations, z_positive=False, want_prim=True):
        positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        rotations = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        n = positions.shape[0]
        rng = np.empty(n)
        prim = np.empty(n, np.uint32) if want_prim else None
        self.ctx._check(self.ctx.L.crt_lidar_batch(self.h, ptr(positions), ptr(rotations), n, int(bool(z_positive)),
                                                   ptr(rng), ptr(prim)))
        return rng, prim

    def lidar_grid(self, position, rotation, nx, ny, half_x, half_y, z_positive=False, out_range=None, out_prim=None):
        g = LidarGridDesc()
        g.position[:] = [float(x) for x in np.asarray(position, dtype=np.float64).ravel()]
        g.rotation[:] = [float(x) for x in np.asarray(rotation, dtype=np.float64).ravel()]
        g.z_positive = int(bool(z_positive))
        g.nx, g.ny = int(nx), int(ny)
        g.half_angle_x, g.half_angle_y = float(half_x), float(half_y)
        rng = np.empty((ny, nx)) if out_range is None else out_range
        prim = np.empty((ny, nx), np.uint32) if out_prim is None else out_prim
        self.ctx._check(self.ctx.L.crt_lidar_grid(self.h, ctypes.byref(g), ptr(rng), ptr(prim)))
        return rng, prim

    def render(self, cam, lights, min_samples=1, max_samples=1, noise_threshold=1.0, num_bounces=1, seed=0,
               request=0, want_radiance=True, out_rgba=None, out_radiance=None):
        c = fill_camera(cam)
        L = fill_lights(lights)
        p = RenderParams(int(min_samples), int(max_samples), float(noise_threshold), int(num_bounces), int(seed),
                         int(request))
        W, H = int(np.floor(cam["resolution"][0])), int(np.floor(cam["resolution"][1]))
        rgba = np.empty((H, W, 4), np.uint8) if out_rgba is None else out_rgba
        rad = (np.empty((H, W, 4), np.float32) if want_radiance else None) if out_radiance is None else out_radiance
        self.ctx._check(self.ctx.L.crt_render(self.h, ctypes.byref(c), L, len(lights), ctypes.byref(p), ptr(rgba),
                                              ptr(rad)))
        return rgba, rad

    def srp(self, sun_dir, quaternions, grid, num_bounces=2, flux=1361.0, c=299792458.0, center_of_mass=(0, 0, 0),
            facet_power=False):
        d = SrpDesc()
        d.sun_dir_inertial[:] = [float(x) for x in sun_dir]
        d.flux, d.c = float(flux), float(c)
        d.center_of_mass[:] = [float(x) for x in center_of_mass]
        d.grid, d.num_bounces = int(grid), int(num_bounces)
        q = np.ascontiguousarray(quaternions, dtype=np.float64).reshape(-1, 4)
        n = q.shape[0]
        f, t = np.empty((n, 3)), np.empty((n, 3))
        fp = np.empty((n, self.stats()["n_tris"])) if facet_power else None
        self.ctx._check(self.ctx.L.crt_srp(self.h, ctypes.byref(d), ptr(q), n, ptr(f), ptr(t), ptr(fp)))
        return f, t, fp

    def srp_into(self, sun_dir, quaternions, grid, force, torque, facet_power=None, num_bounces=2, flux=1361.0,
                 c=299792458.0, center_of_mass=(0, 0, 0)):
        """crt_srp with caller buffers (host arrays or device tensors): quaternions [n, 4] float64,
        force / torque [n, 3] float64, facet_power [n, n_tris] float64 or None."""
        d = SrpDesc()
        d.sun_dir_inertial[:] = [float(x) for x in sun_dir]
        d.flux, d.c = float(flux), float(c)
        d.center_of_mass[:] = [float(x) for x in center_of_mass]
        d.grid, d.num_bounces = int(grid), int(num_bounces)
        n = int(quaternions.shape[0])
        self.ctx._check(self.ctx.L.crt_srp(self.h, ctypes.byref(d), ptr(quaternions), n, ptr(force), ptr(torque),
                                           ptr(facet_power)))

    def srp_static_into(self, sun_dir, quaternions, grid, force, torque, num_bounces=2, flux=1361.0, c=299792458.0,
                        center_of_mass=(0, 0, 0)):
        """crt_srp_static (no device allocation; static scratch) with caller buffers, as srp_into."""
        d = SrpDesc()
        d.sun_dir_inertial[:] = [float(x) for x in sun_dir]
        d.flux, d.c = float(flux), float(c)
        d.center_of_mass[:] = [float(x) for x in center_of_mass]
        d.grid, d.num_bounces = int(grid), int(num_bounces)
        n = int(quaternions.shape[0])
        self.ctx._check(self.ctx.L.crt_srp_static(self.h, ctypes.byref(d), ptr(quaternions), n, ptr(force),
                                                  ptr(torque)))


def make_rays(o, d, tmin=0.0, tmax=3.4e38):
    """Structured FP32 ray array from [n, 3] origins and directions."""
    o, d = np.asarray(o), np.asarray(d)
    r = np.empty(o.shape[0], RAY_DTYPE)
    r["o"], r["d"] = o, d
    r["tmin"], r["tmax"] = tmin, tmax
    return r


class Server:
    """Continuous-batching request loop (crt_server_*).  Scenes are created with server.scene(...) on
    a context of the server object's own (not a lane's), so they can also be called directly while
    requests run; requests are dicts as for Context.batch plus {"kind": "srp", "scene", "sun_dir",
    "quaternions", "grid", "num_bounces", "flux", "c", "center_of_mass"}.  submit() returns a ticket;
    wait() returns (result dict, outputs)."""

    def __init__(self, device=0, lanes=2, lane_budget_bytes=4 << 30, max_batch=256, count_rays=False, wave_paths=0):
        self.L = load()
        self.h = None
        self.ctx = Context(device)
        cfg = ServerConfig(int(lanes), int(lane_budget_bytes), int(max_batch), int(bool(count_rays)), int(wave_paths))
        h = vp()
        rc = self.L.crt_server_create(int(device), ctypes.byref(cfg), ctypes.byref(h))
        if rc != CRT_OK:
            self.ctx.close()
            raise CrtError(rc, self.L.crt_status_string(rc).decode())
        self.h = h
        self._inflight = {}
        self.config = dict(lanes=int(lanes), lane_budget_bytes=int(lane_budget_bytes), max_batch=int(max_batch),
                           count_rays=bool(count_rays), wave_paths=int(wave_paths))

    def scene(self, entities):
        return Scene(self.ctx, entities)

    def submit(self, q, outputs=None):
        sr = ServerRequest()
        keep = []
        r = sr.base
        r.scene = q["scene"].h
        if q["kind"] == "render":
            cam = q["camera"]
            W, H = int(np.floor(cam["resolution"][0])), int(np.floor(cam["resolution"][1]))
            c, Ls = fill_camera(cam), fill_lights(q.get("lights", []))
            p = RenderParams(int(q.get("min_samples", 1)), int(q.get("max_samples", 1)),
                             float(q.get("noise_threshold", 1.0)), int(q.get("num_bounces", 1)), int(q.get("seed", 0)),
                             int(q.get("request", 0)))
            out = outputs or (np.empty((H, W, 4), np.uint8),
                              np.empty((H, W, 4), np.float32) if q.get("radiance") else None)
            keep += [c, Ls, p]
            r.kind, r.camera, r.lights = REQUEST_RENDER, ctypes.pointer(c), ctypes.cast(Ls, vp)
            r.n_lights, r.params = len(q.get("lights", [])), ctypes.pointer(p)
            r.rgba8, r.radiance = ptr(out[0]), ptr(out[1])
        elif q["kind"] == "lidar":
            g = LidarGridDesc()
            g.position[:] = [float(x) for x in np.asarray(q["position"], dtype=np.float64).ravel()]
            g.rotation[:] = [float(x) for x in np.asarray(q["rotation"], dtype=np.float64).ravel()]
            g.z_positive = int(bool(q.get("z_positive", False)))
            g.nx, g.ny = int(q["nx"]), int(q["ny"])
            g.half_angle_x, g.half_angle_y = float(q["half_x"]), float(q["half_y"])
            out = outputs or (np.empty((g.ny, g.nx)), np.empty((g.ny, g.nx), np.uint32))
            keep.append(g)
            r.kind, r.lidar, r.range, r.prim = REQUEST_LIDAR, ctypes.pointer(g), ptr(out[0]), ptr(out[1])
        else:
            out = fill_srp_request(q, sr, outputs, keep)
        t = ctypes.c_uint64()
        rc = self.L.crt_server_submit(self.h, ctypes.byref(sr), ctypes.byref(t))
        if rc != CRT_OK:
            raise CrtError(rc, self.L.crt_server_last_error().decode())
        self._inflight[t.value] = out
        return t.value

    def wait(self, ticket, timeout=-1.0):
        res = ServerResult()
        rc = self.L.crt_server_wait(self.h, ctypes.c_uint64(ticket), float(timeout), ctypes.byref(res))
        if rc != CRT_OK:
            raise CrtError(rc, "wait: " + self.L.crt_status_string(rc).decode())
        out = self._inflight.pop(ticket, None)
        return dict(status=res.status, submit_s=res.submit_s, start_s=res.start_s, end_s=res.end_s,
                    latency_s=res.end_s - res.submit_s, batch_size=res.batch_size), out

    def stats(self):
        s = ServerStats()
        self.L.crt_server_get_stats(self.h, ctypes.byref(s))
        return dict(submitted=s.submitted, completed=s.completed, batches=s.batches, failed=s.failed, rays=s.rays,
                    busy_s=s.busy_s)

    def close(self):
        """Finishes the queued requests, stops the lanes, then releases the scenes."""
        if getattr(self, "h", None):
            self.L.crt_server_destroy(self.h)
            self.h = None
        if getattr(self, "ctx", None) is not None:
            self.ctx.close()
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
