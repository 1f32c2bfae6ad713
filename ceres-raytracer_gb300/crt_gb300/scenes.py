"""Seeded synthetic scenes for the ray-query path (the reference ships no scene assets).

* `cornell()`   36-triangle Cornell box: five unit-cube walls, a short and a tall box rotated
                -/+18 deg about y, a 0.25 x 0.25 ceiling light quad; six entities (ids 1..6).
* `asteroid()`  icosphere, seeded random edge collapse, 6-octave value-noise displacement
                (generated by libcrt_scene.so, see csrc/scenes.cpp).
* `spacecraft()` box bus 2 x 2 x 3 m, two 1 x 6 m panels, 2 m parabolic dish (64 x 64 radial
                mesh); ~50k triangles; per-entity specular/diffuse coefficients.

Meshes are indexed float32 vertices + int32 faces, counter-clockwise seen from the side that
faces the viewer, so the reference's left-handed triangle normal cross(p0-p1, p2-p0) points
away from the viewer as the reference expects (lib/bvh/triangle.hpp:39).
Only +, -, *, / and sqrt are used, so every host produces the same bits.
"""
import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import PKG_DIR

F32 = np.float32


@dataclass
class Mesh:
    vertices: np.ndarray   # [V, 3] float32
    faces: np.ndarray      # [F, 3] int32

    @property
    def n_tris(self):
        return int(self.faces.shape[0])

    def soup(self):
        """[F, 9] float32: p0, p1, p2 per triangle."""
        return np.ascontiguousarray(self.vertices[self.faces].reshape(-1, 9), dtype=F32)

    def vertex_normals(self):
        """Per-vertex normals as the reference OBJ loader computes them (obj.hpp:86-114):
        sum of left-handed face normals cross(p0-p1, p2-p0) of the incident faces, normalised."""
        p = self.vertices.astype(np.float64)[self.faces]
        n = np.cross(p[:, 0] - p[:, 1], p[:, 2] - p[:, 0])
        acc = np.zeros((self.vertices.shape[0], 3))
        for k in range(3):
            np.add.at(acc, self.faces[:, k], n)
        inv = 1.0 / np.sqrt((acc * acc).sum(1))
        return acc * inv[:, None]

    def soup_normals(self):
        """[F, 9] float64 vertex normals per triangle corner."""
        return np.ascontiguousarray(self.vertex_normals()[self.faces].reshape(-1, 9))

    def write_obj(self, path):
        with open(path, "w") as f:
            for v in self.vertices:
                f.write("v %.9g %.9g %.9g\n" % (v[0], v[1], v[2]))
            for t in self.faces:
                f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


@dataclass
class EntitySpec:
    name: str
    mesh: Mesh
    color: tuple = (1.0, 1.0, 1.0)
    smooth: bool = False
    scale: float = 1.0
    position: np.ndarray = field(default_factory=lambda: np.zeros(3))
    rotation: np.ndarray = field(default_factory=lambda: np.eye(3))
    rho_s: float = 0.0
    rho_d: float = 0.0


def quad_mesh(p0, p1, p2, p3):
    """Quad p0-p1-p2-p3 (counter-clockwise seen from its front) as two triangles."""
    v = np.array([p0, p1, p2, p3], dtype=np.float64).astype(F32)
    return Mesh(v, np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32))


def merge(meshes):
    vs, fs, off = [], [], 0
    for m in meshes:
        vs.append(m.vertices)
        fs.append(m.faces + off)
        off += m.vertices.shape[0]
    return Mesh(np.concatenate(vs).astype(F32), np.concatenate(fs).astype(np.int32))


def box_mesh(center, size, c, s):
    """Axis-aligned box of size (sx, sy, sz) rotated about +y by the angle with cosine c and sine s,
    faces counter-clockwise seen from outside."""
    hx, hy, hz = size[0] / 2.0, size[1] / 2.0, size[2] / 2.0
    corners = []
    for x in (-hx, hx):
        for y in (-hy, hy):
            for z in (-hz, hz):
                # rotation about y: x' = c x + s z, z' = -s x + c z
                corners.append((center[0] + (c * x + s * z), center[1] + y, center[2] + (-s * x + c * z)))
    v = np.array(corners, dtype=np.float64).astype(F32)
    # index = 4*ix + 2*iy + iz
    quads = [(0, 1, 3, 2), (4, 6, 7, 5),      # -x, +x
             (0, 4, 5, 1), (2, 3, 7, 6),      # -y, +y
             (0, 2, 6, 4), (1, 5, 7, 3)]      # -z, +z
    f = []
    for a, b, cc, d in quads:
        f += [[a, b, cc], [a, cc, d]]
    return Mesh(v, np.array(f, dtype=np.int32))


# cos / sin of 18 degrees from radicals: cos 18 = sqrt(10 + 2 sqrt 5) / 4, sin 18 = (sqrt 5 - 1) / 4
_SQRT5 = np.sqrt(5.0)
COS18 = float(np.sqrt(10.0 + 2.0 * _SQRT5) / 4.0)
SIN18 = float((_SQRT5 - 1.0) / 4.0)
TAN20 = 0.36397023426620234   # tan(20 deg), double literal


def cornell():
    """The Cornell-box scene: (entities, camera dict, lights list)."""
    white, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    floor = quad_mesh((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0))
    ceiling = quad_mesh((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1))
    back = quad_mesh((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    left = quad_mesh((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1))
    right = quad_mesh((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0))
    short_box = box_mesh((0.68, 0.15, 0.62), (0.3, 0.3, 0.3), COS18, -SIN18)
    tall_box = box_mesh((0.33, 0.3, 0.35), (0.3, 0.6, 0.3), COS18, SIN18)
    y = 0.999
    light_quad = quad_mesh((0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625))
    ents = [EntitySpec("walls", merge([floor, ceiling, back]), white),
            EntitySpec("left", left, red),
            EntitySpec("right", right, green),
            EntitySpec("short_box", short_box, white),
            EntitySpec("tall_box", tall_box, white),
            EntitySpec("light_quad", light_quad, white)]
    focal = 0.035
    camera = dict(focal_length=focal, resolution=[256, 256], sensor_size=[2 * focal * TAN20] * 2,
                  z_positive=False, position=np.array([0.5, 0.5, 2.4]), rotation=np.eye(3))
    light_rot = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]])   # local z -> world -y
    lights = [dict(type="area", intensity=15.0, size=[0.25, 0.25], position=np.array([0.5, 0.99, 0.5]),
                   rotation=light_rot)]
    return ents, camera, lights


_scene_lib = None


def _lib():
    global _scene_lib
    if _scene_lib is None:
        path = os.path.join(PKG_DIR, "libcrt_scene.so")
        if not os.path.exists(path):
            from .build import build
            build()
        lib = ctypes.CDLL(path)
        lib.crt_scene_asteroid.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                           ctypes.POINTER(ctypes.c_size_t)]
        lib.crt_scene_asteroid.restype = ctypes.c_int
        _scene_lib = lib
    return _scene_lib


def write_obj_fast(mesh, path):
    """Write a mesh as OBJ through the C writer ('%.9g', float32 round trip)."""
    lib = _lib()
    v = np.ascontiguousarray(mesh.vertices, dtype=np.float32)
    f = np.ascontiguousarray(mesh.faces, dtype=np.int32)
    lib.crt_obj_write.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
    rc = lib.crt_obj_write(path.encode(), v.ctypes.data, v.shape[0], f.ctypes.data, f.shape[0])
    if rc != 0:
        raise OSError(f"crt_obj_write failed ({rc}) for {path}")


def asteroid_level_for(target_faces):
    """Smallest icosphere level with at least 2.5x the target face count (9 for 2M, 10 for 8M)."""
    level = 0
    while 20 * 4 ** level < 2.5 * target_faces:
        level += 1
    return level


def asteroid(target_faces=2_000_000, level=None, radius=1000.0, amplitude=0.05, octaves=6, seed=0):
    """Procedural asteroid mesh (see csrc/scenes.cpp)."""
    if level is None:
        level = asteroid_level_for(target_faces)
    if target_faces >= 20 * 4 ** level:
        target_faces = 0
    lib = _lib()
    nv, nf = ctypes.c_size_t(), ctypes.c_size_t()
    # closed genus-0 triangle mesh: V - E + F = 2 with E = 3F/2, so V = F/2 + 2 (one generator call)
    cap_f = target_faces or 20 * 4 ** level
    cap_v = cap_f // 2 + 2
    v = np.empty((cap_v, 3), dtype=F32)
    f = np.empty((cap_f, 3), dtype=np.int32)
    rc = lib.crt_scene_asteroid(level, target_faces, radius, amplitude, octaves, seed, v.ctypes.data, cap_v,
                                f.ctypes.data, cap_f, ctypes.byref(nv), ctypes.byref(nf))
    if rc != 0:
        raise RuntimeError(f"crt_scene_asteroid failed ({rc})")
    return Mesh(np.ascontiguousarray(v[:nv.value]), np.ascontiguousarray(f[:nf.value]))


def cached_asteroid(target_faces=2_000_000, seed=0, cache_dir=None, **kw):
    """asteroid() with an on-disk cache (the 2M-triangle mesh takes seconds to generate)."""
    cache_dir = cache_dir or os.environ.get("CRT_SCENE_CACHE", "/tmp/crt_scene_cache")
    os.makedirs(cache_dir, exist_ok=True)
    key = "asteroid_%d_%d_%s.npz" % (target_faces, seed, "_".join(f"{k}{v}" for k, v in sorted(kw.items())))
    path = os.path.join(cache_dir, key)
    if os.path.exists(path):
        d = np.load(path)
        return Mesh(d["v"], d["f"])
    m = asteroid(target_faces, seed=seed, **kw)
    tmp = path + ".tmp.npz"
    np.savez(tmp, v=m.vertices, f=m.faces)
    os.replace(tmp, path)
    return m


def look_at(position, target, up=(0.0, 0.0, 1.0)):
    """Rotation matrix for a camera (z_positive=False) at `position` looking at `target`.

    The reference turns camera-frame directions into world directions with the transpose of the
    stored rotation (cameras/simple_camera.hpp:71-75), and its boresight is -z when z_positive is
    false, so the rows of R are the camera right, up and backward axes in world coordinates."""
    p, t, u = (np.asarray(a, dtype=np.float64) for a in (position, target, up))
    fwd = t - p
    fwd = fwd / np.sqrt(fwd @ fwd)
    right = np.cross(fwd, u)
    if (right @ right) < 1e-20:
        right = np.cross(fwd, np.array([1.0, 0.0, 0.0]))
    right = right / np.sqrt(right @ right)
    cam_up = np.cross(right, fwd)
    return np.array([right, cam_up, -fwd])


def fov_camera(fov_deg_tan_half, resolution, position, target, up=(0.0, 0.0, 1.0), focal=1.0):
    """Camera dict with tan(fov/2) given directly (no trigonometry, for bit-stable constants)."""
    s = 2.0 * focal * fov_deg_tan_half
    return dict(focal_length=focal, resolution=list(resolution), sensor_size=[s, s], z_positive=False,
                position=np.asarray(position, dtype=np.float64), rotation=look_at(position, target, up))


TAN5 = 0.087488663525924   # tan(5 deg)


def unit_vector(seed):
    """Uniform random unit vector from a seed (integer hash, no trigonometry)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    while True:
        v = rng.uniform(-1.0, 1.0, 3)
        n2 = v @ v
        if 1e-6 < n2 <= 1.0:
            return v / np.sqrt(n2)


def grid_mesh(origin, ax, ay, nx, ny, flip=False):
    """Planar nx x ny grid of quads spanning origin + [0,1]*ax + [0,1]*ay."""
    o, ax, ay = (np.asarray(a, dtype=np.float64) for a in (origin, ax, ay))
    i = np.arange(nx + 1) / nx
    j = np.arange(ny + 1) / ny
    v = o[None, None] + i[:, None, None] * ax[None, None] + j[None, :, None] * ay[None, None]
    v = v.reshape(-1, 3).astype(F32)
    idx = lambda a, b: a * (ny + 1) + b
    a, b = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    a, b = a.ravel(), b.ravel()
    q0, q1, q2, q3 = idx(a, b), idx(a + 1, b), idx(a + 1, b + 1), idx(a, b + 1)
    if flip:
        q1, q3 = q3, q1
    f = np.concatenate([np.stack([q0, q1, q2], 1), np.stack([q0, q2, q3], 1)]).astype(np.int32)
    return Mesh(v, f)


def spacecraft(bus_cell=0.05, panel_cell=0.04, dish_rings=64, dish_segments=64):
    """Spacecraft for the radiation-pressure workload: entities with specular/diffuse coefficients
    (bus and dish 0.1 / 0.5, panels 0.3 / 0.2)."""
    nb = lambda L: max(1, int(round(L / bus_cell)))
    hx, hy, hz = 1.0, 1.0, 1.5
    faces = [
        grid_mesh((hx, -hy, -hz), (0, 2 * hy, 0), (0, 0, 2 * hz), nb(2 * hy), nb(2 * hz)),           # +x
        grid_mesh((-hx, -hy, -hz), (0, 0, 2 * hz), (0, 2 * hy, 0), nb(2 * hz), nb(2 * hy)),          # -x
        grid_mesh((-hx, hy, -hz), (0, 0, 2 * hz), (2 * hx, 0, 0), nb(2 * hz), nb(2 * hx)),           # +y
        grid_mesh((-hx, -hy, -hz), (2 * hx, 0, 0), (0, 0, 2 * hz), nb(2 * hx), nb(2 * hz)),          # -y
        grid_mesh((-hx, -hy, hz), (2 * hx, 0, 0), (0, 2 * hy, 0), nb(2 * hx), nb(2 * hy)),           # +z
        grid_mesh((-hx, -hy, -hz), (0, 2 * hy, 0), (2 * hx, 0, 0), nb(2 * hy), nb(2 * hx)),          # -z
    ]
    bus = merge(faces)
    npx, npy = int(round(1.0 / panel_cell)), int(round(6.0 / panel_cell))
    panel_a = grid_mesh((-0.5, 1.2, 0.0), (1.0, 0, 0), (0, 6.0, 0), npx, npy)
    panel_b = grid_mesh((-0.5, -7.2, 0.0), (1.0, 0, 0), (0, 6.0, 0), npx, npy)
    # parabolic dish z = z0 + r^2 / (4 F), radius 1 m, rings x segments, apex at the centre
    F, z0 = 0.6, hz + 0.1
    r = np.arange(1, dish_rings + 1) / dish_rings
    # unit circle points from a regular polygon built by repeated rotation (no libm trigonometry)
    c1 = np.cos(2 * np.pi / dish_segments)
    s1 = np.sin(2 * np.pi / dish_segments)
    ang = np.empty((dish_segments, 2))
    ang[0] = (1.0, 0.0)
    for k in range(1, dish_segments):
        ang[k] = (ang[k - 1, 0] * c1 - ang[k - 1, 1] * s1, ang[k - 1, 0] * s1 + ang[k - 1, 1] * c1)
    pts = [(0.0, 0.0, z0)]
    for ri in r:
        for k in range(dish_segments):
            pts.append((ri * ang[k, 0], ri * ang[k, 1], z0 + ri * ri / (4 * F)))
    v = np.array(pts).astype(F32)
    f = []
    ring = lambda i, k: 1 + i * dish_segments + (k % dish_segments)
    for k in range(dish_segments):
        f.append([0, ring(0, k), ring(0, k + 1)])
    for i in range(dish_rings - 1):
        for k in range(dish_segments):
            a, b, c, d = ring(i, k), ring(i + 1, k), ring(i + 1, k + 1), ring(i, k + 1)
            f += [[a, b, c], [a, c, d]]
    dish = Mesh(v, np.array(f, dtype=np.int32))
    return [EntitySpec("bus", bus, (0.5, 0.5, 0.5), rho_s=0.1, rho_d=0.5),
            EntitySpec("panel_a", panel_a, (0.1, 0.1, 0.4), rho_s=0.3, rho_d=0.2),
            EntitySpec("panel_b", panel_b, (0.1, 0.1, 0.4), rho_s=0.3, rho_d=0.2),
            EntitySpec("dish", dish, (0.8, 0.8, 0.8), rho_s=0.1, rho_d=0.5)]


def quaternion_to_matrix(q):
    """Rotation matrix (body -> inertial) of a unit quaternion (w, x, y, z)."""
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def random_quaternions(n, seed):
    """n uniform random unit quaternions (w, x, y, z), normalised Gaussian 4-vectors."""
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.standard_normal((n, 4))
    q /= np.sqrt((q * q).sum(1))[:, None]
    return q
