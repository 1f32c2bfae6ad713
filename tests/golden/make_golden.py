"""Generate the golden fixtures in tests/golden/ from the reference implementation itself.

Run where the reference sources are available, after `python oracle/build_ref.py <reference dir>`
(or with CRT_REFERENCE_DIR set):

    python tests/golden/make_golden.py

It loads the reference's own pybind11 module `_crt` (oracle/_ref/golden/, built from
src/pybind.cpp unmodified) and oracle/_ref/golden/libref_driver.so (oracle/ref_driver.cpp over
the reference headers), runs them on small seeded scenes written as OBJ files, and stores the
scene inputs together with the reference outputs:

  cornell.npz   Cornell box (36 triangles, 6 entities): BodyFixedGroup intersection / instance /
                normal passes at 128x128, the dynamic-scene passes (rendering_dynamic path), and
                the path tracer's float radiance (mean and Welford M2) at 48x48, 512 spp, 3 bounces,
                and a deterministic 1-spp, 1-bounce point-light render.
  asteroid.npz  8000-triangle asteroid (smooth, rotated, scaled, translated) plus a flat box:
                BodyFixedGroup passes at 64x64, per-ray closest hits (primitive, t, u, v) and
                any-hit flags for seeded rays, and batch_simulate_lidar ranges for 512 poses.
  edges.npz     Cornell box: closest / any hits of edge-case rays (signed zeros, vertices and
                edges, rays in a triangle's plane, tiny and huge directions, far origins,
                inclusive and empty t ranges), BodyFixedGroup passes through two non-square
                cameras (one z_positive), batch LiDAR with the z_positive boresight, and a
                deterministic point-light render of a smooth-shaded asteroid beside a flat box.

`python tests/golden/make_golden.py edges` writes only the named fixtures.

Nothing at test time reads the reference: the tests only read these .npz files.
"""
import ctypes
import importlib.util
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "ceres-raytracer_gb300"))
from crt_gb300 import scenes  # noqa: E402

REF_DIR = os.path.join(REPO, "oracle", "_ref", "golden")


def load_ref_module():
    import sysconfig
    path = os.path.join(REF_DIR, "_crt" + sysconfig.get_config_var("EXT_SUFFIX"))
    spec = importlib.util.spec_from_file_location("_crt", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_driver():
    d = ctypes.CDLL(os.path.join(REF_DIR, "libref_driver.so"))
    vp = ctypes.c_void_p
    d.ref_scene_create.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp]
    d.ref_scene_create.restype = vp
    d.ref_num_tris.argtypes = [vp]
    d.ref_num_tris.restype = ctypes.c_size_t
    d.ref_tris.argtypes = [vp, vp]
    d.ref_trace_closest.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp, vp]
    d.ref_trace_any.argtypes = [vp, vp, ctypes.c_size_t, vp]
    d.ref_render.argtypes = [vp, ctypes.c_double, vp, vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int,
                             ctypes.c_int, ctypes.c_double, ctypes.c_int, vp, vp]
    return d


def entity_arrays(ents, prefix="e"):
    """Flatten entity specs into npz-storable arrays."""
    out = {f"{prefix}_count": np.array(len(ents))}
    for i, e in enumerate(ents):
        out[f"{prefix}{i}_v"] = e.mesh.vertices
        out[f"{prefix}{i}_f"] = e.mesh.faces
        out[f"{prefix}{i}_color"] = np.array(e.color, dtype=np.float64)
        out[f"{prefix}{i}_smooth"] = np.array(int(e.smooth))
        out[f"{prefix}{i}_scale"] = np.array(float(e.scale))
        out[f"{prefix}{i}_pos"] = np.asarray(e.position, dtype=np.float64)
        out[f"{prefix}{i}_rot"] = np.asarray(e.rotation, dtype=np.float64)
    return out


def camera_arrays(cam, prefix="cam"):
    return {f"{prefix}_focal": np.array(cam["focal_length"], dtype=np.float64),
            f"{prefix}_res": np.array(cam["resolution"], dtype=np.float64),
            f"{prefix}_sensor": np.array(cam["sensor_size"], dtype=np.float64),
            f"{prefix}_zpos": np.array(int(cam["z_positive"])),
            f"{prefix}_pos": np.asarray(cam["position"], dtype=np.float64),
            f"{prefix}_rot": np.asarray(cam["rotation"], dtype=np.float64)}


def write_objs(ents, tmp):
    paths = []
    for i, e in enumerate(ents):
        p = os.path.join(tmp, f"{i}_{e.name}.obj")
        e.mesh.write_obj(p)
        paths.append(p)
    return paths


def ref_camera(R, cam):
    c = R.SimpleCamera(float(cam["focal_length"]), list(map(float, cam["resolution"])),
                       list(map(float, cam["sensor_size"])), bool(cam["z_positive"]))
    c.set_pose(np.asarray(cam["position"], dtype=np.float64), np.ascontiguousarray(cam["rotation"], dtype=np.float64))
    return c


def body_fixed_group(R, ents, paths):
    bfes = []
    for e, p in zip(ents, paths):
        b = R.BodyFixedEntity(p, "obj", bool(e.smooth), [float(x) for x in e.color])
        b.set_scale(float(e.scale))
        b.set_pose(np.asarray(e.position, dtype=np.float64), np.ascontiguousarray(e.rotation, dtype=np.float64))
        bfes.append(b)
    return R.BodyFixedGroup(bfes)


def dynamic_entities(R, ents, paths):
    out = []
    for e, p in zip(ents, paths):
        x = R.Entity(p, "obj", bool(e.smooth), [float(x) for x in e.color])
        x.set_scale(float(e.scale))
        x.set_pose(np.asarray(e.position, dtype=np.float64), np.ascontiguousarray(e.rotation, dtype=np.float64))
        out.append(x)
    return out


def driver_scene(D, ents, paths):
    n = len(ents)
    cpaths = (ctypes.c_char_p * n)(*[p.encode() for p in paths])
    smooth = np.array([int(e.smooth) for e in ents], dtype=np.int32)
    colors = np.array([e.color for e in ents], dtype=np.float64)
    scales = np.array([e.scale for e in ents], dtype=np.float64)
    pos = np.array([e.position for e in ents], dtype=np.float64)
    rot = np.array([np.asarray(e.rotation).ravel() for e in ents], dtype=np.float64)
    return D.ref_scene_create(n, cpaths, smooth.ctypes.data, colors.ctypes.data, scales.ctypes.data, pos.ctypes.data,
                              rot.ctypes.data)


def driver_closest(D, h, rays):
    n = rays.shape[0]
    prim = np.empty(n, np.int64)
    t, u, v = np.empty(n), np.empty(n), np.empty(n)
    D.ref_trace_closest(h, rays.ctypes.data, n, prim.ctypes.data, t.ctypes.data, u.ctypes.data, v.ctypes.data)
    return prim, t, u, v


def driver_any(D, h, rays):
    occ = np.empty(rays.shape[0], np.uint8)
    D.ref_trace_any(h, rays.ctypes.data, rays.shape[0], occ.ctypes.data)
    return occ


def light_array(lights):
    arr = np.zeros((len(lights), 16))
    for i, l in enumerate(lights):
        arr[i, 0] = 1.0 if l["type"] == "area" else 0.0
        arr[i, 1] = l["intensity"]
        arr[i, 2:5] = l["position"]
        arr[i, 5:14] = np.asarray(l.get("rotation", np.eye(3))).ravel()
        arr[i, 14:16] = l.get("size", [0.0, 0.0])
    return arr


def make_cornell(R, D, tmp):
    ents, cam, lights = scenes.cornell()
    paths = write_objs(ents, tmp)
    out = entity_arrays(ents)
    cam = dict(cam, resolution=[128, 128])
    out.update(camera_arrays(cam))
    g = body_fixed_group(R, ents, paths)
    c = ref_camera(R, cam)
    out["bf_xyz"] = g.intersection_pass(c)
    out["bf_ids"] = g.instance_pass(c)
    out["bf_normals"] = g.normal_pass(c)
    dyn = dynamic_entities(R, ents, paths)
    out["dyn_ids"] = R.instance_pass(c, dyn)
    out["dyn_normals"] = R.normal_pass(c, dyn)
    out["dyn_xyz"] = R.intersection_pass(c, dyn)
    # path tracer radiance (reference RNG under the determinism shim)
    rcam = dict(cam, resolution=[48, 48])
    out.update(camera_arrays(rcam, "rcam"))
    h = driver_scene(D, ents, paths)
    W = H = 48
    spp, bounces = 512, 3
    L = light_array(lights)
    rad = np.empty((H, W, 3), np.float32)
    m2 = np.empty((H, W, 3), np.float32)
    # keep every argument array alive for the duration of the call
    res_a = np.array(rcam["resolution"], dtype=np.float64)
    sen_a = np.array(rcam["sensor_size"], dtype=np.float64)
    pos_a = np.asarray(rcam["position"], dtype=np.float64)
    rot_a = np.ascontiguousarray(rcam["rotation"], dtype=np.float64)
    D.ref_render(h, float(rcam["focal_length"]), res_a.ctypes.data, sen_a.ctypes.data, int(rcam["z_positive"]),
                 pos_a.ctypes.data, rot_a.ctypes.data, len(lights), L.ctypes.data, spp, spp, 0.0, bounces,
                 rad.ctypes.data, m2.ctypes.data)
    out["render_mean"] = rad
    out["render_m2"] = m2
    out["render_spp"] = np.array(spp)
    out["render_bounces"] = np.array(bounces)
    out["lights"] = L
    # deterministic render: point light, 1 sample at the pixel corner, 1 bounce (no random draws)
    point = [dict(type="point", intensity=0.5, position=np.array([0.5, 0.8, 0.5]))]
    Lp = light_array(point)
    radp = np.empty((H, W, 3), np.float32)
    D.ref_render(h, float(rcam["focal_length"]), res_a.ctypes.data, sen_a.ctypes.data, int(rcam["z_positive"]),
                 pos_a.ctypes.data, rot_a.ctypes.data, 1, Lp.ctypes.data, 1, 1, 0.0, 1, radp.ctypes.data, None)
    out["point_lights"] = Lp
    out["point_radiance"] = radp
    return out


def make_asteroid(R, D, tmp):
    ast = scenes.asteroid(8000, seed=7)
    c, s = 0.8, 0.6
    rot = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]]) @ np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    ents = [scenes.EntitySpec("asteroid", ast, (0.1, 0.1, 0.1), smooth=True, scale=1.25,
                              position=np.array([10.0, -20.0, 5.0]), rotation=rot),
            scenes.EntitySpec("box", scenes.box_mesh((0.0, 0.0, 0.0), (300.0, 200.0, 100.0), 1.0, 0.0), (0.5, 0.5, 0.5),
                              position=np.array([1500.0, 200.0, 0.0]))]
    paths = write_objs(ents, tmp)
    out = entity_arrays(ents)
    cam = scenes.fov_camera(0.3, (64, 64), (6000.0, 1000.0, 2500.0), (200.0, 0.0, 0.0))
    out.update(camera_arrays(cam))
    g = body_fixed_group(R, ents, paths)
    rc = ref_camera(R, cam)
    out["bf_xyz"] = g.intersection_pass(rc)
    out["bf_ids"] = g.instance_pass(rc)
    out["bf_normals"] = g.normal_pass(rc)
    # seeded rays: origins on a 4 km shell aimed near the body, plus short/inside rays
    rng = np.random.Generator(np.random.PCG64(2024))
    n = 3072
    o = rng.normal(size=(n, 3))
    o = 4000.0 * o / np.linalg.norm(o, axis=1)[:, None]
    tgt = rng.uniform(-1400.0, 1400.0, size=(n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1)[:, None]
    rays = np.zeros((n, 8))
    rays[:, 0:3], rays[:, 3:6], rays[:, 6], rays[:, 7] = o, d, 0.0, np.finfo(np.float64).max
    # a quarter of the rays get a finite tmax (shadow-style queries)
    q = n // 4
    rays[:q, 7] = rng.uniform(1000.0, 5000.0, size=q)
    # FP32-representable origins, directions and bounds: an FP32 tracer sees the very same rays
    rays[:, :7] = rays[:, :7].astype(np.float32).astype(np.float64)
    rays[:q, 7] = rays[:q, 7].astype(np.float32).astype(np.float64)
    out["rays"] = rays
    h = driver_scene(D, ents, paths)
    out["ref_tris"] = np.empty(0)
    ntri = D.ref_num_tris(h)
    tri = np.empty((ntri, 21))
    D.ref_tris(h, tri.ctypes.data)
    out["ref_tris"] = tri
    out["closest_prim"], out["closest_t"], out["closest_u"], out["closest_v"] = driver_closest(D, h, rays)
    out["any_occluded"] = driver_any(D, h, rays)
    # batch lidar through the reference module (lidars/simple_lidar.hpp, do_lidar.hpp:80-155)
    npose = 512
    pp = rng.normal(size=(npose, 3))
    pp = 3000.0 * pp / np.linalg.norm(pp, axis=1)[:, None]
    rots = np.zeros((3, 3, 100000))
    rlist = []
    for k in range(npose):
        aim = rng.uniform(-900.0, 900.0, size=3)
        Rk = scenes.look_at(pp[k], aim, up=(0.0, 0.0, 1.0) if abs(pp[k][2]) < 2900 else (1.0, 0.0, 0.0))
        rots[:, :, k] = Rk
        rlist.append(Rk)
    lid = R.SimpleLidar(False)
    lid.batch_set_pose(np.ascontiguousarray(pp), rots, npose)
    out["lidar_pos"] = pp
    out["lidar_rot"] = np.array(rlist)
    out["lidar_range"] = g.batch_simulate_lidar(lid, 1.0)[0]
    return out


def edge_rays(ents):
    """Rays at the corners of the traversal and triangle-test rules (Cornell box, FP64):
    axis-aligned rays with +0.0 / -0.0 in their zero components; rays aimed exactly at triangle
    vertices and edge midpoints (non-unit directions); rays leaving a surface point along, into and
    out of its plane; direction components far below and far above 1; origins 1e6 away."""
    rays = []

    def add(o, d, tmin=0.0, tmax=np.finfo(np.float64).max):
        rays.append([o[0], o[1], o[2], d[0], d[1], d[2], tmin, tmax])

    for o in ((0.3, 0.7, 0.8), (0.05, 0.95, 0.9), (0.7, 0.45, 0.2)):
        for k in range(3):
            for sgn in (1.0, -1.0):
                for z0 in (0.0, -0.0):
                    for z1 in (0.0, -0.0):
                        d = [0.0, 0.0, 0.0]
                        d[k] = sgn
                        d[(k + 1) % 3], d[(k + 2) % 3] = z0, z1
                        add(o, d)
    targets = []
    for e in ents:
        v = np.asarray(e.mesh.vertices, dtype=np.float64)
        for f in np.asarray(e.mesh.faces):
            for i in range(3):
                a, b = v[f[i]], v[f[(i + 1) % 3]]
                targets.append(a)
                targets.append(0.5 * (a + b))
    targets = np.unique(np.round(np.array(targets), 12), axis=0)
    for o in (np.array([0.5, 0.5, 0.9]), np.array([0.5, 0.5, 2.4])):
        for t in targets:
            if np.abs(t - o).max() > 0:
                add(o, t - o)
    rng = np.random.Generator(np.random.PCG64(77))
    for _ in range(8):
        x, z = rng.uniform(0.02, 0.4, size=2)
        o = (x, 0.0, z)                          # on the floor (y = 0), away from the boxes
        for d in ((0.0, 1.0, 0.0), (0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (-0.6, 0.0, 0.8), (0.3, 1e-18, 0.4)):
            add(o, d)
        o = (x + 0.3, z + 0.3, 0.0)              # on the back wall (z = 0)
        for d in ((0.0, 0.0, 1.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), (0.7, -0.7, 0.0)):
            add(o, d)
    for o in ((0.5, 0.5, 0.5), (0.2, 0.3, 0.6)):
        for d in ((1e-20, 1.0, -1e-20), (1e-300, -1e-300, -1.0), (3e-17, 2e-16, 1.0), (1e-6, 2e-6, -3e-6),
                  (1e6, -2e6, 3e6), (1e-150, 1e-150, -1e-150), (-1e-170, 2e-170, 0.0)):
            add(o, d)
    for _ in range(24):
        dirv = rng.normal(size=3)
        o = 1e6 * dirv / np.linalg.norm(dirv)
        add(o, rng.uniform(0.1, 0.9, size=3) - o)
    return np.array(rays, dtype=np.float64)


def make_edges(R, D, tmp):
    ents, _, _ = scenes.cornell()
    paths = write_objs(ents, tmp)
    out = entity_arrays(ents)
    h = driver_scene(D, ents, paths)
    base = edge_rays(ents)
    # inclusive t bounds: for rays that hit, tmax = t and tmin = t (both still hit), tmax one ulp
    # below t, and tmin above tmax (never hits)
    prim, t, _, _ = driver_closest(D, h, base)
    hit = np.nonzero(prim >= 0)[0][::5]
    extra = []
    for i in hit:
        r = base[i].copy()
        r[7] = t[i]
        extra.append(r.copy())
        r[6], r[7] = t[i], np.finfo(np.float64).max
        extra.append(r.copy())
        r[6], r[7] = 0.0, np.nextafter(t[i], 0.0)
        extra.append(r.copy())
        r[6], r[7] = 0.5 * t[i] + 1e-9, 0.5 * t[i]
        extra.append(r.copy())
    rays = np.concatenate([base, np.array(extra)]) if extra else base
    out["rays"] = rays
    out["closest_prim"], out["closest_t"], out["closest_u"], out["closest_v"] = driver_closest(D, h, rays)
    out["any_occluded"] = driver_any(D, h, rays)
    # BodyFixedGroup passes through non-square cameras: z_positive boresight (+z of the camera frame,
    # turned into the box by diag(1, -1, -1)) with non-square pixels, and a tilted -z camera
    g = body_fixed_group(R, ents, paths)
    cams = {"zcam": dict(focal_length=0.02, resolution=[40.0, 24.0], sensor_size=[0.03, 0.02], z_positive=True,
                         position=np.array([0.5, 0.5, 2.4]), rotation=np.diag([1.0, -1.0, -1.0])),
            "wcam": dict(focal_length=0.03, resolution=[36.0, 20.0], sensor_size=[0.036, 0.024], z_positive=False,
                         position=np.array([0.9, 0.8, 2.0]),
                         rotation=scenes.look_at(np.array([0.9, 0.8, 2.0]), (0.5, 0.4, 0.3)))}
    for name, cam in cams.items():
        out.update(camera_arrays(cam, name))
        c = ref_camera(R, cam)
        out[name + "_xyz"] = g.intersection_pass(c)
        out[name + "_ids"] = g.instance_pass(c)
        out[name + "_normals"] = g.normal_pass(c)
    # batch LiDAR with the z_positive boresight (+z of the sensor frame, simple_lidar.hpp:42-64)
    rng = np.random.Generator(np.random.PCG64(78))
    npose = 64
    lp = np.where(np.arange(npose)[:, None] % 2 == 0, rng.uniform(0.1, 0.9, size=(npose, 3)),
                  rng.uniform(-2.0, 3.0, size=(npose, 3)))
    rots = np.zeros((3, 3, 100000))
    for k in range(npose):
        aim = rng.uniform(0.2, 0.8, size=3)
        # look_at points -z at the target; flip to put +z there
        rots[:, :, k] = np.diag([1.0, -1.0, -1.0]) @ scenes.look_at(lp[k], aim, up=(0.0, 0.3, 1.0))
    lid = R.SimpleLidar(True)
    lid.batch_set_pose(np.ascontiguousarray(lp), rots, npose)
    out["zlidar_pos"] = lp
    out["zlidar_rot"] = np.ascontiguousarray(np.moveaxis(rots[:, :, :npose], 2, 0))
    out["zlidar_range"] = g.batch_simulate_lidar(lid, 1.0)[0]
    # deterministic render of a smooth-shaded body (1 spp at integer pixel coordinates, 1 bounce,
    # point light: no random draws): pins the interpolated shading normal and the unclamped
    # Lambert term on a rotated, scaled and translated entity, through a non-square camera
    c, s_ = 0.6, 0.8
    rot = np.array([[1.0, 0.0, 0.0], [0.0, c, -s_], [0.0, s_, c]]) @ np.array([[c, 0.0, s_], [0.0, 1.0, 0.0],
                                                                               [-s_, 0.0, c]])
    sents = [scenes.EntitySpec("smooth", scenes.asteroid(3000, seed=9), (0.3, 0.25, 0.2), smooth=True, scale=0.9,
                               position=np.array([40.0, -30.0, 20.0]), rotation=rot),
             scenes.EntitySpec("flat", scenes.box_mesh((0.0, 0.0, 0.0), (400.0, 300.0, 200.0), 1.0, 0.0), (0.5, 0.5, 0.5),
                               position=np.array([1300.0, 0.0, 0.0]))]
    spaths = write_objs(sents, tmp)
    out.update(entity_arrays(sents, "s"))
    scam = scenes.fov_camera(0.25, (48, 30), (4000.0, 2500.0, 2000.0), (300.0, 0.0, 0.0))
    out.update(camera_arrays(scam, "scam"))
    sl = [dict(type="point", intensity=4.0e7, position=np.array([3000.0, 5000.0, 4000.0]))]
    Ls = light_array(sl)
    hs = driver_scene(D, sents, spaths)
    W, H = int(scam["resolution"][0]), int(scam["resolution"][1])
    rad = np.empty((H, W, 3), np.float32)
    res_a = np.array(scam["resolution"], dtype=np.float64)
    sen_a = np.array(scam["sensor_size"], dtype=np.float64)
    pos_a = np.asarray(scam["position"], dtype=np.float64)
    rot_a = np.ascontiguousarray(scam["rotation"], dtype=np.float64)
    D.ref_render(hs, float(scam["focal_length"]), res_a.ctypes.data, sen_a.ctypes.data, int(scam["z_positive"]),
                 pos_a.ctypes.data, rot_a.ctypes.data, 1, Ls.ctypes.data, 1, 1, 0.0, 1, rad.ctypes.data, None)
    out["s_lights"] = Ls
    out["s_radiance"] = rad
    return out


def main():
    """Writes every fixture, or only those named on the command line (cornell, asteroid, edges)."""
    which = sys.argv[1:] or ["cornell", "asteroid", "edges"]
    makers = {"cornell": make_cornell, "asteroid": make_asteroid, "edges": make_edges}
    R = load_ref_module()
    D = load_driver()
    with tempfile.TemporaryDirectory() as tmp:
        for name in which:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **makers[name](R, D, tmp))
    for name in which:
        print(name + ".npz", os.path.getsize(os.path.join(HERE, name + ".npz")))


if __name__ == "__main__":
    main()
