"""Seeded synthetic workloads with the shapes of the benchmark configurations.

asteroid_config()   procedural asteroid (icosphere level 9 decimated to 2M triangles, radius 1 km,
                    6-octave value noise, 5 % amplitude, albedo 0.1); camera 2048^2, 10 deg FOV at
                    5 km; sun as a point light 1e9 m away along a random direction with
                    intensity / d^2 = 1; 1 spp, 1 bounce (primary + shadow ray); LiDAR 1024^2 beams
                    over +-5 deg from the camera pose.
batched_config()    64 requests on the same asteroid: 32 renders (resolution in {128..2048}^2, spp in
                    {1, 4, 16, 64}, 2 bounces, poses on a 3-10 km shell) and 32 LiDAR scans of
                    64^2 .. 1024^2 beams; seed 1.
srp_config()        spacecraft (~50k triangles), 256 random attitudes, 4096^2 rays, 2 bounces.
"""
import numpy as np

from . import scenes

SUN_DISTANCE = 1.0e9


def asteroid_entities(target_faces=2_000_000, seed=0, smooth=False):
    mesh = scenes.cached_asteroid(target_faces, seed=seed)
    return [scenes.EntitySpec("asteroid", mesh, (0.1, 0.1, 0.1), smooth=smooth)]


def pose_on_shell(rng, rmin, rmax):
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    return d * rng.uniform(rmin, rmax)


def asteroid_config(res=2048, lidar_n=1024, seed=0):
    cam_pos = 5000.0 * scenes.unit_vector(1000 + seed)
    camera = scenes.fov_camera(scenes.TAN5, (res, res), cam_pos, (0.0, 0.0, 0.0))
    sun = scenes.unit_vector(2000 + seed)
    lights = [dict(type="point", intensity=SUN_DISTANCE ** 2, position=SUN_DISTANCE * sun)]
    lidar = dict(position=cam_pos, rotation=camera["rotation"], nx=lidar_n, ny=lidar_n,
                 half_x=np.deg2rad(5.0), half_y=np.deg2rad(5.0))
    return dict(camera=camera, lights=lights, lidar=lidar, spp=1, bounces=1)


def lidar_grid_rays(lid):
    """FP64 beam rays [nx * ny, 8] (origin, direction, tmin 0, tmax max) of a LiDAR beam grid in the
    order crt_lidar_grid reports them (row-major [ny][nx]): beam (i, j) along
    R^T normalize(tan_x[i], tan_y[j], -1) (+1 with z_positive), tan of angles uniform over each half
    angle."""
    nx, ny = int(lid["nx"]), int(lid["ny"])
    tx = np.tan(-lid["half_x"] + (np.arange(nx) + 0.5) * 2 * lid["half_x"] / nx)
    ty = np.tan(-lid["half_y"] + (np.arange(ny) + 0.5) * 2 * lid["half_y"] / ny)
    zs = 1.0 if lid.get("z_positive", False) else -1.0
    s = np.stack(np.broadcast_arrays(tx[None, :], ty[:, None], zs * np.ones((ny, nx))), -1).reshape(-1, 3)
    s /= np.linalg.norm(s, axis=1)[:, None]
    rays = np.zeros((nx * ny, 8))
    rays[:, 0:3] = np.asarray(lid["position"], dtype=np.float64)
    rays[:, 3:6] = s @ np.asarray(lid["rotation"], dtype=np.float64)
    rays[:, 7] = np.finfo(np.float64).max
    return rays


def camera_rays(cam):
    """FP64 camera rays [W * H, 8] at integer pixel coordinates, row-major, as SimpleCamera::pixel_to_ray
    (cameras/simple_camera.hpp:61-81): direction R^T normalize((u - W/2) / sx, (H/2 - v) / sy, -+f)
    with sx = W / sensor_w, sy = H / sensor_h; origin the camera position."""
    W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
    sx = cam["resolution"][0] / cam["sensor_size"][0]
    sy = cam["resolution"][1] / cam["sensor_size"][1]
    f = cam["focal_length"] if cam.get("z_positive", False) else -cam["focal_length"]
    u = np.arange(W, dtype=np.float64)
    v = np.arange(H, dtype=np.float64)
    d = np.empty((H, W, 3))
    d[..., 0] = ((u - cam["resolution"][0] / 2.0) / sx)[None, :]
    d[..., 1] = ((cam["resolution"][1] / 2.0 - v) / sy)[:, None]
    d[..., 2] = f
    d = d.reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1)[:, None]
    rays = np.zeros((W * H, 8))
    rays[:, 0:3] = np.asarray(cam["position"], dtype=np.float64)
    rays[:, 3:6] = d @ np.asarray(cam["rotation"], dtype=np.float64).reshape(3, 3)
    rays[:, 7] = np.finfo(np.float64).max
    return rays


def batched_config(seed=1, n_render=32, n_lidar=32):
    rng = np.random.Generator(np.random.PCG64(seed))
    sun = scenes.unit_vector(3000 + seed)
    lights = [dict(type="point", intensity=SUN_DISTANCE ** 2, position=SUN_DISTANCE * sun)]
    reqs = []
    for i in range(n_render):
        res = int(rng.choice([128, 256, 512, 1024, 2048]))
        spp = int(rng.choice([1, 4, 16, 64]))
        pos = pose_on_shell(rng, 3000.0, 10000.0)
        # FOV wide enough to frame the body from the pose's range
        tan_half = 1100.0 / np.linalg.norm(pos)
        cam = scenes.fov_camera(tan_half, (res, res), pos, (0.0, 0.0, 0.0))
        reqs.append(dict(kind="render", camera=cam, lights=lights, spp=spp, bounces=2, request=i))
    for i in range(n_lidar):
        n = int(rng.choice([64, 128, 256, 512, 1024]))
        pos = pose_on_shell(rng, 3000.0, 10000.0)
        R = scenes.look_at(pos, (0.0, 0.0, 0.0))
        reqs.append(dict(kind="lidar", position=pos, rotation=R, nx=n, ny=n, half_x=np.deg2rad(5.0),
                         half_y=np.deg2rad(5.0), request=n_render + i))
    order = rng.permutation(len(reqs))
    return [reqs[k] for k in order]


def request_rays(req):
    """Primary rays of a request (renders: pixels x samples; LiDAR: beams)."""
    if req["kind"] == "render":
        w, h = req["camera"]["resolution"]
        return int(w) * int(h) * int(req["spp"])
    return int(req["nx"]) * int(req["ny"])


def srp_config(n_att=256, grid=4096, seed=0):
    ents = scenes.spacecraft()
    q = scenes.random_quaternions(n_att, seed=seed)
    return dict(entities=ents, quaternions=q, grid=grid, num_bounces=2, sun=np.array([1.0, 0.0, 0.0]))


SERVED_BODIES = ((100_000, 2), (500_000, 3), (2_000_000, 4), (8_000_000, 5))


def served_bodies(bodies=SERVED_BODIES):
    """Entity lists of the four resident asteroids of the served stream (faces, seed)."""
    return [asteroid_entities(f, seed=s) for f, s in bodies]


def served_stream(rate=200.0, seconds=60.0, seed=7, n_bodies=4):
    """Poisson request stream over the resident bodies: arrival times (s) and request dicts.

    50 % renders (resolution in {128..2048}^2, spp in {1, 2, 4, 8, 16}, primary + sun-shadow ray as
    the asteroid render, poses on a 3-10 km shell), 30 % LiDAR scans ({64..1024}^2 beams over
    +-5 deg) and 20 % SRP queries (one attitude, {512, 1024, 2048}^2 sun-ray grid, 2 bounces).
    Each request names its body by index (`body`)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(rng.poisson(rate * seconds))
    times = np.sort(rng.uniform(0.0, seconds, n))
    sun = scenes.unit_vector(4000 + seed)
    lights = [dict(type="point", intensity=SUN_DISTANCE ** 2, position=SUN_DISTANCE * sun)]
    out = []
    for i, t in enumerate(times):
        body = int(rng.integers(n_bodies))
        u = rng.uniform()
        if u < 0.5:
            res = int(rng.choice([128, 256, 512, 1024, 2048]))
            spp = int(rng.choice([1, 2, 4, 8, 16]))
            pos = pose_on_shell(rng, 3000.0, 10000.0)
            cam = scenes.fov_camera(1100.0 / np.linalg.norm(pos), (res, res), pos, (0.0, 0.0, 0.0))
            q = dict(kind="render", camera=cam, lights=lights, min_samples=spp, max_samples=spp,
                     noise_threshold=0.0, num_bounces=1, seed=seed, request=i, size=res)
        elif u < 0.8:
            m = int(rng.choice([64, 128, 256, 512, 1024]))
            pos = pose_on_shell(rng, 3000.0, 10000.0)
            q = dict(kind="lidar", position=pos, rotation=scenes.look_at(pos, (0.0, 0.0, 0.0)), nx=m, ny=m,
                     half_x=np.deg2rad(5.0), half_y=np.deg2rad(5.0), size=m)
        else:
            g = int(rng.choice([512, 1024, 2048]))
            q = dict(kind="srp", sun_dir=sun, quaternions=scenes.random_quaternions(1, seed=10_000 + i), grid=g,
                     num_bounces=2, size=g)
        q["body"] = body
        out.append((float(t), q))
    return out
