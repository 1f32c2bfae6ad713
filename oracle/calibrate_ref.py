"""Calibrate the CPU baseline (TEST / MEASUREMENT INFRASTRUCTURE ONLY): the reference's own release
build against the FP64 restatement in crt_oracle.c on the benchmark's workload, same host, same
threads.

The reference binary is oracle/_ref/perf/_crt<ext>, compiled by oracle/build_ref.py from the
reference sources with the reference's CMake release flags (CMakeLists.txt:15-16); it exists only
where those sources are at hand, so this runs in the development container, not on the GPU host.
bench.py times the restatement (its `cpu_baseline`, kind "port") because the reference sources do
not travel; this script gives the factor between the two.

Workload (the bench's step): the 2M-triangle procedural asteroid, a 2048^2 render at 1 spp with the
sun as a point light (primary + shadow rays, do_render.hpp:28-141) and LiDAR beams of the 1024^2
grid (do_batch_lidar, one pose per beam, calls of 100,000 poses, do_lidar.hpp:80-155).  Both sides
build their BVH once, untimed; OMP_NUM_THREADS = all host cores.

    python oracle/calibrate_ref.py [n_beams]
"""
import importlib.util
import json
import os
import sys
import sysconfig
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (os.path.join(REPO, "ceres-raytracer_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def load_ref_module():
    path = os.path.join(HERE, "_ref", "perf", "_crt" + sysconfig.get_config_var("EXT_SUFFIX"))
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} missing: run oracle/build_ref.py <reference dir> first")
    spec = importlib.util.spec_from_file_location("_crt", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main(n_beams=300_000):
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    from crt_gb300 import scenes, workloads
    R = load_ref_module()
    ents = workloads.asteroid_entities(2_000_000)
    cfg = workloads.asteroid_config(2048, 1024)
    cam, light = cfg["camera"], cfg["lights"][0]
    out = {"host_cores": threads}
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "asteroid.obj")
        scenes.write_obj_fast(ents[0].mesh, path)
        t = time.perf_counter()
        bfe = R.BodyFixedEntity(path, "obj", False, [0.1, 0.1, 0.1])
        g = R.BodyFixedGroup([bfe])
        out["reference_build_s"] = round(time.perf_counter() - t, 3)
    c = R.SimpleCamera(float(cam["focal_length"]), [float(x) for x in cam["resolution"]],
                       [float(x) for x in cam["sensor_size"]], False)
    c.set_pose(np.asarray(cam["position"], dtype=np.float64), np.ascontiguousarray(cam["rotation"]))
    pl = R.PointLight(float(light["intensity"]))
    pl.set_position(np.asarray(light["position"], dtype=np.float64))
    t = time.perf_counter()
    g.render(c, [pl], 1, 1, 1.0, 1)
    ref_render_s = time.perf_counter() - t
    # the same rays on the restatement: primary + one shadow ray per hit
    o = oracle.Scene(ents, nthreads=threads)
    _, ids, _, _ = o.passes(cam)
    rays_render = cam["resolution"][0] * cam["resolution"][1] + int((ids > 0).sum())
    t = time.perf_counter()
    o.render(cam, cfg["lights"], 1, 1, 1.0, 1)
    port_render_s = time.perf_counter() - t
    # LiDAR beams of the grid as per-beam poses (the reference casts one boresight ray per pose)
    beams = workloads.lidar_grid_rays(cfg["lidar"])
    sel = np.random.Generator(np.random.PCG64(5)).choice(len(beams), n_beams, replace=False)
    beams = beams[np.sort(sel)]
    pos = beams[:, 0:3]
    ref_lidar_s = 0.0
    for a in range(0, n_beams, 100_000):
        b = min(n_beams, a + 100_000)
        rots = np.zeros((3, 3, 100_000))
        for k in range(a, b):
            rots[:, :, k - a] = scenes.look_at(pos[k], pos[k] + beams[k, 3:6])
        lid = R.SimpleLidar(False)
        lid.batch_set_pose(np.ascontiguousarray(pos[a:b]), rots, b - a)
        t = time.perf_counter()
        g.batch_simulate_lidar(lid, 1.0)
        ref_lidar_s += time.perf_counter() - t
    t = time.perf_counter()
    o.trace_closest(beams)
    port_lidar_s = time.perf_counter() - t
    ref_rate = (rays_render + n_beams) / (ref_render_s + ref_lidar_s) / 1e6
    port_rate = (rays_render + n_beams) / (port_render_s + port_lidar_s) / 1e6
    out.update(rays_render=int(rays_render), beams=n_beams, reference_render_s=round(ref_render_s, 3),
               reference_lidar_s=round(ref_lidar_s, 3), port_render_s=round(port_render_s, 3),
               port_lidar_s=round(port_lidar_s, 3), reference_mrays_s=round(ref_rate, 2),
               port_mrays_s=round(port_rate, 2), port_over_reference=round(port_rate / ref_rate, 2))
    print(json.dumps(out))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 300_000)
