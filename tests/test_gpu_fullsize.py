"""Size-independent properties at the benchmark's full sizes: the 2M-triangle asteroid, a 2048^2
camera and a 1024^2 LiDAR grid.  The comparison with the oracle at these sizes is in
test_gpu_config_parity.py; these are consistency relations that hold bit for bit:

* any-hit reports an occluder exactly when closest-hit reports a hit (same triangle test, inclusive
  t range);
* every call is deterministic (bitwise identical on repetition);
* a full-size render and scan give bitwise the same result alone and inside a batch;
* requests beyond the documented limits are refused with CRT_ERR_INVALID.
"""
import numpy as np
import pytest

from crt_gb300 import lib, scenes, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    ctx = lib.Context(0)
    sc = ctx.scene(workloads.asteroid_entities(2_000_000))
    cfg = workloads.asteroid_config(2048, 1024)
    yield ctx, sc, cfg
    ctx.close()


def crt_rays(cam):
    r64 = workloads.camera_rays(cam)                # o.xyz, d.xyz, tmin, tmax (FP64)
    r = np.empty((r64.shape[0], 8), dtype=np.float32)
    r[:, 0:3] = r64[:, 0:3]
    r[:, 3] = 0.0
    r[:, 4:7] = r64[:, 3:6]
    r[:, 7] = np.finfo(np.float32).max
    return r


def test_any_hit_agrees_with_closest_hit(big):
    ctx, sc, cfg = big
    rays = crt_rays(cfg["camera"])
    # add rays that miss: the same rays pointed away from the body
    away = rays.copy()
    away[:, 4:7] *= -1.0
    allr = np.concatenate([rays, away])
    hits = sc.trace_closest(allr)
    occ = sc.trace_any(allr)
    hit = hits["prim"] != lib.CRT_MISS
    np.testing.assert_array_equal(occ.astype(bool), hit)
    assert hit[:len(rays)].mean() > 0.99 and not hit[len(rays):].any()


def test_calls_are_deterministic(big):
    ctx, sc, cfg = big
    cam, lid = cfg["camera"], cfg["lidar"]
    a = sc.render(cam, cfg["lights"], 1, 1, 1.0, 1, want_radiance=True)
    b = sc.render(cam, cfg["lights"], 1, 1, 1.0, 1, want_radiance=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    r1 = sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"])
    r2 = sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"])
    np.testing.assert_array_equal(r1[0], r2[0])
    np.testing.assert_array_equal(r1[1], r2[1])


def test_full_size_batch_equals_standalone(big):
    ctx, sc, cfg = big
    cam, lid, lights = cfg["camera"], cfg["lidar"], cfg["lights"]
    reqs = [dict(kind="render", scene=sc, camera=cam, lights=lights, min_samples=2, max_samples=2,
                 noise_threshold=0.0, num_bounces=2, seed=9, request=4, radiance=True),
            dict(kind="lidar", scene=sc, position=lid["position"], rotation=lid["rotation"], nx=lid["nx"],
                 ny=lid["ny"], half_x=lid["half_x"], half_y=lid["half_y"])]
    outs, st = ctx.batch(reqs)
    alone_r = sc.render(cam, lights, 2, 2, 0.0, 2, seed=9, request=4)
    alone_l = sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"])
    np.testing.assert_array_equal(outs[0][0], alone_r[0])
    np.testing.assert_array_equal(outs[0][1], alone_r[1])
    np.testing.assert_array_equal(outs[1][0], alone_l[0])
    np.testing.assert_array_equal(outs[1][1], alone_l[1])


def test_limits_are_refused(big):
    ctx, sc, cfg = big
    q = scenes.random_quaternions(1, seed=1)
    with pytest.raises(lib.CrtError) as e:
        sc.srp([1.0, 0.0, 0.0], q, 32769)
    assert e.value.status == -1
    lights = cfg["lights"] * 17
    with pytest.raises(lib.CrtError) as e:
        sc.render(cfg["camera"], lights, 1, 1, 1.0, 1)
    assert e.value.status == -1
    lid = cfg["lidar"]
    with pytest.raises(lib.CrtError) as e:
        sc.lidar_grid(lid["position"], lid["rotation"], 16, 16, 1.6, 0.1)
    assert e.value.status == -1
