"""Size-independent properties at the benchmark's full sizes: the 2M-triangle asteroid, a 2048^2
camera and a 1024^2 LiDAR grid (the oracle is too slow to traverse these in a test, so the checks
are consistency relations the reference's semantics imply):

* any-hit reports an occluder exactly when closest-hit reports a hit (same triangle test, inclusive
  t range);
* the intersection / instance passes agree with closest-hit traversal of the same camera rays;
* every call is deterministic (bitwise identical on repetition);
* LiDAR grid ranges equal |hit point - sensor| of closest-hit traversal of the same beams;
* a full-size render and scan give bitwise the same result alone and inside a batch;
* requests beyond the documented limits are refused with CRT_ERR_INVALID.
"""
import numpy as np
import pytest

import oracle
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
    r64 = oracle.camera_rays(cam)                   # o.xyz, d.xyz, tmin, tmax (FP64)
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


def test_passes_agree_with_closest_hit(big):
    ctx, sc, cfg = big
    cam = cfg["camera"]
    xyz, ids, nrm = sc.passes(cam)
    rays = crt_rays(cam)
    hits = sc.trace_closest(rays)
    W, H = cam["resolution"]
    hit = (hits["prim"] != lib.CRT_MISS).reshape(H, W)
    np.testing.assert_array_equal(ids != 0, hit)
    o = rays[:, 0:3].astype(np.float64)
    d = rays[:, 4:7].astype(np.float64)
    p = (o + hits["t"][:, None].astype(np.float64) * d).reshape(H, W, 3)
    err = np.linalg.norm(p - xyz, axis=2)[hit]
    scale = np.linalg.norm(o[0]) + 2000.0
    assert np.quantile(err, 0.999) < 1e-5 * scale
    assert np.allclose(np.linalg.norm(nrm[hit], axis=1), 1.0, atol=1e-6)


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


def test_lidar_grid_ranges_match_closest_hit(big):
    ctx, sc, cfg = big
    lid = cfg["lidar"]
    nx, ny = lid["nx"], lid["ny"]
    rng, prim = sc.lidar_grid(lid["position"], lid["rotation"], nx, ny, lid["half_x"], lid["half_y"])
    # the beam directions of crt_lidar_grid (header: tan of uniformly spaced angles, world = R^T)
    tx = np.tan(-lid["half_x"] + (np.arange(nx) + 0.5) * 2 * lid["half_x"] / nx)
    ty = np.tan(-lid["half_y"] + (np.arange(ny) + 0.5) * 2 * lid["half_y"] / ny)
    sel = np.random.Generator(np.random.PCG64(3)).choice(nx * ny, 4096, replace=False)
    jx, jy = sel % nx, sel // nx
    dc = np.stack([tx[jx], ty[jy], -np.ones(len(sel))], axis=1)
    dc /= np.linalg.norm(dc, axis=1, keepdims=True)
    dw = dc @ np.asarray(lid["rotation"], dtype=np.float64)
    o = np.broadcast_to(np.asarray(lid["position"], dtype=np.float64), dw.shape)
    hits = sc.trace_closest(lib.make_rays(o.astype(np.float32), dw.astype(np.float32)))
    same = hits["prim"] == prim.reshape(-1)[sel]
    assert same.mean() > 0.999
    t = hits["t"][same].astype(np.float64)
    ok = np.abs(t - rng.reshape(-1)[sel][same]) <= 1e-5 * (np.linalg.norm(o[0]) + 2000.0)
    assert ok.mean() > 0.999


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
