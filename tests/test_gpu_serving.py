"""Serving loop (crt_server_*): continuous batching over resident scenes.

* every result equals the same request run alone (bit for bit), whatever waves it shared;
* requests join running lanes: with small waves and a long render resident, later requests share
  its waves and finish before it;
* admission by memory budget: with a budget smaller than any request each request runs alone;
* malformed requests are refused at submission and the server keeps serving;
* waits are bounded (CRT_ERR_TIMEOUT), no GPU-side waiting is involved; a ticket never issued or
  already collected is refused (CRT_ERR_INVALID).
"""
import threading
import time

import numpy as np
import pytest

from crt_gb300 import lib, scenes
from helpers import camera_from, entities_from, lights_from, load_golden

pytestmark = pytest.mark.gpu


def request_mix(d, cornell, ast, n=14, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    cam = camera_from(d, "rcam")
    reqs = []
    for k in range(n):
        kind = ["render", "lidar", "srp"][k % 3]
        if kind == "render":
            res = int(rng.choice([8, 16, 32]))
            reqs.append(dict(kind="render", scene=cornell, camera=dict(cam, resolution=[res, res]),
                             lights=lights_from(d["lights"]), min_samples=2, max_samples=2, noise_threshold=0.0,
                             num_bounces=2, seed=k, request=k, radiance=True))
        elif kind == "lidar":
            pos = 3000.0 * scenes.unit_vector(70 + k)
            reqs.append(dict(kind="lidar", scene=ast, position=pos, rotation=scenes.look_at(pos, (0, 0, 0)),
                             nx=int(rng.integers(8, 40)), ny=int(rng.integers(8, 40)), half_x=0.1, half_y=0.08))
        else:
            reqs.append(dict(kind="srp", scene=ast, sun_dir=scenes.unit_vector(90 + k),
                             quaternions=scenes.random_quaternions(2, seed=k), grid=96, num_bounces=1))
    return reqs


def alone(q):
    sc = q["scene"]
    if q["kind"] == "render":
        return sc.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], q["noise_threshold"],
                         q["num_bounces"], seed=q["seed"], request=q["request"])
    if q["kind"] == "lidar":
        return sc.lidar_grid(q["position"], q["rotation"], q["nx"], q["ny"], q["half_x"], q["half_y"])
    f, t, _ = sc.srp(q["sun_dir"], q["quaternions"], q["grid"], num_bounces=q["num_bounces"])
    return f, t


# count_rays: lanes run the counting build and launch each wave's kernels one by one; without it each
# wave is replayed from a CUDA graph captured per wave shape (the production path)
@pytest.fixture(scope="module", params=[True, False], ids=["counting", "graphs"])
def server(request):
    srv = lib.Server(0, lanes=2, lane_budget_bytes=1 << 30, max_batch=8, count_rays=request.param, wave_paths=1 << 16)
    d = load_golden("cornell")
    cornell = srv.scene(entities_from(d))
    ast = srv.scene([scenes.EntitySpec("a", scenes.asteroid(20_000, seed=6), (0.2, 0.2, 0.2), rho_s=0.2,
                                       rho_d=0.3)])
    yield srv, d, cornell, ast
    srv.close()


def test_results_same_alone_and_in_the_mix(server):
    srv, d, cornell, ast = server
    reqs = request_mix(d, cornell, ast)
    expected = [alone(q) for q in reqs]
    tickets = [None] * len(reqs)

    def client(idx):
        for i in idx:
            tickets[i] = srv.submit(reqs[i])
            time.sleep(0.001 * (i % 3))

    threads = [threading.Thread(target=client, args=(range(k, len(reqs), 2),)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    sizes = []
    for q, e, tk in zip(reqs, expected, tickets):
        res, out = srv.wait(tk, timeout=60.0)
        assert res["status"] == 0
        assert res["end_s"] >= res["start_s"] >= res["submit_s"]
        sizes.append(res["batch_size"])
        for a, b in zip(out, e):
            if b is not None:
                np.testing.assert_array_equal(a, b)
    st = srv.stats()
    assert st["completed"] >= len(reqs) and st["failed"] == 0
    assert st["rays"] > 0 or not srv.config["count_rays"]


@pytest.mark.parametrize("count_rays", [True, False], ids=["counting", "graphs"])
def test_adaptive_and_long_renders_share_waves(count_rays):
    srv = lib.Server(0, lanes=1, lane_budget_bytes=1 << 30, max_batch=64, count_rays=count_rays, wave_paths=1 << 16)
    try:
        d = load_golden("cornell")
        cornell = srv.scene(entities_from(d))
        cam = camera_from(d, "rcam")
        area = lights_from(d["lights"])
        # 256 x 240 x 32 spp: one sample (61,440 paths) per wave of 65,536 paths, so 32 waves
        long_q = dict(kind="render", scene=cornell, camera=dict(cam, resolution=[256, 240]), lights=area,
                      min_samples=32, max_samples=32, noise_threshold=0.0, num_bounces=2, seed=5, request=1,
                      radiance=True)
        short = [dict(kind="render", scene=cornell, camera=dict(cam, resolution=[20, 16]), lights=area, min_samples=4,
                      max_samples=4, noise_threshold=0.0, num_bounces=2, seed=6, request=20 + r, radiance=True)
                 for r in range(2)]
        short.append(dict(kind="lidar", scene=cornell, position=[0.5, 0.5, 2.4], rotation=np.eye(3), nx=9, ny=7,
                          half_x=0.1, half_y=0.1))
        adaptive = [dict(kind="render", scene=cornell, camera=dict(cam, resolution=[20, 16]), lights=area,
                         min_samples=2, max_samples=24, noise_threshold=1.5, num_bounces=2, seed=7, request=10 + r,
                         radiance=True) for r in range(3)]
        reqs = [long_q] + short + adaptive
        expected = [alone(q) for q in reqs]
        tickets = [srv.submit(q) for q in reqs]
        results = [srv.wait(t, timeout=120.0) for t in tickets]
        for (res, out), e in zip(results, expected):
            assert res["status"] == 0
            for a, b in zip(out, e):
                if b is not None:
                    np.testing.assert_array_equal(a, b)
        # the short requests joined the long render's waves and left before it
        end_long = results[0][0]["end_s"]
        assert all(res["end_s"] < end_long for res, _ in results[1:1 + len(short)])
        assert all(res["batch_size"] > 1 for res, _ in results[1:1 + len(short)])
    finally:
        srv.close()


@pytest.mark.parametrize("count_rays", [True, False], ids=["counting", "graphs"])
def test_srp_query_spans_waves_shared_with_renders(count_rays):
    """An SRP query larger than one wave (2 attitudes of 600^2 sun rays, 65,536 items per wave) rides in
    the waves' primary traces one range per wave, while a render and a LiDAR scan share those waves;
    force and torque equal crt_srp's bit for bit, the render and the scan their standalone calls (waves
    launched one by one, or replayed from graphs whose SRP stages read the range on the device)."""
    srv = lib.Server(0, lanes=1, lane_budget_bytes=1 << 30, max_batch=64, count_rays=count_rays, wave_paths=1 << 16)
    try:
        d = load_golden("cornell")
        cornell = srv.scene(entities_from(d))
        craft = srv.scene(scenes.spacecraft(bus_cell=0.25, panel_cell=0.2, dish_rings=16, dish_segments=16))
        cam = camera_from(d, "rcam")
        reqs = [dict(kind="srp", scene=craft, sun_dir=[0.2, 1.0, 0.1], quaternions=scenes.random_quaternions(2, seed=8),
                     grid=600, num_bounces=2),
                dict(kind="render", scene=cornell, camera=dict(cam, resolution=[64, 48]), lights=lights_from(d["lights"]),
                     min_samples=8, max_samples=8, noise_threshold=0.0, num_bounces=2, seed=3, request=2, radiance=True),
                dict(kind="lidar", scene=cornell, position=[0.5, 0.5, 2.4], rotation=np.eye(3), nx=9, ny=7, half_x=0.1,
                     half_y=0.1),
                dict(kind="srp", scene=craft, sun_dir=[1.0, 0.0, 0.0], quaternions=scenes.random_quaternions(3, seed=9),
                     grid=128, num_bounces=1)]
        expected = [alone(q) for q in reqs]
        tickets = [srv.submit(q) for q in reqs]
        results = [srv.wait(t, timeout=120.0) for t in tickets]
        for (res, out), e in zip(results, expected):
            assert res["status"] == 0
            for a, b in zip(out, e):
                if b is not None:
                    np.testing.assert_array_equal(a, b)
        assert results[1][0]["batch_size"] > 1 and results[2][0]["batch_size"] > 1
        assert srv.stats()["batches"] >= 12   # 6 ranges per 600^2 attitude
    finally:
        srv.close()


def test_admission_budget_runs_large_requests_alone():
    srv = lib.Server(0, lanes=1, lane_budget_bytes=1, max_batch=64)
    try:
        d = load_golden("cornell")
        cornell = srv.scene(entities_from(d))
        cam = camera_from(d, "rcam")
        reqs = [dict(kind="render", scene=cornell, camera=dict(cam, resolution=[16, 16]),
                     lights=lights_from(d["lights"]), min_samples=1, max_samples=1, noise_threshold=0.0,
                     num_bounces=1, seed=1, request=k) for k in range(5)]
        tickets = [srv.submit(q) for q in reqs]
        for q, tk in zip(reqs, tickets):
            res, out = srv.wait(tk, timeout=60.0)
            assert res["status"] == 0 and res["batch_size"] == 1
            np.testing.assert_array_equal(out[0], alone(q)[0])
        assert srv.stats()["batches"] == 5
    finally:
        srv.close()


def test_malformed_request_refused_and_service_continues(server):
    srv, d, cornell, ast = server
    bad = dict(kind="lidar", scene=ast, position=[0, 0, 3000.0], rotation=np.eye(3), nx=0, ny=4, half_x=0.1,
               half_y=0.1)
    with pytest.raises(lib.CrtError):
        srv.submit(bad)
    good = dict(bad, nx=4)
    res, out = srv.wait(srv.submit(good), timeout=60.0)
    assert res["status"] == 0
    np.testing.assert_array_equal(out[0], alone(good)[0])


def test_bad_srp_attitude_fails_alone(server):
    """An SRP query with a zero quaternion fails at admission (status != 0); the lane keeps serving."""
    srv, d, cornell, ast = server
    bad = dict(kind="srp", scene=ast, sun_dir=[1.0, 0.0, 0.0], quaternions=np.zeros((1, 4)), grid=64, num_bounces=1)
    res, _ = srv.wait(srv.submit(bad), timeout=60.0)
    assert res["status"] != 0
    good = dict(bad, quaternions=scenes.random_quaternions(1, seed=1))
    res, out = srv.wait(srv.submit(good), timeout=60.0)
    assert res["status"] == 0
    np.testing.assert_array_equal(out[0], alone(good)[0])


def test_wait_is_bounded(server):
    srv, d, cornell, _ = server
    # a ticket never issued is refused at once, even by an unbounded wait
    t = time.perf_counter()
    with pytest.raises(lib.CrtError) as e:
        srv.wait(10 ** 9, timeout=-1.0)
    assert e.value.status == -1 and time.perf_counter() - t < 5.0
    # a wait shorter than the request ends with CRT_ERR_TIMEOUT (1024^2 x 16 spp x 3 bounces: 16.8 M
    # paths, milliseconds of GPU work after admission); the result is then collected exactly once
    cam = camera_from(d, "rcam")
    q = dict(kind="render", scene=cornell, camera=dict(cam, resolution=[1024, 1024]), lights=lights_from(d["lights"]),
             min_samples=16, max_samples=16, noise_threshold=0.0, num_bounces=3, seed=5, request=5, radiance=True)
    tk = srv.submit(q)
    with pytest.raises(lib.CrtError) as e:
        srv.wait(tk, timeout=0.0)
    assert e.value.status == -4
    res, out = srv.wait(tk, timeout=120.0)
    assert res["status"] == 0 and np.isfinite(out[1]).all()
    with pytest.raises(lib.CrtError) as e:
        srv.wait(tk, timeout=0.0)
    assert e.value.status == -1
