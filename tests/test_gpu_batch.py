"""Batched requests (crt_batch): many renders and LiDAR scans, on several resident scenes, in one set
of persistent launches.  Every request's result must equal its standalone call bit for bit: the
random streams are keyed by (seed, request) and pixels consume their samples in order, so grouping
requests or samples into waves changes nothing."""
import numpy as np
import pytest

from crt_gb300 import lib, scenes
from helpers import camera_from, entities_from, lights_from, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ctx = lib.Context(0)
    d = load_golden("cornell")
    cornell = ctx.scene(entities_from(d))
    ast = ctx.scene([scenes.EntitySpec("a", scenes.asteroid(20_000, seed=4), (0.2, 0.2, 0.2), smooth=True)])
    yield ctx, d, cornell, ast
    ctx.close()


def make_requests(d, cornell, ast):
    cam = camera_from(d, "rcam")
    area = lights_from(d["lights"])
    point = lights_from(d["point_lights"])
    sun = [dict(type="point", intensity=1e18, position=1e9 * scenes.unit_vector(3))]
    reqs = []
    rng = np.random.Generator(np.random.PCG64(5))
    for k in range(6):
        res = int(rng.choice([8, 16, 24, 40]))
        spp = int(rng.choice([1, 2, 5]))
        nb = int(rng.choice([1, 2, 3]))
        reqs.append(dict(kind="render", scene=cornell, camera=dict(cam, resolution=[res, res + 3]),
                         lights=area + (point if k % 2 else []), min_samples=spp, max_samples=spp,
                         noise_threshold=0.0, num_bounces=nb, seed=11 + k, request=k, radiance=True))
    for k in range(3):
        pos = 4000.0 * scenes.unit_vector(40 + k)
        reqs.append(dict(kind="render", scene=ast, camera=scenes.fov_camera(0.25, (32, 20), pos, (0, 0, 0)),
                         lights=sun, min_samples=2, max_samples=2, noise_threshold=0.0, num_bounces=2, seed=3,
                         request=100 + k, radiance=True))
    for k in range(4):
        pos = 3500.0 * scenes.unit_vector(60 + k)
        reqs.append(dict(kind="lidar", scene=ast, position=pos, rotation=scenes.look_at(pos, (0, 0, 0)),
                         nx=17 + 8 * k, ny=9 + 4 * k, half_x=np.deg2rad(6), half_y=np.deg2rad(4)))
    reqs.append(dict(kind="lidar", scene=cornell, position=[0.5, 0.5, 2.4], rotation=np.eye(3), nx=13, ny=11,
                     half_x=0.2, half_y=0.2))
    # 96,000 paths: more than the smallest wave (65,536 paths), so that setting splits the batch
    reqs.append(dict(kind="render", scene=cornell, camera=dict(cam, resolution=[160, 150]), lights=area,
                     min_samples=4, max_samples=4, noise_threshold=0.0, num_bounces=1, seed=29, request=50,
                     radiance=True))
    order = rng.permutation(len(reqs))
    return [reqs[i] for i in order]


def standalone(q):
    sc = q["scene"]
    if q["kind"] == "srp":
        f, t, _ = sc.srp(q["sun_dir"], q["quaternions"], q["grid"], num_bounces=q["num_bounces"])
        return f, t
    if q["kind"] == "render":
        return sc.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], q["noise_threshold"],
                         q["num_bounces"], seed=q["seed"], request=q["request"])
    return sc.lidar_grid(q["position"], q["rotation"], q["nx"], q["ny"], q["half_x"], q["half_y"])


def assert_same(a, b):
    for x, y in zip(a, b):
        if x is None:
            assert y is None
        else:
            np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("use_graphs,wave_paths", [(True, 1 << 23), (False, 1 << 23), (True, 1 << 16),
                                                   (False, 1 << 16)])
def test_batch_equals_standalone(setup, use_graphs, wave_paths):
    ctx, d, cornell, ast = setup
    reqs = make_requests(d, cornell, ast)
    ctx.set_tuning(queue_chunk=1, wave_paths=1 << 23, use_graphs=True)
    alone = [standalone(q) for q in reqs]
    ctx.set_tuning(queue_chunk=2, wave_paths=wave_paths, use_graphs=use_graphs)
    outs, st = ctx.batch(reqs)
    ctx.set_tuning()
    for q, a, b in zip(reqs, alone, outs):
        assert_same(a, b)
    assert st["render_paths"] == sum(int(q["camera"]["resolution"][0]) * int(q["camera"]["resolution"][1]) *
                                     q["max_samples"] for q in reqs if q["kind"] == "render")
    if wave_paths == 1 << 16:
        assert st["waves"] > 1


def test_adaptive_requests_in_batch(setup):
    ctx, d, cornell, ast = setup
    cam = camera_from(d, "rcam")
    area = lights_from(d["lights"])
    reqs = [dict(kind="render", scene=cornell, camera=dict(cam, resolution=[20, 16]), lights=area, min_samples=2,
                 max_samples=24, noise_threshold=1.5, num_bounces=2, seed=7, request=r, radiance=True)
            for r in range(3)]
    reqs.append(dict(kind="render", scene=cornell, camera=dict(cam, resolution=[12, 12]), lights=area,
                     min_samples=4, max_samples=4, noise_threshold=0.0, num_bounces=2, seed=8, request=9,
                     radiance=True))
    alone = [standalone(q) for q in reqs]
    outs, st = ctx.batch(reqs)
    for a, b in zip(alone, outs):
        assert_same(a, b)
    assert st["waves"] > 2


def test_empty_and_lidar_only_batches(setup):
    ctx, d, cornell, ast = setup
    outs, st = ctx.batch([])
    assert outs == [] and st["waves"] == 0
    q = dict(kind="lidar", scene=cornell, position=[0.5, 0.5, 2.4], rotation=np.eye(3), nx=7, ny=5, half_x=0.1,
             half_y=0.1)
    outs, st = ctx.batch([q])
    assert_same(outs[0], standalone(q))


def test_bad_request_rejected(setup):
    ctx, d, cornell, ast = setup
    q = dict(kind="lidar", scene=cornell, position=[0.5, 0.5, 2.4], rotation=np.eye(3), nx=0, ny=5, half_x=0.1,
             half_y=0.1)
    with pytest.raises(lib.CrtError):
        ctx.batch([q])


def srp_requests(ctx, ast):
    craft = ctx.scene(scenes.spacecraft(bus_cell=0.25, panel_cell=0.2, dish_rings=16, dish_segments=16))
    return [
        # 256^2: one attitude per 65,536-item wave at the smallest wave size; specular panels
        dict(kind="srp", scene=craft, sun_dir=[1.0, 0.2, -0.1], quaternions=scenes.random_quaternions(3, seed=2),
             grid=256, num_bounces=2),
        # 600^2: one attitude spans several waves (parts of an attitude)
        dict(kind="srp", scene=craft, sun_dir=[0.0, 1.0, 0.0], quaternions=scenes.random_quaternions(1, seed=3),
             grid=600, num_bounces=1),
        # no specular entity: primary segment only, several attitudes per wave
        dict(kind="srp", scene=ast, sun_dir=[0.3, -0.5, 0.8], quaternions=scenes.random_quaternions(5, seed=4),
             grid=128, num_bounces=2),
    ]


@pytest.mark.parametrize("wave_paths,graphs", [(1 << 23, True), (1 << 16, True), (1 << 16, False)])
def test_mixed_batch_with_srp_equals_standalone(setup, wave_paths, graphs):
    """crt_batch_mixed: SRP requests ride in the waves' primary traces beside camera paths and LiDAR
    beams.  Renders and LiDAR scans equal their standalone calls bit for bit, and force and torque
    equal crt_srp's bit for bit however the sun-ray grids are cut into waves (partial sums are kept
    per block of the request's items), with the waves replayed as one CUDA graph (the SRP stages read
    the wave's range from its device descriptor) or launched one by one."""
    ctx, d, cornell, ast = setup
    reqs = make_requests(d, cornell, ast)[:8]
    srps = srp_requests(ctx, ast)
    mixed = reqs[:3] + [srps[0]] + reqs[3:6] + srps[1:] + reqs[6:]
    ctx.set_tuning(queue_chunk=1, wave_paths=1 << 23, use_graphs=True)
    alone = [standalone(q) for q in mixed]
    ctx.set_tuning(queue_chunk=1, wave_paths=wave_paths, use_graphs=graphs)
    outs, st = ctx.batch(mixed)
    ctx.set_tuning()
    for q, a, b in zip(mixed, alone, outs):
        assert_same(a, b)
    f, t = outs[3]
    assert np.isfinite(f).all() and (np.abs(f).sum(1) > 0).all()
    if wave_paths == 1 << 16:
        assert st["waves"] >= 6 + 3


def test_srp_only_batch_and_device_outputs(setup):
    """A batch of SRP requests alone, with force / torque in device memory, equals crt_srp."""
    torch = pytest.importorskip("torch")
    ctx, d, cornell, ast = setup
    q = srp_requests(ctx, ast)[0]
    f_dev = torch.zeros((3, 3), dtype=torch.float64, device="cuda")
    t_dev = torch.zeros((3, 3), dtype=torch.float64, device="cuda")
    ctx.batch([q], outputs=[(f_dev, t_dev)])
    torch.cuda.synchronize()
    f, t = standalone(q)
    np.testing.assert_array_equal(f_dev.cpu().numpy(), f)
    np.testing.assert_array_equal(t_dev.cpu().numpy(), t)


def test_mixed_batch_with_adaptive_render(setup):
    """Adaptive renders run their later samples in waves planned after the SRP ranges: results still
    equal the standalone calls."""
    ctx, d, cornell, ast = setup
    cam = camera_from(d, "rcam")
    reqs = [dict(kind="render", scene=cornell, camera=dict(cam, resolution=[20, 16]), lights=lights_from(d["lights"]),
                 min_samples=2, max_samples=16, noise_threshold=1.5, num_bounces=2, seed=7, request=3, radiance=True),
            srp_requests(ctx, ast)[1]]
    alone = [standalone(q) for q in reqs]
    ctx.set_tuning(queue_chunk=1, wave_paths=1 << 16, use_graphs=True)
    outs, st = ctx.batch(reqs)
    ctx.set_tuning()
    for a, b in zip(alone, outs):
        assert_same(a, b)
    assert st["waves"] > 6
