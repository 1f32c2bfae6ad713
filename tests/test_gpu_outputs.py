"""Output placement through the C ABI: results written to device memory, to pageable host memory
(staged in device scratch and copied back) and to mapped page-locked host memory (written by the
kernels in place) are bit-identical, for renders, passes, LiDAR grids and ray traces."""
import numpy as np
import pytest

from crt_gb300 import lib, scenes, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    torch = pytest.importorskip("torch")
    ctx = lib.Context(0)
    sc = ctx.scene(workloads.asteroid_entities(100_000, seed=5))
    yield torch, ctx, sc
    ctx.close()


def buffers(torch, shape, dtype):
    """The same output three ways: device tensor, pageable numpy array, pinned host tensor."""
    tdt = {np.uint8: torch.uint8, np.float32: torch.float32, np.float64: torch.float64, np.uint32: torch.int32}[dtype]
    return (torch.empty(shape, dtype=tdt, device="cuda"), np.empty(shape, dtype),
            torch.empty(shape, dtype=tdt, pin_memory=True))


def host(a, dtype):
    if hasattr(a, "cpu"):
        return a.cpu().numpy().view(dtype)
    return a


def test_render_outputs_agree(scene):
    torch, ctx, sc = scene
    cfg = workloads.asteroid_config(256, 64)
    cam, lights = cfg["camera"], cfg["lights"]
    outs = []
    for rgba, rad in zip(buffers(torch, (256, 256, 4), np.uint8), buffers(torch, (256, 256, 4), np.float32)):
        sc.render(cam, lights, 4, 4, 0.0, 2, seed=3, out_rgba=rgba, out_radiance=rad)
        ctx.synchronize()
        outs.append((host(rgba, np.uint8), host(rad, np.float32)))
    assert outs[0][0].any() and np.isfinite(outs[0][1]).all()
    for o in outs[1:]:
        np.testing.assert_array_equal(o[0], outs[0][0])
        np.testing.assert_array_equal(o[1], outs[0][1])


def test_passes_lidar_and_traces_agree(scene):
    torch, ctx, sc = scene
    cfg = workloads.asteroid_config(192, 96)
    cam, lid = cfg["camera"], cfg["lidar"]
    res = []
    for rng, prim in zip(buffers(torch, (96, 96), np.float64), buffers(torch, (96, 96), np.uint32)):
        sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"],
                      out_range=rng, out_prim=prim)
        ctx.synchronize()
        res.append((host(rng, np.float64), host(prim, np.uint32)))
    assert (res[0][1] != lib.CRT_MISS).any()
    for r in res[1:]:
        np.testing.assert_array_equal(r[0], res[0][0])
        np.testing.assert_array_equal(r[1], res[0][1])
    passes = []
    for xyz, ids, nrm in zip(buffers(torch, (192, 192, 3), np.float64), buffers(torch, (192, 192), np.uint32),
                             buffers(torch, (192, 192, 3), np.float64)):
        sc.passes(cam, xyz=xyz, ids=ids, normals=nrm)
        ctx.synchronize()
        passes.append((host(xyz, np.float64), host(ids, np.uint32), host(nrm, np.float64)))
    for p in passes[1:]:
        for a, b in zip(p, passes[0]):
            np.testing.assert_array_equal(a, b)
    rays64 = workloads.camera_rays(cam)
    rays = np.zeros(len(rays64), lib.RAY_DTYPE)
    rays["o"] = rays64[:, 0:3]
    rays["d"] = rays64[:, 3:6]
    rays["tmax"] = np.finfo(np.float32).max
    hits = []
    for out in buffers(torch, (len(rays), 4), np.float32):
        sc.trace_closest(rays, out=out)
        ctx.synchronize()
        hits.append(host(out, np.float32).view(np.uint32))
    for h in hits[1:]:
        np.testing.assert_array_equal(h, hits[0])
