"""GPU parity of BVH build + closest/any-hit traversal + passes + LiDAR, through the C ABI.

References: the golden fixtures produced by the reference implementation (tests/golden/) and the
FP64 oracle on the same seeded scenes.  Rules (FP32 device path vs FP64 reference):
  * primitive / instance IDs bit-exact except rays whose hit lies within 1e-6 x (|origin| + scene
    extent) of an edge of the hit triangle on either side (helpers.excused_id_mismatch);
  * hit distance, hit point, normal and LiDAR range within 1e-5 relative.
"""
import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes
from helpers import (DIST_REL, EDGE_REL, camera_from, entities_from, excused_id_mismatch, load_golden,
                     point_near_any_edge, ray_edge_distance, scene_extent, to_f32_rays)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


def rays32(rays64):
    r = np.empty(rays64.shape[0], lib.RAY_DTYPE)
    r["o"] = rays64[:, 0:3]
    r["d"] = rays64[:, 3:6]
    r["tmin"] = rays64[:, 6]
    r["tmax"] = np.minimum(rays64[:, 7], np.finfo(np.float32).max)
    return r


def check_closest(tris12, rays64, prim_ref, t_ref, hits, max_excused_frac=0.01):
    prim = hits["prim"].astype(np.int64)
    prim[hits["prim"] == lib.CRT_MISS] = -1
    t = hits["t"].astype(np.float64)
    mism = prim != prim_ref
    if mism.any():
        ok = excused_id_mismatch(tris12, rays64, prim, t, prim_ref, t_ref)
        bad = mism & ~ok
        assert not bad.any(), f"{bad.sum()} unexcused ID mismatches of {len(prim)} (first {np.nonzero(bad)[0][:5]})"
        assert mism.mean() <= max_excused_frac, mism.mean()
    same = (prim == prim_ref) & (prim >= 0)
    np.testing.assert_allclose(t[same], t_ref[same], rtol=DIST_REL)
    return prim, t


def camera_parity(ctx_scene, o, cam, ref=None):
    """GPU passes vs the FP64 oracle (and optionally the reference's own pass outputs `ref` =
    (xyz, ids, normals)).  Instance-id mismatches are allowed only where the pixel's ray passes
    within EDGE_REL * (|origin| + extent) of an edge of the triangle hit by the oracle or the GPU;
    points and normals must agree within 1e-5 on every other hit pixel."""
    gx, gi, gn = ctx_scene.passes(cam)
    ox, oi, on, oprim = o.passes(cam)
    if ref is not None:
        np.testing.assert_array_equal(oi, ref[1])
        np.testing.assert_allclose(ox, ref[0], rtol=0, atol=1e-9)
    rays = oracle.camera_rays(cam)
    tris = o.tris()
    oprim = oprim.ravel()
    hits = ctx_scene.trace_closest(rays32(to_f32_rays(rays)))
    gprim = np.where(hits["prim"] == lib.CRT_MISS, -1, hits["prim"].astype(np.int64))
    eps = EDGE_REL * (np.linalg.norm(rays[:, :3], axis=1) + scene_extent(tris))
    near = np.zeros(len(oprim), bool)
    for pr in (oprim, gprim):
        idx = np.nonzero(pr >= 0)[0]
        near[idx] |= ray_edge_distance(tris, pr[idx], rays[idx]) <= eps[idx]
    near = near.reshape(oi.shape)
    # a pixel that one side misses: its other side's hit point must sit on a triangle edge
    rest = np.nonzero(((gi != oi) & ~near).ravel())[0]
    if len(rest):
        pts = np.where((oi.ravel()[rest] > 0)[:, None], ox.reshape(-1, 3)[rest], gx.reshape(-1, 3)[rest])
        near.ravel()[rest] = point_near_any_edge(tris, pts, eps[rest])
    bad = (gi != oi) & ~near
    assert not bad.any(), f"{bad.sum()} instance-id mismatches away from triangle edges"
    assert (gi != oi).mean() < 0.01
    ok = (gi == oi) & (oi > 0) & ~near
    scale = np.maximum(np.linalg.norm(ox, axis=-1), 1e-30)
    relx = np.linalg.norm(gx - ox, axis=-1)[ok] / scale[ok]
    assert relx.max() < DIST_REL, relx.max()
    assert np.abs(gn - on)[ok].max() < DIST_REL
    both_miss = (oi == 0) & (gi == 0)
    assert (gx[both_miss] == 0).all() and (gn[both_miss] == 0).all()
    return gi, oi


def test_abi_version_and_context(ctx):
    assert lib.load().crt_abi_version() == 2


@pytest.mark.parametrize("name", ["cornell", "asteroid"])
def test_passes_vs_reference_golden(ctx, name):
    d = load_golden(name)
    ents = entities_from(d)
    sc = ctx.scene(ents)
    st = sc.stats()
    assert st["n_tris"] == sum(e.mesh.n_tris for e in ents)
    assert st["n_nodes"] >= 1 and st["depth"] >= 1
    camera_parity(sc, oracle.Scene(ents), camera_from(d), ref=(d["bf_xyz"], d["bf_ids"], d["bf_normals"]))


def test_closest_and_any_vs_reference_golden(ctx):
    d = load_golden("asteroid")
    ents = entities_from(d)
    sc = ctx.scene(ents)
    tris = oracle.Scene(ents).tris()
    rays = d["rays"]
    hits = sc.trace_closest(rays32(rays))
    check_closest(tris, rays, d["closest_prim"], d["closest_t"], hits)
    occ = sc.trace_any(rays32(rays))
    mism = occ != d["any_occluded"]
    assert mism.mean() < 0.005, mism.mean()


def test_batch_lidar_vs_reference_golden(ctx):
    d = load_golden("asteroid")
    sc = ctx.scene(entities_from(d))
    rng, prim = sc.lidar_batch(d["lidar_pos"], d["lidar_rot"])
    ref = d["lidar_range"]
    both = (rng > 0) & (ref > 0)
    assert ((rng > 0) != (ref > 0)).mean() < 0.01
    np.testing.assert_allclose(rng[both], ref[both], rtol=DIST_REL)
    assert ((rng == 0) == (prim == lib.CRT_MISS)).all()


@pytest.fixture(scope="module")
def ast100k():
    ents = [scenes.EntitySpec("a", scenes.asteroid(100_000, seed=3), (0.1, 0.1, 0.1), smooth=True)]
    return ents, oracle.Scene(ents)


def test_asteroid_100k_camera_vs_oracle(ctx, ast100k):
    ents, o = ast100k
    sc = ctx.scene(ents)
    cam = scenes.fov_camera(scenes.TAN5 * 2.4, (256, 256), (0.0, -5000.0, 800.0), (0.0, 0.0, 0.0))
    gi, oi = camera_parity(sc, o, cam)
    assert 0.3 < (oi > 0).mean() < 1.0
    # per-pixel closest hit through the raw ray interface with the same (FP32-rounded) camera rays
    rays = to_f32_rays(oracle.camera_rays(cam))
    prim_o, t_o, _, _ = o.trace_closest(rays)
    hits = sc.trace_closest(rays32(rays))
    check_closest(o.tris(), rays, prim_o, t_o, hits)


def test_random_rays_vs_oracle(ctx, ast100k):
    ents, o = ast100k
    sc = ctx.scene(ents)
    rng = np.random.Generator(np.random.PCG64(99))
    n = 200_000
    org = rng.normal(size=(n, 3))
    org = rng.uniform(1500, 6000, size=(n, 1)) * org / np.linalg.norm(org, axis=1)[:, None]
    tgt = rng.uniform(-1100, 1100, size=(n, 3))
    dirs = tgt - org
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    rays = np.zeros((n, 8))
    rays[:, :3], rays[:, 3:6], rays[:, 7] = org, dirs, 3.0e38
    # a slice of rays start inside the body (origins at radius < 900)
    rays[: n // 10, :3] *= 0.12
    rays = to_f32_rays(rays)
    prim_o, t_o, _, _ = o.trace_closest(rays)
    hits = sc.trace_closest(rays32(rays))
    check_closest(o.tris(), rays, prim_o, t_o, hits)
    # any-hit with finite tmax: bracket the closest hit distance
    has = prim_o >= 0
    sh = rays.copy()
    sh[has, 7] = (t_o[has] * (1 + 1e-4)).astype(np.float32)
    occ = sc.trace_any(rays32(sh))
    assert occ[has].mean() > 0.999
    sh[has, 7] = (t_o[has] * (1 - 1e-3)).astype(np.float32)
    occ2 = sc.trace_any(rays32(sh))
    occ_o = o.trace_any(sh)
    assert (occ2 != occ_o).mean() < 0.002


def test_lidar_grid_matches_per_beam_batch(ctx, ast100k):
    """The beam grid equals do_batch_lidar run with one pose per beam (the reference's only way to
    cast many beams): same ranges, same triangle ids."""
    ents, o = ast100k
    sc = ctx.scene(ents)
    pos = np.array([300.0, -4200.0, 900.0])
    R = scenes.look_at(pos, (0.0, 0.0, 0.0))
    nx = ny = 64
    half = np.deg2rad(5.0)
    rng_g, prim_g = sc.lidar_grid(pos, R, nx, ny, half, half)
    # per-beam rotation R_b with R_b^T (0, 0, -1) = R^T normalize(tan_x, tan_y, -1)
    tx = np.tan(-half + (np.arange(nx) + 0.5) * 2 * half / nx)
    ty = np.tan(-half + (np.arange(ny) + 0.5) * 2 * half / ny)
    s = np.stack(np.broadcast_arrays(tx[None, :], ty[:, None], -np.ones((ny, nx))), -1).reshape(-1, 3)
    s /= np.linalg.norm(s, axis=1)[:, None]
    dw = s @ R            # R^T s for each row
    rots = np.array([scenes.look_at(pos, pos + d, up=(0.0, 0.0, 1.0)) for d in dw])
    rng_o, prim_o = o.lidar_batch(np.repeat(pos[None], nx * ny, 0), rots)
    rng_b, prim_b = sc.lidar_batch(np.repeat(pos[None], nx * ny, 0), rots)
    hit = rng_o > 0
    assert hit.mean() > 0.9
    assert (prim_g.ravel().astype(np.int64) != np.where(prim_o < 0, lib.CRT_MISS, prim_o)).mean() < 0.005
    ok = (prim_g.ravel() == prim_o) & hit
    np.testing.assert_allclose(rng_g.ravel()[ok], rng_o[ok], rtol=DIST_REL)
    np.testing.assert_allclose(rng_b[ok], rng_o[ok], rtol=DIST_REL)


@pytest.mark.parametrize("ntri", [0, 1, 2, 3, 4, 5, 17])
def test_tiny_scenes(ctx, ntri):
    """Empty scene, single-leaf roots (1-3 triangles) and small trees: every ray vs brute force."""
    rng = np.random.Generator(np.random.PCG64(ntri))
    if ntri:
        v = rng.uniform(-1, 1, size=(3 * ntri, 3)).astype(np.float32)
        f = np.arange(3 * ntri, dtype=np.int32).reshape(-1, 3)
        ents = [scenes.EntitySpec("t", scenes.Mesh(v, f))]
    else:
        ents = [scenes.EntitySpec("t", scenes.Mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)))]
    sc = ctx.scene(ents)
    n = 4096
    org = rng.normal(size=(n, 3)) * 3
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    # axis-aligned directions exercise the safe reciprocal
    dirs[:64] = np.eye(3)[rng.integers(0, 3, 64)] * rng.choice([-1, 1], size=(64, 1))
    rays = np.zeros((n, 8))
    rays[:, :3], rays[:, 3:6], rays[:, 7] = org, dirs, 3.0e38
    rays = to_f32_rays(rays)
    hits = sc.trace_closest(rays32(rays))
    if ntri == 0:
        assert (hits["prim"] == lib.CRT_MISS).all()
        return
    o = oracle.Scene(ents)
    prim_o, t_o, _, _ = o.trace_closest(rays)
    check_closest(o.tris(), rays, prim_o, t_o, hits, max_excused_frac=0.02)


def test_ray_edge_cases(ctx):
    ents, _, _ = scenes.cornell()
    sc = ctx.scene(ents)
    # empty batch
    assert sc.trace_closest(np.zeros(0, lib.RAY_DTYPE)).shape == (0,)
    r = np.zeros(8, lib.RAY_DTYPE)
    r["o"] = [0.5, 0.5, 0.5]
    r["d"] = [[0, 1, 0], [0, -1, 0], [1, 0, 0], [0, 0, -1], [np.nan, 0, 0], [0, 0, 0],
              [-0.0, -1.0, -0.0], [-0.0, -0.0, -1.0]]
    r["tmin"], r["tmax"] = 0.0, 3.0e38
    r["tmin"][3], r["tmax"][3] = 5.0, 1.0        # empty interval: no hit
    h = sc.trace_closest(r)
    assert h["prim"][0] != lib.CRT_MISS and abs(h["t"][0] - (0.999 - 0.5)) < 1e-5   # light quad below ceiling
    assert h["prim"][1] != lib.CRT_MISS and abs(h["t"][1] - 0.5) < 1e-6             # floor
    assert h["prim"][2] != lib.CRT_MISS
    assert h["prim"][3] == lib.CRT_MISS
    assert h["prim"][4] == lib.CRT_MISS and h["prim"][5] == lib.CRT_MISS             # NaN / zero direction
    # negative zeros count as negative (std::signbit) and agree with the reciprocal's sign
    assert h["prim"][6] == h["prim"][1] and h["t"][6] == h["t"][1]
    o = oracle.Scene(ents)
    rr = np.zeros((1, 8))
    rr[0, :3], rr[0, 3:6], rr[0, 7] = [0.5, 0.5, 0.5], [-0.0, -0.0, -1.0], np.finfo(np.float64).max
    p_o, t_o, _, _ = o.trace_closest(rr)
    assert h["prim"][7] == p_o[0] and abs(h["t"][7] - t_o[0]) < 1e-6
    occ = sc.trace_any(r)
    assert list(occ[:4]) == [1, 1, 1, 0] and occ[6] == 1 and occ[7] == 1


def test_obj_loader_matches_generator(ctx, tmp_path):
    """crt_mesh_load_obj (obj.hpp semantics) returns the same triangles and vertex normals."""
    m = scenes.asteroid(8000, seed=5)
    p = str(tmp_path / "a.obj")
    m.write_obj(p)
    import ctypes
    L = lib.load()
    h = ctypes.c_void_p()
    assert L.crt_mesh_load_obj(p.encode(), ctypes.byref(h)) == 0
    n = L.crt_mesh_num_tris(h)
    xyz = np.ctypeslib.as_array((ctypes.c_float * (9 * n)).from_address(L.crt_mesh_xyz(h))).copy()
    nrm = np.ctypeslib.as_array((ctypes.c_float * (9 * n)).from_address(L.crt_mesh_normals(h))).copy()
    L.crt_mesh_destroy(h)
    np.testing.assert_array_equal(xyz.reshape(-1, 9), m.soup())
    np.testing.assert_allclose(nrm.reshape(-1, 9), m.soup_normals(), atol=1e-7)
    assert L.crt_mesh_load_obj(str(tmp_path / "missing.obj").encode(), ctypes.byref(h)) == -5


def test_counting_mode(ctx, ast100k):
    ents, _ = ast100k
    sc = ctx.scene(ents)
    cam = scenes.fov_camera(scenes.TAN5 * 2.4, (128, 128), (0.0, -5000.0, 800.0), (0.0, 0.0, 0.0))
    ctx.reset_counters()
    ctx.set_counting(True)
    sc.passes(cam)
    ctx.set_counting(False)
    c = ctx.counters()
    assert c["rays"] == 128 * 128
    assert c["nodes"] >= c["rays"] and c["tris"] > 0
    assert c["launches"] >= 1


def test_z_positive_camera_and_lidar_match_oracle(ctx):
    """Cameras and LiDARs with z_positive (boresight +z in their frame, simple_camera.hpp:61-81,
    simple_lidar.hpp:42-64): passes and per-pose LiDAR equal the oracle's; a z_positive beam grid
    with the frame turned about y equals the default grid mirrored in x."""
    d = load_golden("cornell")
    ents = entities_from(d)
    sc, o = ctx.scene(ents), oracle.Scene(ents)
    F = np.diag([-1.0, 1.0, -1.0])   # half turn about y: the +z boresight looks where -z did
    cam = camera_from(d, "rcam")
    camz = dict(cam, z_positive=True, rotation=F @ np.asarray(cam["rotation"]), resolution=[40, 32])
    gx, gi, gn = sc.passes(camz)
    ox, oi, on, _ = o.passes(camz)
    assert (oi > 0).mean() > 0.9
    assert (gi == oi).mean() > 0.99
    ok = (gi == oi) & (oi > 0)
    np.testing.assert_allclose(gx[ok], ox[ok], rtol=DIST_REL, atol=1e-9)
    pos = np.array([[0.5, 0.5, 2.4], [0.3, 0.6, 2.0], [0.7, 0.2, 1.5]])
    rot = np.stack([F, F, F]).reshape(3, 9)
    rng, prim = sc.lidar_batch(pos, rot, z_positive=True)
    rng_o, prim_o = o.lidar_batch(pos, rot, z_positive=True)
    np.testing.assert_array_equal(prim, prim_o)
    np.testing.assert_allclose(rng, rng_o, rtol=DIST_REL)
    g_z, p_z = sc.lidar_grid([0.5, 0.5, 2.4], F, 11, 9, 0.3, 0.2, z_positive=True)
    g_0, p_0 = sc.lidar_grid([0.5, 0.5, 2.4], np.eye(3), 11, 9, 0.3, 0.2)
    assert (p_z[:, ::-1] == p_0).mean() > 0.95
    same = p_z[:, ::-1] == p_0
    np.testing.assert_allclose(g_z[:, ::-1][same], g_0[same], rtol=1e-9)
