"""GPU parity of BVH build + closest/any-hit traversal + passes + LiDAR, through the C ABI.

References: the golden fixtures produced by the reference implementation (tests/golden/) and the
FP64 oracle on the same seeded scenes.  Rules (FP32 device path vs FP64 reference):
  * primitive / instance IDs bit-exact except rays whose line passes within 1e-6 x (|origin| + scene
    extent) of an edge of the triangle hit on either side (helpers.unexcused); no other ray may
    differ, and any-hit flags follow the same rule;
  * hit distance, hit point, normal and LiDAR range within 1e-5 relative.
"""
import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes, workloads
from helpers import (DIST_REL, TriIndex, camera_from, check_hits, check_occlusion, check_passes, entities_from,
                     load_golden, to_f32_rays)

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


def gpu_prim(hits):
    return np.where(hits["prim"] == lib.CRT_MISS, -1, hits["prim"].astype(np.int64))


def check_closest(index, rays64, prim_ref, t_ref, hits):
    """Closest hits equal the reference's (same triangle, t within DIST_REL) on every ray the edge
    rule does not excuse."""
    return check_hits(index, rays64, gpu_prim(hits), hits["t"], prim_ref, t_ref)


def camera_parity(ctx_scene, o, cam, ref=None, index=None):
    """GPU passes vs the FP64 oracle (and the oracle vs the reference's own pass outputs `ref` =
    (xyz, ids, normals)): every pixel agrees or is excused by the edge rule (helpers.check_passes)."""
    gx, gi, gn = ctx_scene.passes(cam)
    ox, oi, on, oprim = o.passes(cam)
    if ref is not None:
        np.testing.assert_array_equal(oi, ref[1])
        np.testing.assert_allclose(ox, ref[0], rtol=0, atol=1e-9)
    index = index or TriIndex(o.tris())
    rays = workloads.camera_rays(cam)
    gprim = gpu_prim(ctx_scene.trace_closest(rays32(to_f32_rays(rays))))
    check_passes(index, rays, (gx, gi, gn), (ox, oi, on, oprim), gprim=gprim)
    return gi, oi


def lidar_rays(pos, rot, z_positive=False):
    """FP64 boresight rays of per-pose LiDAR (SimpleLidar::batch_cast_rays: R^T (0, 0, -+1))."""
    rot = np.asarray(rot, dtype=np.float64).reshape(-1, 3, 3)
    b = np.array([0.0, 0.0, 1.0 if z_positive else -1.0])
    rays = np.zeros((len(rot), 8))
    rays[:, 0:3] = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    rays[:, 3:6] = np.einsum("nij,i->nj", rot, b)
    rays[:, 7] = np.finfo(np.float64).max
    return rays


def check_lidar(index, pos, rot, rng, prim, rng_ref, prim_ref, z_positive=False):
    """Per-pose LiDAR ranges / triangles against the reference's: the edge rule on the boresight rays,
    ranges within DIST_REL, a miss reported as range 0."""
    assert ((rng == 0) == (prim == lib.CRT_MISS)).all()
    gp = np.where(prim == lib.CRT_MISS, -1, prim.astype(np.int64))
    op = np.asarray(prim_ref, dtype=np.int64) if prim_ref is not None else np.where(rng_ref > 0, -2, -1)
    return check_hits(index, lidar_rays(pos, rot, z_positive), gp, rng, op, rng_ref)


def test_abi_version_and_context(ctx):
    assert lib.load().crt_abi_version() == 3


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
    index = TriIndex(tris)
    hits = sc.trace_closest(rays32(rays))
    check_closest(index, rays, d["closest_prim"], d["closest_t"], hits)
    occ = sc.trace_any(rays32(rays))

    def occluders(idx):   # each side's closest hit of the same rays
        gp = gpu_prim(hits)[idx]
        op = d["closest_prim"][idx]
        return [gp, op], [], [hits["t"][idx].astype(np.float64), d["closest_t"][idx]]
    check_occlusion(index, rays, occ, d["any_occluded"], occluders)


def test_batch_lidar_vs_reference_golden(ctx):
    d = load_golden("asteroid")
    sc = ctx.scene(entities_from(d))
    ents = entities_from(d)
    o = oracle.Scene(ents)
    rng, prim = sc.lidar_batch(d["lidar_pos"], d["lidar_rot"])
    rng_o, prim_o = o.lidar_batch(d["lidar_pos"], d["lidar_rot"])
    np.testing.assert_array_equal(rng_o, d["lidar_range"])     # the oracle reproduces the reference
    check_lidar(TriIndex(o.tris()), d["lidar_pos"], d["lidar_rot"], rng, prim, d["lidar_range"], prim_o)


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
    check_closest(TriIndex(o.tris()), rays, prim_o, t_o, hits)


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
    index = TriIndex(o.tris())
    check_closest(index, rays, prim_o, t_o, hits)
    # any-hit with finite tmax: just past and short of the closest hit distance, against the oracle;
    # where they differ, the side reporting the occlusion meets an edge or meets its triangle at tmax
    has = prim_o >= 0
    for f in (1 + 1e-4, 1 - 1e-3):
        sh = rays.copy()
        sh[has, 7] = (t_o[has] * f).astype(np.float32)
        occ = sc.trace_any(rays32(sh))
        occ_o = o.trace_any(sh)
        hg = sc.trace_closest(rays32(sh))
        po, to, _, _ = o.trace_closest(sh)

        def occluders(idx):
            return [gpu_prim(hg)[idx], po[idx]], [], [hg["t"][idx].astype(np.float64), to[idx]]
        check_occlusion(index, sh, occ, occ_o, occluders)
        if f > 1:
            assert occ_o[has].all()


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
    index = TriIndex(o.tris())
    poses = np.repeat(pos[None], nx * ny, 0)
    check_lidar(index, poses, rots, rng_g.ravel(), prim_g.ravel(), rng_o, prim_o)
    check_lidar(index, poses, rots, rng_b, prim_b, rng_o, prim_o)


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
    check_closest(TriIndex(o.tris()), rays, prim_o, t_o, hits)


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
    index = TriIndex(o.tris())
    gi, oi = camera_parity(sc, o, camz, index=index)
    assert (oi > 0).mean() > 0.9
    pos = np.array([[0.5, 0.5, 2.4], [0.3, 0.6, 2.0], [0.7, 0.2, 1.5]])
    rot = np.stack([F, F, F]).reshape(3, 9)
    rng, prim = sc.lidar_batch(pos, rot, z_positive=True)
    rng_o, prim_o = o.lidar_batch(pos, rot, z_positive=True)
    check_lidar(index, pos, rot, rng, prim, rng_o, prim_o, z_positive=True)
    # beam grid with the +z boresight against the oracle's closest hits of the same FP64 beams
    lid = dict(position=[0.5, 0.5, 2.4], rotation=F, nx=11, ny=9, half_x=0.3, half_y=0.2, z_positive=True)
    g_z, p_z = sc.lidar_grid(lid["position"], F, 11, 9, 0.3, 0.2, z_positive=True)
    beams = workloads.lidar_grid_rays(lid)
    pb, tb, _, _ = o.trace_closest(beams)
    check_hits(index, beams, np.where(p_z.ravel() == lib.CRT_MISS, -1, p_z.ravel().astype(np.int64)),
               g_z.ravel(), pb, np.where(pb >= 0, tb, 0.0))
    assert (pb >= 0).mean() > 0.9
