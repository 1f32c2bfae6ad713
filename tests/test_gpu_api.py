"""The drop-in `crt` package: the reference's Python calls, unchanged, against the reference's outputs.

Scenes are written as OBJ files and loaded through crt.BodyFixedEntity / crt.Entity, exactly as a
reference user would; outputs are compared with the fixtures the reference produced on the same
files (tests/golden/).
"""
import numpy as np
import pytest

import oracle
from crt_gb300 import workloads
from helpers import (DIST_REL, TriIndex, camera_from, check_passes, edge_eps, entities_from, load_golden,
                     unexcused)

pytestmark = pytest.mark.gpu


def crt_objects(d, tmp_path, dynamic=False):
    import crt
    from crt.cameras import SimpleCamera
    ents = entities_from(d)
    objs = []
    for i, e in enumerate(ents):
        p = str(tmp_path / f"{i}.obj")
        e.mesh.write_obj(p)
        cls = crt.Entity if dynamic else crt.BodyFixedEntity
        objs.append(cls(p, color=list(e.color), smooth_shading=e.smooth, position=e.position, rotation=e.rotation,
                        scale=e.scale))
    cam = camera_from(d)
    camera = SimpleCamera(cam["focal_length"], cam["resolution"], cam["sensor_size"], cam["z_positive"],
                          position=cam["position"], rotation=cam["rotation"])
    return objs, camera


def agree(d, ids, xyz, normals, ref_ids, ref_xyz, ref_n, cam=None):
    """The API's passes against the reference's: every pixel agrees (ids, points and normals within
    DIST_REL) or its ray passes within the edge distance of an edge of the triangle that the oracle
    (which reproduces the reference's passes exactly) hit, or of a triangle at either side's hit
    point (helpers.check_passes)."""
    ents = entities_from(d)
    o = oracle.Scene(ents)
    cam = cam or camera_from(d)
    _, oi, _, oprim = o.passes(cam)
    np.testing.assert_array_equal(oi, ref_ids)
    check_passes(TriIndex(o.tris()), workloads.camera_rays(cam), (xyz, ids, normals),
                 (ref_xyz, ref_ids, ref_n, oprim))


@pytest.mark.parametrize("name", ["cornell", "asteroid"])
def test_body_fixed_group_passes(name, tmp_path):
    import crt
    d = load_golden(name)
    objs, camera = crt_objects(d, tmp_path)
    group = crt.BodyFixedGroup(objs)
    ids = group.instance_pass(camera)
    xyz = group.intersection_pass(camera)
    nrm = group.normal_pass(camera)
    assert ids.dtype == np.uint32 and xyz.dtype == np.float64 and xyz.shape == d["bf_xyz"].shape
    agree(d, ids, xyz, nrm, d["bf_ids"], d["bf_xyz"], d["bf_normals"])
    ids2, img = group.instance_pass(camera, return_image=True)
    assert img.shape == ids.shape + (3,)


def test_dynamic_rendering_functions(tmp_path):
    from crt import rendering
    d = load_golden("cornell")
    objs, camera = crt_objects(d, tmp_path, dynamic=True)
    ids = rendering.instance_pass(camera, objs)
    xyz = rendering.intersection_pass(camera, objs)
    nrm = rendering.normal_pass(camera, objs)
    agree(d, ids, xyz, nrm, d["dyn_ids"], d["dyn_xyz"], d["dyn_normals"])


def test_render_and_lidar_through_api(tmp_path):
    import crt
    from crt.lidars import SimpleLidar
    from crt.lights import PointLight
    d = load_golden("asteroid")
    objs, camera = crt_objects(d, tmp_path)
    group = crt.BodyFixedGroup(objs)
    light = PointLight(1.0e18, position=1.0e9 * np.array([0.6, 0.0, 0.8]))
    img = group.render(camera, light, 1, 1, 1.0, 1)
    assert img.dtype == np.uint8 and img.shape == (64, 64, 4) and (img[..., 3] == 255).all()
    img2, rad = group.render(camera, [light], 1, 1, 1.0, 1, return_radiance=True)
    np.testing.assert_array_equal(img, img2)
    # batch LiDAR with the reference's (3, 3, n) rotation layout
    lidar = SimpleLidar()
    pos, rot = d["lidar_pos"], d["lidar_rot"]
    lidar.batch_set_pose(pos, np.transpose(rot, (1, 2, 0)))
    rng = group.batch_simulate_lidar(lidar)
    assert rng.shape == (1, len(pos))
    ref = d["lidar_range"]
    # hit / miss and ranges: equal within DIST_REL, or the boresight passes within the edge distance
    # of an edge of the oracle's triangle or of a triangle at the GPU's hit point
    o = oracle.Scene(entities_from(d))
    rng_o, prim_o = o.lidar_batch(pos, rot)
    np.testing.assert_array_equal(rng_o, ref)
    R = np.asarray(rot).reshape(-1, 3, 3)
    rays = np.zeros((len(pos), 8))
    rays[:, 0:3], rays[:, 3:6], rays[:, 7] = pos, -R[:, 2, :], np.finfo(np.float64).max
    index = TriIndex(o.tris())
    diff = np.nonzero(((rng[0] == 0) != (ref == 0)) | (np.abs(rng[0] - ref) > DIST_REL * np.abs(ref)))[0]
    gpt = np.where((rng[0][diff] > 0)[:, None], rays[diff, 0:3] + rng[0][diff][:, None] * rays[diff, 3:6], np.nan)
    bad = unexcused(index, rays[diff], edge_eps(rays[diff], index.extent), prims=[prim_o[diff]], points=[gpt])
    assert len(bad) == 0, (diff[bad][:5], rng[0][diff[bad][:5]], ref[diff[bad][:5]])
    # single-pose LiDAR equals the first batch pose
    single = SimpleLidar(position=pos[0], rotation=rot[0])
    assert abs(group.simulate_lidar(single) - rng[0, 0]) <= DIST_REL * max(rng[0, 0], 1.0)
    # beam-grid extension
    scan = SimpleLidar(position=pos[1], rotation=rot[1])
    scan.set_beam_grid(32, 16, np.deg2rad(4), np.deg2rad(2))
    r2, p2 = group.lidar_scan(scan)
    assert r2.shape == (16, 32) and p2.dtype == np.uint32
    assert ((r2 == 0) == (p2 == 0xFFFFFFFF)).all()


def test_transform_to_body_moves_queries(tmp_path):
    """A group pose is applied to cameras through transform_to_body (body_fixed.py:87-101): posing the
    group and the camera together gives the unposed query's body-frame rays, so instance ids equal the
    oracle's on the unposed camera except on rays at triangle edges."""
    import crt
    from crt.cameras import SimpleCamera
    d = load_golden("cornell")
    objs, camera = crt_objects(d, tmp_path)
    group = crt.BodyFixedGroup(objs)
    cam = camera_from(d)

    def query(position, rotation):
        # the passes move the camera they are given into the body frame (as the reference does), so
        # each pass gets a fresh camera object
        mk = lambda: SimpleCamera(cam["focal_length"], cam["resolution"], cam["sensor_size"], cam["z_positive"],
                                  position=position, rotation=rotation)
        return group.instance_pass(mk()), group.intersection_pass(mk())

    results = [query(cam["position"], cam["rotation"])]
    # rotate the group by 90 deg about z and move it; rotate / move the camera with it
    Rz = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    t = np.array([10.0, -3.0, 2.0])
    group.set_pose(t, Rz)
    results.append(query(Rz.T @ cam["position"] + t, cam["rotation"] @ Rz))
    o = oracle.Scene(entities_from(d))
    ox, oi, _, oprim = o.passes(cam)
    rays = workloads.camera_rays(cam)
    index = TriIndex(o.tris())
    for got, gx in results:
        diff = np.nonzero((got != oi).ravel())[0]
        pts = [np.where((oi.ravel()[diff] > 0)[:, None], ox.reshape(-1, 3)[diff], np.nan),
               np.where((got.ravel()[diff] > 0)[:, None], gx.reshape(-1, 3)[diff], np.nan)]
        bad = unexcused(index, rays[diff], edge_eps(rays[diff], index.extent), prims=[oprim.ravel()[diff]],
                        points=pts)
        assert len(bad) == 0, (diff[bad][:5], got.ravel()[diff[bad][:5]], oi.ravel()[diff[bad][:5]])
    np.testing.assert_array_equal(results[0][0], results[1][0])
