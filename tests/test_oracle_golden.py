"""Pin the CPU oracle against fixtures produced by the reference implementation (no GPU).

The fixtures in tests/golden/ were generated by tests/golden/make_golden.py from the reference
compiled from its own sources.  The oracle restates the same FP64 arithmetic, so outside exact
ties (rays through shared edges, where the reference keeps the later-tested triangle) results
are identical.
"""
import numpy as np
import pytest

import oracle
from helpers import (camera_from, entities_from, excused_id_mismatch, lights_from, load_golden,
                     radiance_stats_ok)


@pytest.fixture(scope="module")
def cornell():
    d = load_golden("cornell")
    return d, oracle.Scene(entities_from(d))


@pytest.fixture(scope="module")
def asteroid():
    d = load_golden("asteroid")
    return d, oracle.Scene(entities_from(d))


def test_scene_assembly_matches_reference(asteroid):
    """Transform chain resize -> rotate -> translate (transform.hpp:43-85) reproduces the reference's
    FP64 triangles bit for bit, including the smooth-shading vertex normals."""
    d, s = asteroid
    ref = d["ref_tris"]
    assert s.n_tris == ref.shape[0]
    np.testing.assert_array_equal(s.tris(), ref[:, :12])


@pytest.mark.parametrize("which", ["bf", "dyn"])
def test_cornell_passes(cornell, which):
    d, s = cornell
    xyz, ids, nrm, prim = s.passes(camera_from(d))
    np.testing.assert_array_equal(ids, d[f"{which}_ids"])
    np.testing.assert_allclose(xyz, d[f"{which}_xyz"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(nrm, d[f"{which}_normals"], rtol=0, atol=1e-12)
    assert 0.5 < (ids > 0).mean() < 1.0


def test_asteroid_passes(asteroid):
    d, s = asteroid
    xyz, ids, nrm, prim = s.passes(camera_from(d))
    np.testing.assert_array_equal(ids, d["bf_ids"])
    np.testing.assert_allclose(xyz, d["bf_xyz"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(nrm, d["bf_normals"], rtol=0, atol=1e-12)
    assert (ids == 1).any() and (ids == 2).any() and (ids == 0).any()


def test_closest_hit_rays(asteroid):
    d, s = asteroid
    rays = d["rays"]
    prim, t, u, v = s.trace_closest(rays)
    ref_p = d["closest_prim"]
    mism = prim != ref_p
    if mism.any():
        ok = excused_id_mismatch(s.tris(), rays, prim, t, ref_p, d["closest_t"])
        assert ok[mism].all()
    same = ~mism & (prim >= 0)
    np.testing.assert_allclose(t[same], d["closest_t"][same], rtol=1e-12)
    np.testing.assert_allclose(u[same], d["closest_u"][same], rtol=0, atol=1e-12)
    np.testing.assert_allclose(v[same], d["closest_v"][same], rtol=0, atol=1e-12)
    assert 0.2 < (prim >= 0).mean() < 0.9


def test_any_hit_rays(asteroid):
    d, s = asteroid
    occ = s.trace_any(d["rays"])
    assert (occ != d["any_occluded"]).sum() == 0
    # finite-tmax rays (first quarter) are occluded less often than unbounded ones
    q = len(occ) // 4
    assert occ[:q].mean() <= occ[q:].mean()


def test_batch_lidar(asteroid):
    d, s = asteroid
    rng, prim = s.lidar_batch(d["lidar_pos"], d["lidar_rot"])
    np.testing.assert_allclose(rng, d["lidar_range"], rtol=1e-12, atol=0)
    assert ((rng == 0) == (prim < 0)).all()


def test_point_light_render_deterministic(cornell):
    """1 spp at integer pixel coordinates, 1 bounce: no random draws, so the radiance is exact."""
    d, s = cornell
    rad, u8, taken = s.render(camera_from(d, "rcam"), lights_from(d["point_lights"]), 1, 1, 0.0, 1)
    np.testing.assert_allclose(rad[..., :3], d["point_radiance"], rtol=1e-6, atol=1e-6)
    assert (rad[..., 3] == 1).all() and (taken == 1).all()
    exp_u8 = np.clip(d["point_radiance"] * 256, 0, 255).astype(np.uint8)
    assert (np.abs(u8[..., :3].astype(int) - exp_u8) <= 1).all()


def test_area_light_render_statistics(cornell):
    """Monte-Carlo radiance vs the reference path tracer (different random streams): per pixel
    within 4 sigma, image mean within 0.5 %.  Pixels whose primary hit lies within 5 cm of the
    light plane are excluded: there the reference's area light (intensity / d^2 with no cosine
    term, lights/area_light.hpp:70-72) gives an estimator of unbounded variance."""
    d, s = cornell
    cam = camera_from(d, "rcam")
    spp = int(d["render_spp"])
    bounces = int(d["render_bounces"])
    lights = lights_from(d["lights"])
    # Welford second moments of the oracle from repeated independent single-sample renders would be
    # slow; instead render twice with disjoint seeds and use the reference's per-pixel variance.
    rad, _, _ = s.render(cam, lights, spp, spp, 0.0, bounces, seed=11)
    xyz, ids, _, _ = s.passes(cam)
    mask = ~((ids == 1) & (xyz[..., 1] > 0.94)) & (ids != 6) & (ids > 0)
    ref = d["render_mean"]
    m2 = d["render_m2"]
    z = radiance_stats_ok(rad[..., :3], m2, spp, ref, m2, spp, mask=np.repeat(mask[..., None], 3, -1))
    assert (z > 4).mean() < 0.01, (z > 4).mean()
    ours, theirs = rad[..., :3][mask].mean(), ref[mask].mean()
    assert abs(ours / theirs - 1) < 0.005, (ours, theirs)


def test_philox_known_answer():
    """Philox4x32-10 known-answer vectors from the Random123 distribution (counter, key -> output)."""
    np.testing.assert_array_equal(oracle.philox(0, 0, 0, 0, 0, 0),
                                  np.array([0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8], dtype=np.uint32))
    np.testing.assert_array_equal(
        oracle.philox(0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff),
        np.array([0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd], dtype=np.uint32))
    np.testing.assert_array_equal(
        oracle.philox(0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344, 0xa4093822, 0x299f31d0),
        np.array([0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1], dtype=np.uint32))


@pytest.fixture(scope="module")
def edges():
    d = load_golden("edges")
    return d, oracle.Scene(entities_from(d))


def test_edge_case_rays(edges):
    """Edge-case rays on the Cornell box (axis-aligned with signed zeros, aimed at vertices and edge
    midpoints, in a triangle's plane, tiny / huge direction components, origins 1e6 away, t ranges
    closed at the hit distance or empty): closest hits bit for bit outside exact ties on shared
    edges and vertices, where both sides report the same distance; any-hit flags identical."""
    d, s = edges
    rays = d["rays"]
    prim, t, u, v = s.trace_closest(rays)
    ref_p, ref_t = d["closest_prim"], d["closest_t"]
    mism = prim != ref_p
    assert mism.mean() < 0.05
    assert excused_id_mismatch(s.tris(), rays, prim, t, ref_p, ref_t)[mism].all()
    assert ((prim >= 0) == (ref_p >= 0)).all()
    both = prim >= 0
    np.testing.assert_allclose(t[both & mism], ref_t[both & mism], rtol=1e-12)
    same = ~mism & both
    np.testing.assert_array_equal(t[same], ref_t[same])
    np.testing.assert_array_equal(u[same], d["closest_u"][same])
    np.testing.assert_array_equal(v[same], d["closest_v"][same])
    assert (s.trace_any(rays) == d["any_occluded"]).all()
    # the fixture exercises what it claims: hits and misses, closed and empty t ranges
    assert 0.5 < both.mean() < 0.95
    closed = (rays[:, 7] == ref_t) & (rays[:, 6] <= rays[:, 7])
    assert closed.sum() >= 50 and (ref_p[closed] >= 0).all()
    assert (ref_p[rays[:, 6] > rays[:, 7]] < 0).all()


@pytest.mark.parametrize("name", ["zcam", "wcam"])
def test_non_square_camera_passes(edges, name):
    """Intersection / instance / normal passes through non-square cameras (W != H, non-square
    pixels; one with the z_positive boresight) equal the reference's BodyFixedGroup passes."""
    d, s = edges
    cam = camera_from(d, name)
    xyz, ids, nrm, _ = s.passes(cam)
    W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
    assert ids.shape == (H, W) and W != H
    np.testing.assert_array_equal(ids, d[name + "_ids"])
    np.testing.assert_allclose(xyz, d[name + "_xyz"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(nrm, d[name + "_normals"], rtol=0, atol=1e-12)
    assert 0.2 < (ids > 0).mean() < 1.0


def test_smooth_point_light_render_deterministic(edges):
    """1 spp at integer pixel coordinates, 1 bounce, point light on a smooth-shaded, rotated,
    scaled and translated asteroid beside a flat box, through a non-square camera: no random
    draws, so the oracle's radiance equals the reference's (interpolated shading normals and the
    unclamped Lambert term, negative where the shading normal turns from the light)."""
    d, _ = edges
    s = oracle.Scene(entities_from(d, "s"))
    cam = camera_from(d, "scam")
    rad, _, taken = s.render(cam, lights_from(d["s_lights"]), 1, 1, 0.0, 1)
    ref = d["s_radiance"]
    np.testing.assert_allclose(rad[..., :3], ref, rtol=1e-6, atol=1e-7)
    assert (taken == 1).all() and (ref > 0).any(-1).sum() > 300 and (ref < 0).any()


def test_z_positive_lidar_batch(edges):
    """Batch LiDAR with the z_positive boresight (64 poses inside and around the Cornell box) equals
    the reference's batch_simulate_lidar; the -z boresight would give other ranges."""
    d, s = edges
    pos, rot = d["zlidar_pos"], d["zlidar_rot"].reshape(-1, 9)
    rng, prim = s.lidar_batch(pos, rot, z_positive=True)
    np.testing.assert_array_equal(rng, d["zlidar_range"])
    assert ((rng == 0) == (prim < 0)).all() and (rng > 0).mean() > 0.8
    assert (s.lidar_batch(pos, rot, z_positive=False)[0] != rng).mean() > 0.5
