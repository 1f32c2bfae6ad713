"""GPU wavefront path tracer vs the reference fixtures and the FP64 oracle, through the C ABI.

* Deterministic renders (1 spp at pixel centres, 1 bounce, point lights: no random draws): radiance
  equals the oracle's (which reproduces the reference's, tests/test_oracle_golden.py) within FP32
  rounding on every pixel except those whose primary or shadow ray passes within the edge distance
  of a triangle edge, or whose shadow ray re-enters its own surface within the shade stage's
  decision margin of that triangle's edge (helpers.check_direct_render).
* Same seed as the oracle: both draw the same Philox streams; per pixel within 4 sigma of the
  Monte-Carlo error (sigma from the oracle's per-pixel sample variance), at most 1e-3 of the pixel
  values beyond, image mean within 0.5 % (helpers.check_mc_radiance).
* Area light, 512 spp, 3 bounces vs the reference's own path tracer (different random streams):
  per pixel within 4 sigma with at most 1e-3 of the values beyond, image mean within 0.5 % (pixels
  next to the light plane excluded, see test_oracle_golden.test_area_light_render_statistics).
"""
import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes, workloads
from helpers import (TriIndex, camera_from, check_direct_render, check_mc_radiance, entities_from, lights_from,
                     load_golden, radiance_stats_ok, to_f32_rays)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def cornell(ctx):
    d = load_golden("cornell")
    ents = entities_from(d)
    return d, ents, ctx.scene(ents), oracle.Scene(ents)


def direct_parity(sc, o, cam, lights, rad, orad, what):
    """check_direct_render for a 1-spp, 1-bounce point-light render of scene sc (GPU) / o (oracle)."""
    index = TriIndex(o.tris())
    rays = workloads.camera_rays(cam)
    ox, _, _, oprim = o.passes(cam)
    gx = sc.passes(cam)[0]
    h = sc.trace_closest(rays32(to_f32_rays(rays)))
    gprim = np.where(h["prim"] == lib.CRT_MISS, -1, h["prim"].astype(np.int64))

    def trace_o(r):
        p, t, _, _ = o.trace_closest(r)
        return p, t

    def trace_g(r):
        hh = sc.trace_closest(rays32(to_f32_rays(r)))
        return np.where(hh["prim"] == lib.CRT_MISS, -1, hh["prim"].astype(np.int64)), hh["t"].astype(np.float64)
    return check_direct_render(index, rays, rad, orad, ox, oprim, gx, gprim, lights, trace_o, trace_g, what=what)


def rays32(rays64):
    r = np.empty(rays64.shape[0], lib.RAY_DTYPE)
    r["o"] = rays64[:, 0:3]
    r["d"] = rays64[:, 3:6]
    r["tmin"] = rays64[:, 6]
    r["tmax"] = np.minimum(rays64[:, 7], np.finfo(np.float32).max)
    return r


def test_point_light_deterministic(cornell):
    d, ents, sc, o = cornell
    cam = camera_from(d, "rcam")
    lights = lights_from(d["point_lights"])
    rgba, rad = sc.render(cam, lights, 1, 1, 0.0, 1)
    ref = d["point_radiance"]
    orad, _, _ = o.render(cam, lights, 1, 1, 0.0, 1)
    np.testing.assert_allclose(orad[..., :3], ref, rtol=1e-6, atol=1e-6)
    direct_parity(sc, o, cam, lights, rad, orad, "Cornell point-light render")
    assert abs(rad[..., :3].mean() / ref.mean() - 1) < 5e-3
    assert (rad[..., 3] == 1).all()
    # quantisation: clamp(v * 256, 0, 255) truncated to uint8 (do_render.hpp:118-134)
    np.testing.assert_array_equal(rgba, np.clip(rad * 256, 0, 255).astype(np.uint8))


def test_same_seed_matches_oracle(cornell):
    d, ents, sc, o = cornell
    cam = dict(camera_from(d, "rcam"), resolution=[32, 32])
    lights = lights_from(d["lights"])
    _, rad = sc.render(cam, lights, 8, 8, 0.0, 3, seed=5)
    orad, _, _, m2 = o.render(cam, lights, 8, 8, 0.0, 3, seed=5, with_m2=True)
    check_mc_radiance(rad, orad, m2, 8, what="same seed, 8 spp")


def test_area_light_statistics_vs_reference(cornell):
    d, ents, sc, o = cornell
    cam = camera_from(d, "rcam")
    spp, bounces = int(d["render_spp"]), int(d["render_bounces"])
    _, rad = sc.render(cam, lights_from(d["lights"]), spp, spp, 0.0, bounces, seed=1)
    xyz, ids, _, _ = o.passes(cam)
    mask = ~((ids == 1) & (xyz[..., 1] > 0.94)) & (ids != 6) & (ids > 0)
    ref, m2 = d["render_mean"], d["render_m2"]
    z = radiance_stats_ok(rad[..., :3], m2, spp, ref, m2, spp, mask=np.repeat(mask[..., None], 3, -1))
    assert (z > 4).mean() <= 1e-3, (z > 4).mean()
    ours, theirs = rad[..., :3][mask].mean(), ref[mask].mean()
    assert abs(ours / theirs - 1) < 0.005, (ours, theirs)


def test_adaptive_sampling_matches_oracle(cornell):
    d, ents, sc, o = cornell
    cam = dict(camera_from(d, "rcam"), resolution=[24, 24])
    lights = lights_from(d["lights"])
    _, rad = sc.render(cam, lights, 2, 32, 2.0, 2, seed=9)
    orad, _, taken, m2 = o.render(cam, lights, 2, 32, 2.0, 2, seed=9, with_m2=True)
    assert taken.min() >= 2 and taken.max() <= 32 and (taken < 32).any()
    check_mc_radiance(rad, orad, m2, taken, what="adaptive sampling")


@pytest.mark.parametrize("res,spp,thr", [((37, 23), (4, 4), 0.0), ((29, 19), (2, 16), 2.0), ((5, 3), (3, 3), 0.0)])
def test_odd_resolutions_match_oracle(cornell, res, spp, thr):
    """Camera paths are traced in 8 x 4 pixel tiles: images whose sides are not multiples of 8 and 4
    (partial tiles, a short last band) still sample every pixel once per sample, as the oracle."""
    d, ents, sc, o = cornell
    cam = dict(camera_from(d, "rcam"), resolution=list(res))
    lights = lights_from(d["lights"])
    _, rad = sc.render(cam, lights, spp[0], spp[1], thr, 2, seed=7)
    orad, _, taken, m2 = o.render(cam, lights, spp[0], spp[1], thr, 2, seed=7, with_m2=True)
    assert rad.shape == (res[1], res[0], 4) and (rad[..., 3] == 1).all()
    check_mc_radiance(rad, orad, m2, taken, what=f"{res[0]}x{res[1]}")


def test_multiple_lights_and_no_bounce(cornell):
    d, ents, sc, o = cornell
    cam = dict(camera_from(d, "rcam"), resolution=[16, 16])
    lights = lights_from(d["lights"]) + lights_from(d["point_lights"])
    _, rad = sc.render(cam, lights, 4, 4, 0.0, 2, seed=3)
    orad, _, _, m2 = o.render(cam, lights, 4, 4, 0.0, 2, seed=3, with_m2=True)
    check_mc_radiance(rad, orad, m2, 4, what="area + point lights")
    rgba, rad0 = sc.render(cam, lights, 1, 1, 0.0, 0)   # no bounce: black, alpha 1
    assert (rad0[..., :3] == 0).all() and (rgba[..., 3] == 255).all()


def test_asteroid_sun_render_vs_oracle(ctx):
    """Config-2 style render (1 spp, 1 bounce, sun as a distant point light) on a 100k asteroid."""
    ents = [scenes.EntitySpec("a", scenes.asteroid(100_000, seed=3), (0.1, 0.1, 0.1))]
    sc = ctx.scene(ents)
    o = oracle.Scene(ents)
    view = scenes.unit_vector(12)
    sun = np.cross(view, scenes.unit_vector(11))          # sun at 90 deg: the terminator crosses the view
    sun /= np.linalg.norm(sun)
    lights = [dict(type="point", intensity=1.0e18, position=1.0e9 * sun)]
    cam = scenes.fov_camera(scenes.TAN5 * 2.4, (128, 128), 5000.0 * view, (0.0, 0.0, 0.0))
    _, rad = sc.render(cam, lights, 1, 1, 1.0, 1)
    orad, _, _ = o.render(cam, lights, 1, 1, 1.0, 1)
    st = direct_parity(sc, o, cam, lights, rad, orad, "100k asteroid sun render")
    print("asteroid sun render", st)
    lit = orad[..., 0] > 0
    assert 0.2 < lit.mean() < 0.9


def test_open_quad_self_occlusion_matches_oracle(ctx):
    """A shadow ray that points into the surface it leaves stops on its own triangle in the reference
    (its origin is 1e-4 off the surface along -n, unidirectional.hpp:55-57), so on an open quad only
    a light on the offset side contributes; a light on the other side adds nothing, not its negative
    Lambert term.  Such rays are resolved in the shade stage and never traced."""
    quad = scenes.quad_mesh((-1.0, 0.0, -0.7), (0.9, 0.0, -1.0), (1.1, 0.0, 0.8), (-0.8, 0.0, 1.0))
    ents = [scenes.EntitySpec("q", quad, (0.7, 0.5, 0.3))]
    sc, o = ctx.scene(ents), oracle.Scene(ents)
    cam = scenes.fov_camera(0.5, (48, 40), (0.05, 3.0, 0.03), (0.0, 0.0, 0.0))
    blocked = dict(type="point", intensity=3.0, position=[0.3, 2.0, 0.2])    # camera side: behind n's offset
    lit = dict(type="point", intensity=2.0, position=[-0.2, -2.0, 0.1])
    _, rad = sc.render(cam, [blocked], 1, 1, 0.0, 1)
    orad, _, _ = o.render(cam, [blocked], 1, 1, 0.0, 1)
    assert (orad[..., :3] == 0).all()
    direct_parity(sc, o, cam, [blocked], rad, orad, "open quad, light behind the offset side")
    _, rad2 = sc.render(cam, [blocked, lit], 1, 1, 0.0, 1)
    orad2, _, _ = o.render(cam, [blocked, lit], 1, 1, 0.0, 1)
    assert (orad2[..., 0] > 0).mean() > 0.3
    direct_parity(sc, o, cam, [blocked, lit], rad2, orad2, "open quad, two lights")
    # counting build: the blocked light's shadow rays are not traced (at most an edge band is)
    ctx.set_counting(True)
    try:
        ctx.reset_counters()
        sc.render(cam, [blocked], 1, 1, 0.0, 1)
        rays = ctx.counters()["rays"]
    finally:
        ctx.set_counting(False)
    hits = int((orad2[..., 0] > 0).sum())
    assert 48 * 40 <= rays < 48 * 40 + 0.05 * hits, (rays, hits)


def test_terminator_shadow_rays_resolved_in_shade(ctx):
    """Asteroid with the terminator across the view: shadow rays from the night side stop on their
    own triangle (closed mesh: the traced result would be 'occluded' too), so fewer shadow rays are
    traced than primary rays hit, and the image equals the oracle's as before."""
    ents = [scenes.EntitySpec("a", scenes.asteroid(100_000, seed=3), (0.1, 0.1, 0.1))]
    sc = ctx.scene(ents)
    view = scenes.unit_vector(12)
    sun = np.cross(view, scenes.unit_vector(11))
    sun /= np.linalg.norm(sun)
    lights = [dict(type="point", intensity=1.0e18, position=1.0e9 * sun)]
    cam = scenes.fov_camera(scenes.TAN5 * 2.4, (128, 128), 5000.0 * view, (0.0, 0.0, 0.0))
    ctx.set_counting(True)
    try:
        ctx.reset_counters()
        _, rad = sc.render(cam, lights, 1, 1, 1.0, 1)
        rays = ctx.counters()["rays"]
    finally:
        ctx.set_counting(False)
    xyz, ids, _ = sc.passes(cam)
    hits = int((ids > 0).sum())
    lit = int((rad[..., 0] > 0).sum())
    shadow = rays - 128 * 128
    assert lit <= shadow < hits, (lit, shadow, hits)
    assert shadow < 0.9 * hits


@pytest.mark.parametrize("bounces", [2, 3])
def test_smooth_shaded_multi_bounce_render_vs_oracle(ctx, bounces):
    """Smooth-shaded asteroid, 2 and 3 bounces, 128^2 x 32 spp, the oracle's random streams: bounce
    directions sampled about the interpolated normal can point into the flat surface they leave (the
    reference then meets its own triangle again, and so does the device ray, which tests that
    triangle in this case); per-pixel radiance within 4 sigma, image mean within 0.5 %."""
    ents = [scenes.EntitySpec("a", scenes.asteroid(100_000, seed=3), (0.3, 0.3, 0.3), smooth=True)]
    sc, o = ctx.scene(ents), oracle.Scene(ents)
    view = scenes.unit_vector(21)
    sun = view + 0.5 * scenes.unit_vector(22)   # lit from near the camera: most of the view is sunlit
    sun /= np.linalg.norm(sun)
    lights = [dict(type="point", intensity=1.0e18, position=1.0e9 * sun)]
    cam = scenes.fov_camera(scenes.TAN5 * 2.4, (128, 128), 5000.0 * view, (0.0, 0.0, 0.0))
    _, rad = sc.render(cam, lights, 32, 32, 0.0, bounces, seed=11)
    orad, _, _, m2 = o.render(cam, lights, 32, 32, 0.0, bounces, seed=11, with_m2=True)
    assert (orad[..., 0] > 0).mean() > 0.5
    check_mc_radiance(rad, orad, m2, 32, what=f"smooth-shaded {bounces}-bounce asteroid")
