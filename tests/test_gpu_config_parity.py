"""GPU against the FP64 oracle at the benchmarked configurations, through the C ABI.

* Procedural asteroid of 2M triangles (the bench's step): intersection / instance / normal passes
  through the 2048^2 camera, the 1 spp sun render (primary + shadow ray) and the 1024^2 LiDAR grid
  (range + triangle id).
* Cornell box as configured (256^2, 16 spp, 3 bounces, area light, seed 0) and its three passes.
* Spacecraft (~49k triangles) radiation pressure at grid 4096, 2 specular bounces.

Rules (FP32 device path vs FP64 oracle, the benchmark spec's tolerances):
  * IDs bit-exact; the only rays allowed to differ pass within 1e-6 x (|origin| + scene extent) of
    an edge of a triangle that one side hit (helpers.unexcused); zero unexcused rays are allowed;
  * hit points, normals, LiDAR ranges within 1e-5 relative;
  * deterministic radiance (1 spp at pixel centres, 1 bounce, point light): equal within FP32
    rounding except pixels whose primary or shadow ray is excused by the edge rule, or whose shadow
    ray re-enters its own surface within the shade stage's decision margin of that triangle's edge;
  * Monte-Carlo radiance with the same random streams: per pixel within 4 sigma (sigma from the
    oracle's per-pixel sample variance), at most 1e-3 of the pixel values beyond that, image mean
    within 0.5 %;
  * force, torque and total absorbed power within 1e-4 relative; each facet's absorbed power within
    1e-4 of itself plus the power of two rays (flux x cell area): a ray through an edge shared by two
    facets may land on either (the edge rule), moving its power and its specular continuation's.
"""
import os

import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes, workloads
from helpers import TriIndex, check_direct_render, check_hits, check_mc_radiance, check_passes, to_f32_rays

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def rays32(rays64):
    r = np.empty(rays64.shape[0], lib.RAY_DTYPE)
    r["o"] = rays64[:, 0:3]
    r["d"] = rays64[:, 3:6]
    r["tmin"] = rays64[:, 6]
    r["tmax"] = np.minimum(rays64[:, 7], np.finfo(np.float32).max)
    return r


def gpu_prim(hits):
    return np.where(hits["prim"] == lib.CRT_MISS, -1, hits["prim"].astype(np.int64))


@pytest.fixture(scope="module")
def ast2m():
    ents = workloads.asteroid_entities(2_000_000)
    ctx = lib.Context(0)
    sc = ctx.scene(ents)
    o = oracle.Scene(ents, nthreads=NTHREADS)
    index = TriIndex(o.tris())
    yield ctx, sc, o, index, workloads.asteroid_config(2048, 1024)
    ctx.close()


def test_asteroid_passes_2048_vs_oracle(ast2m):
    ctx, sc, o, index, cfg = ast2m
    cam = cfg["camera"]
    rays = workloads.camera_rays(cam)
    gpu = sc.passes(cam)
    ref = o.passes(cam)
    gprim = gpu_prim(sc.trace_closest(rays32(to_f32_rays(rays))))
    st = check_passes(index, rays, gpu, ref, gprim=gprim, what="asteroid 2048^2 passes")
    print("asteroid passes", st)
    assert st["hit"] > 0.9 * st["pixels"]


def test_asteroid_lidar_grid_1024_vs_oracle(ast2m):
    ctx, sc, o, index, cfg = ast2m
    lid = cfg["lidar"]
    g_rng, g_prim = sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"],
                                  lid["half_y"])
    rays = workloads.lidar_grid_rays(lid)
    o_prim, o_t, o_u, o_v = o.trace_closest(rays)
    tris = index.tris
    hit = o_prim >= 0
    pr = np.where(hit, o_prim, 0)
    x = tris[pr, 0:3] - o_u[:, None] * tris[pr, 3:6] + o_v[:, None] * tris[pr, 6:9]   # u p1 + v p2 + w p0
    o_rng = np.where(hit, np.linalg.norm(x - rays[:, 0:3], axis=1), 0.0)
    gp = np.where(g_prim.ravel() == lib.CRT_MISS, -1, g_prim.ravel().astype(np.int64))
    g_r = g_rng.ravel()
    assert ((g_r == 0) == (gp < 0)).all()
    n = check_hits(index, rays, gp, g_r, o_prim, o_rng, what="LiDAR 1024^2 beams")
    print("lidar beams", len(rays), "hit", int(hit.sum()), "excused id mismatches", n)
    assert hit.mean() > 0.9


def tracers(sc, o):
    """Closest-hit functions of [k, 8] FP64 rays -> (prim, t) for the oracle and the GPU."""
    def trace_o(r):
        p, t, _, _ = o.trace_closest(r)
        return p, t

    def trace_g(r):
        h = sc.trace_closest(rays32(to_f32_rays(r)))
        return gpu_prim(h), h["t"].astype(np.float64)
    return trace_o, trace_g


def test_asteroid_sun_render_2048_vs_oracle(ast2m):
    """1 spp at pixel centres, 1 bounce, the sun as a distant point light: no random draws."""
    ctx, sc, o, index, cfg = ast2m
    cam, lights = cfg["camera"], cfg["lights"]
    _, rad = sc.render(cam, lights, 1, 1, 1.0, cfg["bounces"])
    orad, _, _ = o.render(cam, lights, 1, 1, 1.0, cfg["bounces"])
    assert (rad[..., 3] == 1).all()
    rays = workloads.camera_rays(cam)
    ox, _, _, oprim = o.passes(cam)
    gx = sc.passes(cam)[0]
    gprim = gpu_prim(sc.trace_closest(rays32(to_f32_rays(rays))))
    st = check_direct_render(index, rays, rad, orad, ox, oprim, gx, gprim, lights, *tracers(sc, o),
                             what="asteroid 2048^2 sun render")
    print("sun render", st)
    g, r = rad[..., :3].astype(np.float64), orad[..., :3].astype(np.float64)
    assert abs(g.mean() / r.mean() - 1) < 5e-3
    assert (r[..., 0] > 0).mean() > 0.5


@pytest.fixture(scope="module")
def cornell():
    ents, cam, lights = scenes.cornell()
    ctx = lib.Context(0)
    sc = ctx.scene(ents)
    o = oracle.Scene(ents, nthreads=NTHREADS)
    yield ctx, sc, o, TriIndex(o.tris()), cam, lights
    ctx.close()


def test_cornell_config_passes_vs_oracle(cornell):
    ctx, sc, o, index, cam, lights = cornell
    assert cam["resolution"] == [256, 256]
    rays = workloads.camera_rays(cam)
    gprim = gpu_prim(sc.trace_closest(rays32(to_f32_rays(rays))))
    st = check_passes(index, rays, sc.passes(cam), o.passes(cam), gprim=gprim, what="Cornell 256^2 passes")
    print("cornell passes", st)


def test_cornell_config_render_vs_oracle(cornell):
    """Config 0 as stated: 256^2, 16 spp, 3 bounces, area light, seed 0, against the oracle's
    identical Philox streams."""
    ctx, sc, o, index, cam, lights = cornell
    _, rad = sc.render(cam, lights, 16, 16, 0.0, 3, seed=0)
    orad, _, taken, m2 = o.render(cam, lights, 16, 16, 0.0, 3, seed=0, with_m2=True)
    assert (taken == 16).all()
    st = check_mc_radiance(rad, orad, m2, 16, what="Cornell 256^2 16 spp")
    print("cornell render", st)


def srp_params(stats, sun_body, grid, nb, cm):
    b = np.array(stats["bounds"], dtype=np.float64)
    lo, hi = b[:3], b[3:]
    p = oracle.SrpParams()
    p.sun_dir[:] = list(sun_body)
    p.flux, p.c = 1361.0, 299792458.0
    p.center[:] = list(0.5 * (lo + hi))
    p.half_extent = 0.5 * float(np.sqrt(((hi - lo) ** 2).sum()))
    p.center_of_mass[:] = list(cm)
    p.grid, p.num_bounces = grid, nb
    return p


def sun_rays(stats, sun_body, grid, rows):
    """FP64 primary sun rays of grid rows `rows` (the construction of srp_attitude / the oracle)."""
    b = np.array(stats["bounds"], dtype=np.float64)
    lo, hi = b[:3], b[3:]
    ctr = 0.5 * (lo + hi)
    Rb = 0.5 * float(np.sqrt(((hi - lo) ** 2).sum()))
    h = 2.0 * Rb / grid
    sb = np.asarray(sun_body, dtype=np.float64)
    ax = np.array([0.0, 1.0, 0.0]) if abs(sb[0]) >= 0.9 else np.array([1.0, 0.0, 0.0])
    e1 = np.cross(sb, ax)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(sb, e1)
    org = ctr + sb * (2.0 * Rb + 1.0) + e1 * (-Rb + 0.5 * h) + e2 * (-Rb + 0.5 * h)
    px = np.arange(grid, dtype=np.float64)
    py = np.asarray(rows, dtype=np.float64)
    o = org[None, None, :] + px[None, :, None] * h * e1 + py[:, None, None] * h * e2
    rays = np.zeros((len(rows) * grid, 8))
    rays[:, 0:3] = o.reshape(-1, 3)
    rays[:, 3:6] = -sb
    rays[:, 7] = np.finfo(np.float64).max
    return rays


def test_spacecraft_srp_grid4096_vs_oracle():
    """Config 3's spacecraft and grid: 3 attitudes x 4096^2 sun rays x 2 specular bounces."""
    ents = scenes.spacecraft()
    ctx = lib.Context(0)
    try:
        sc = ctx.scene(ents)
        o = oracle.Scene(ents, nthreads=NTHREADS)
        index = TriIndex(o.tris())
        stats = sc.stats()
        assert stats["n_tris"] > 40_000
        q = scenes.random_quaternions(3, seed=77)
        s_i = np.array([1.0, 0.0, 0.0])
        cm = (0.1, -0.2, 0.05)
        G = 4096
        f, t, fp = sc.srp(s_i, q, grid=G, num_bounces=2, center_of_mass=cm, facet_power=True)
        for a in range(len(q)):
            sb = scenes.quaternion_to_matrix(q[a]).T @ s_i
            of, ot, ofp = o.srp(srp_params(stats, sb, G, 2, cm))
            ef = np.linalg.norm(f[a] - of) / np.linalg.norm(of)
            et = np.linalg.norm(t[a] - ot) / max(np.linalg.norm(ot), 1e-3 * np.linalg.norm(of))
            # per facet: a ray through an edge shared by two facets may land on either, moving at most
            # its power (flux x cell area) and that of its specular continuation between them
            e_ray = 1361.0 * (index.extent / G) ** 2
            excess = np.abs(fp[a] - ofp) - 1e-4 * ofp
            print(f"srp attitude {a}: force rel {ef:.2e} torque rel {et:.2e} facet L1 "
                  f"{np.abs(fp[a] - ofp).sum() / ofp.sum():.2e}, max facet diff / ray power "
                  f"{np.abs(fp[a] - ofp).max() / e_ray:.2f}, facets beyond 1e-4: {(excess > 0).sum()}")
            assert ef <= 1e-4 and et <= 1e-4
            assert abs(fp[a].sum() / ofp.sum() - 1) <= 1e-4
            assert (excess <= 2 * e_ray).all()
            # primary sun rays, every 8th grid row: hit triangles equal outside the edge rule
            rays = sun_rays(stats, sb, G, np.arange(0, G, 8))
            hits = sc.trace_closest(rays32(to_f32_rays(rays)))
            o_prim, o_t, _, _ = o.trace_closest(rays)
            check_hits(index, rays, gpu_prim(hits), hits["t"], o_prim, o_t, what=f"sun rays, attitude {a}")
            assert (o_prim >= 0).any()
    finally:
        ctx.close()


def test_batched_mix_requests_vs_oracle(ast2m):
    """The 64-request mix of the batched configuration (renders 128^2..2048^2 at 1..64 spp with 2
    bounces, LiDAR scans 64^2..1024^2) run as one crt_batch; every LiDAR scan and every render of at
    most 2^20 paths is compared with the oracle: scans by the edge rule on their FP64 beams, renders
    (the oracle's identical Philox streams) by the 4-sigma rule."""
    ctx, sc, o, index, cfg = ast2m
    reqs = []
    for q in workloads.batched_config(seed=1):
        if q["kind"] == "render":
            reqs.append(dict(kind="render", scene=sc, camera=q["camera"], lights=q["lights"], min_samples=q["spp"],
                             max_samples=q["spp"], noise_threshold=0.0, num_bounces=q["bounces"], seed=1,
                             request=q["request"], radiance=True))
        else:
            reqs.append(dict(kind="lidar", scene=sc, position=q["position"], rotation=q["rotation"], nx=q["nx"],
                             ny=q["ny"], half_x=q["half_x"], half_y=q["half_y"]))
    outs, st = ctx.batch(reqs)
    assert st["waves"] >= 1
    renders = scans = 0
    for q, out in zip(reqs, outs):
        if q["kind"] == "lidar":
            lid = dict(position=q["position"], rotation=q["rotation"], nx=q["nx"], ny=q["ny"], half_x=q["half_x"],
                       half_y=q["half_y"])
            rays = workloads.lidar_grid_rays(lid)
            o_prim, o_t, o_u, o_v = o.trace_closest(rays)
            tris = index.tris
            pr = np.where(o_prim >= 0, o_prim, 0)
            x = tris[pr, 0:3] - o_u[:, None] * tris[pr, 3:6] + o_v[:, None] * tris[pr, 6:9]
            o_rng = np.where(o_prim >= 0, np.linalg.norm(x - rays[:, 0:3], axis=1), 0.0)
            g_rng, g_prim = out[0].ravel(), out[1].ravel()
            gp = np.where(g_prim == lib.CRT_MISS, -1, g_prim.astype(np.int64))
            check_hits(index, rays, gp, g_rng, o_prim, o_rng, what=f"batched LiDAR {q['nx']}^2")
            scans += 1
        else:
            W, H = q["camera"]["resolution"]
            if W * H * q["max_samples"] > (1 << 20):
                continue
            orad, _, taken, m2 = o.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], 0.0,
                                          q["num_bounces"], seed=1, request=q["request"], with_m2=True)
            st = check_mc_radiance(out[1], orad, m2, taken, what=f"batched render {W}^2 x {q['max_samples']} spp")
            print(f"batched render {W}^2 x {q['max_samples']} spp", st)
            renders += 1
    assert scans == 32 and renders >= 10
