"""Watertightness of the FP32 triangle test on closed meshes, through the C ABI.

A ray that enters a closed mesh must meet its surface.  The reference tests triangles in FP64
(triangle.hpp:140-160), where rays slip between two triangles only through cracks some 1e-16 of the
coordinates wide; an FP32 restatement of the same formula, evaluated from each triangle's own p0,
leaves cracks about one ulp of the ray's coordinates wide along every shared edge, through which a
camera or LiDAR ray reaches the far side of the body and a shadow ray escapes it.  These tests aim
rays exactly at shared edges and vertices of closed meshes (the worst case: every ray crosses the
surface within rounding of an edge) and require every one of them to stop at the surface:
  * rays from outside toward an edge point or a vertex: a closest hit no farther than that point
    (plus the FP32 rounding of t and of the ray, 1e-6 x (|origin| + extent));
  * rays from inside the body toward the same points: an any-hit within that distance, and a closest
    hit no farther.
"""
import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes, workloads
from helpers import scene_extent, tri_vertices

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


def targets(tris12, n, rng):
    """n points on shared edges (midpoints and random fractions of edge p0-p1, p1-p2, p2-p0) and
    vertices of randomly chosen triangles, and those triangles' unit normals."""
    p0, p1, p2 = tri_vertices(tris12)
    k = rng.integers(0, len(tris12), n)
    nrm = tris12[k, 9:12] / np.linalg.norm(tris12[k, 9:12], axis=1)[:, None]
    which = rng.integers(0, 3, n)
    a = np.choose(which[:, None], [p0[k], p1[k], p2[k]])
    b = np.choose(which[:, None], [p1[k], p2[k], p0[k]])
    f = np.where(rng.random(n) < 0.25, 0.5, rng.random(n))
    f = np.where(rng.random(n) < 0.2, 0.0, f)   # a fifth on vertices
    return a + f[:, None] * (b - a), nrm


def unit_vectors(n, rng):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1)[:, None]


def rays_to(origins, pts, extra=0.0):
    """FP32 rays (RAY_DTYPE) from origins toward pts, tmax = distance + extra, and the distances."""
    d = pts - origins
    dist = np.linalg.norm(d, axis=1)
    r = np.empty(len(pts), lib.RAY_DTYPE)
    r["o"] = origins
    r["d"] = d / dist[:, None]
    r["tmin"] = 0.0
    r["tmax"] = dist + extra
    return r, dist


# the 200k-triangle asteroid about the origin, the same asteroid 3.9 km off it (coordinates of a few
# thousand: larger rounding), and a unit icosphere of 20480 triangles
@pytest.mark.parametrize("mesh,n_rays", [("asteroid", 400_000), ("asteroid_offset", 200_000), ("sphere", 200_000)])
def test_rays_at_edges_and_vertices_stop_at_the_surface(ctx, mesh, n_rays):
    centre = np.zeros(3)
    if mesh.startswith("asteroid"):
        ents = workloads.asteroid_entities(200_000, seed=3)
        radius = 1000.0
        if mesh == "asteroid_offset":
            centre = np.array([3000.0, -2000.0, 1500.0])
            ents[0].position = centre
    else:
        ents = [scenes.EntitySpec("sphere", scenes.asteroid(level=5, radius=1.0, amplitude=0.0), (0.7, 0.7, 0.7))]
        radius = 1.0
    o = oracle.Scene(ents)
    tris = o.tris()
    ext = scene_extent(tris)
    sc = ctx.scene(ents)
    rng = np.random.default_rng(11)
    pts, nrm = targets(tris, n_rays, rng)
    # from outside: origins 5 radii away within 27 degrees of the outward normal (no grazing rays: an
    # FP32 ray passes its FP64 target within about 1e-7 of its length, which at grazing incidence
    # could miss the body or meet it behind the target without any crack)
    out = nrm * np.sign(((pts - centre) * nrm).sum(1))[:, None]
    w = unit_vectors(n_rays, rng)
    u = out + 0.5 * w * np.sign((w * out).sum(1))[:, None]   # w in the outward hemisphere: <= atan(1/2)
    u /= np.linalg.norm(u, axis=1)[:, None]
    org = pts + 5.0 * radius * u
    r, dist = rays_to(org, pts)
    r["tmax"] = np.finfo(np.float32).max
    h = sc.trace_closest(r)
    tol = 1e-6 * (np.linalg.norm(org, axis=1) + ext)
    miss = h["prim"] == lib.CRT_MISS
    far = ~miss & (h["t"] > dist + tol)
    assert miss.sum() == 0 and far.sum() == 0, (f"{mesh}: {int(miss.sum())} rays missed and {int(far.sum())} "
                                                f"passed the surface of {n_rays} aimed at edges and vertices")
    # from inside (near the centre): the ray leaves the body through the surface
    org_in = centre + 0.05 * radius * unit_vectors(n_rays, rng)
    r, dist = rays_to(org_in, pts)
    tol = 1e-6 * (np.linalg.norm(org_in, axis=1) + ext)
    r["tmax"] = dist + tol
    occ = sc.trace_any(r)
    assert occ.all(), f"{mesh}: {int((occ == 0).sum())} of {n_rays} rays left the body unoccluded"
    r["tmax"] = np.finfo(np.float32).max
    h = sc.trace_closest(r)
    bad = (h["prim"] == lib.CRT_MISS) | (h["t"] > dist + tol)
    assert not bad.any(), f"{mesh}: {int(bad.sum())} of {n_rays} rays from inside passed the surface"
