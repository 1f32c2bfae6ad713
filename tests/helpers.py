"""Shared helpers for the test suite: fixture loading, scene specs, parity metrics."""
import os
import sys

import numpy as np

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
PKG = os.path.join(REPO, "ceres-raytracer_gb300")
for p in (PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

from crt_gb300 import scenes  # noqa: E402

GOLDEN = os.path.join(TESTS, "golden")

# Parity tolerances (the ray-query path computes in FP32, the reference in FP64):
#  * IDs bit-exact except rays whose hit lies within EDGE_REL * (|ray origin| + scene extent)
#    of an edge of the triangle hit on either side (1e-6 relative to the coordinate scale);
#  * distances, points, normals: 1e-5 relative.
EDGE_REL = 1e-6
DIST_REL = 1e-5


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def entities_from(d, prefix="e"):
    ents = []
    for i in range(int(d[f"{prefix}_count"])):
        ents.append(scenes.EntitySpec(
            name=f"{prefix}{i}", mesh=scenes.Mesh(d[f"{prefix}{i}_v"], d[f"{prefix}{i}_f"]),
            color=tuple(float(x) for x in d[f"{prefix}{i}_color"]), smooth=bool(d[f"{prefix}{i}_smooth"]),
            scale=float(d[f"{prefix}{i}_scale"]), position=np.array(d[f"{prefix}{i}_pos"]),
            rotation=np.array(d[f"{prefix}{i}_rot"])))
    return ents


def camera_from(d, prefix="cam"):
    return dict(focal_length=float(d[prefix + "_focal"]), resolution=[float(x) for x in d[prefix + "_res"]],
                sensor_size=[float(x) for x in d[prefix + "_sensor"]], z_positive=bool(d[prefix + "_zpos"]),
                position=np.array(d[prefix + "_pos"]), rotation=np.array(d[prefix + "_rot"]))


def lights_from(arr):
    out = []
    for l in np.atleast_2d(arr):
        out.append(dict(type="area" if l[0] == 1 else "point", intensity=float(l[1]), position=np.array(l[2:5]),
                        rotation=np.array(l[5:14]).reshape(3, 3), size=[float(l[14]), float(l[15])]))
    return out


def tri_vertices(tris12):
    """(p0, p1, p2) from FP64 p0, e1, e2, n rows (p1 = p0 - e1, p2 = p0 + e2, triangle.hpp:81-82)."""
    p0 = tris12[:, 0:3]
    return p0, p0 - tris12[:, 3:6], p0 + tris12[:, 6:9]


def point_segment_distance(p, a, b):
    ab = b - a
    t = np.clip(((p - a) * ab).sum(-1) / np.maximum((ab * ab).sum(-1), 1e-300), 0.0, 1.0)
    q = a + t[..., None] * ab
    return np.sqrt(((p - q) ** 2).sum(-1))


def edge_distance(tris12, prim, points):
    """World distance from each point to the nearest edge of triangle prim (prim >= 0)."""
    p0, p1, p2 = tri_vertices(tris12[prim])
    return np.minimum(np.minimum(point_segment_distance(points, p0, p1), point_segment_distance(points, p1, p2)),
                      point_segment_distance(points, p2, p0))


def intersect_fp64(tris12, prim, rays):
    """Reference triangle test (triangle.hpp:140-160) of each ray against triangle prim: (hit, t, u, v)."""
    p0, e1, e2, n = tris12[prim, 0:3], tris12[prim, 3:6], tris12[prim, 6:9], tris12[prim, 9:12]
    o, d = rays[:, 0:3], rays[:, 3:6]
    c = p0 - o
    r = np.cross(d, c)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / (n * d).sum(-1)
        u = (r * e2).sum(-1) * inv
        v = (r * e1).sum(-1) * inv
        t = (n * c).sum(-1) * inv
    w = 1.0 - u - v
    return (u >= 0) & (v >= 0) & (w >= 0), t, u, v


def scene_extent(tris12):
    p0, p1, p2 = tri_vertices(tris12)
    lo = np.minimum(np.minimum(p0, p1), p2).min(0)
    hi = np.maximum(np.maximum(p0, p1), p2).max(0)
    return float(np.sqrt(((hi - lo) ** 2).sum()))


def excused_id_mismatch(tris12, rays, prim_a, t_a, prim_b, t_b):
    """Boolean mask of ID mismatches that the parity rule excuses: the hit point of either side lies
    within EDGE_REL*(|origin| + extent) of an edge of its own triangle, or both sides hit at the same
    distance (coplanar ties), or one side misses while the other grazes an edge."""
    ext = scene_extent(tris12)
    o = rays[:, 0:3]
    eps = EDGE_REL * (np.sqrt((o * o).sum(-1)) + ext)
    d = rays[:, 3:6]
    ok = np.zeros(len(prim_a), dtype=bool)
    for prim, t in ((prim_a, t_a), (prim_b, t_b)):
        has = prim >= 0
        idx = np.nonzero(has)[0]
        if len(idx):
            pts = o[idx] + t[idx, None] * d[idx]
            ok[idx] |= edge_distance(tris12, prim[idx], pts) <= eps[idx] + DIST_REL * np.abs(t[idx]) * 0.0
    both = (prim_a >= 0) & (prim_b >= 0)
    ok |= both & (np.abs(t_a - t_b) <= DIST_REL * np.maximum(np.abs(t_a), 1e-30))
    return ok


def rel_err(a, b, scale=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if scale is None:
        scale = np.maximum(np.abs(b), 1e-30)
    return np.abs(a - b) / scale


def radiance_stats_ok(mean_a, m2_a, n_a, mean_b, m2_b, n_b, mask=None, zmax=4.0):
    """Per-pixel z-scores of the difference of two Monte-Carlo means with Welford M2 sums."""
    va = m2_a / max(n_a - 1, 1) / n_a
    vb = m2_b / max(n_b - 1, 1) / n_b
    se = np.sqrt(np.maximum(va, 0) + np.maximum(vb, 0)) + 1e-7
    z = np.abs(mean_a - mean_b) / se
    if mask is not None:
        z = z[mask]
    return z
