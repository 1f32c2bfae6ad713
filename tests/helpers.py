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


def line_segment_distance(o, d, a, b):
    """Distance between the line o + s d and the segment [a, b] (row-wise)."""
    e = b - a
    w = a - o
    dd = (d * d).sum(-1)
    de = (d * e).sum(-1)
    ee = np.maximum((e * e).sum(-1), 1e-300)
    dw = (d * w).sum(-1)
    ew = (e * w).sum(-1)
    den = dd * ee - de * de
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(den > 1e-300 * dd * ee, (de * dw - dd * ew) / den, 0.0)
    t = np.clip(t, 0.0, 1.0)
    s = (dw + t * de) / np.maximum(dd, 1e-300)
    q = w + t[:, None] * e - s[:, None] * d
    return np.sqrt((q * q).sum(-1))


def ray_edge_distance(tris12, prim, rays):
    """Distance between each ray's line and the nearest edge of triangle prim: how close the ray
    passes to the triangle's boundary (independent of the incidence angle)."""
    p0, p1, p2 = tri_vertices(tris12[prim])
    o, d = rays[:, 0:3], rays[:, 3:6]
    return np.minimum(np.minimum(line_segment_distance(o, d, p0, p1), line_segment_distance(o, d, p1, p2)),
                      line_segment_distance(o, d, p2, p0))


def point_near_any_edge(tris12, points, eps):
    """True where a point lies within eps of an edge of any triangle (brute force over the triangles
    whose box contains the point, for the few pixels that need it).  Covers rays through a shared
    edge that one side reports as a miss (the Moeller-Trumbore test is not watertight)."""
    p0, p1, p2 = tri_vertices(tris12)
    lo = np.minimum(np.minimum(p0, p1), p2)
    hi = np.maximum(np.maximum(p0, p1), p2)
    out = np.zeros(len(points), dtype=bool)
    for k, (x, e) in enumerate(zip(points, np.broadcast_to(eps, (len(points),)))):
        cand = np.nonzero(((lo - e) <= x).all(1) & (x <= (hi + e)).all(1))[0]
        if len(cand) == 0:
            continue
        xx = np.broadcast_to(x, (len(cand), 3))
        d = np.minimum(np.minimum(point_segment_distance(xx, p0[cand], p1[cand]),
                                  point_segment_distance(xx, p1[cand], p2[cand])),
                       point_segment_distance(xx, p2[cand], p0[cand]))
        out[k] = (d <= e).any()
    return out


def excused_id_mismatch(tris12, rays, prim_a, t_a, prim_b, t_b):
    """Boolean mask of ID mismatches that the parity rule excuses: the ray passes within
    EDGE_REL * (|origin| + scene extent) of an edge of the triangle hit on either side (exact ties
    on shared edges, and FP32 rounding of rays that graze a triangle boundary), or both sides hit
    at the same distance (coplanar overlapping triangles)."""
    ext = scene_extent(tris12)
    o = rays[:, 0:3]
    eps = EDGE_REL * (np.sqrt((o * o).sum(-1)) + ext)
    ok = np.zeros(len(prim_a), dtype=bool)
    for prim in (prim_a, prim_b):
        idx = np.nonzero(prim >= 0)[0]
        if len(idx):
            ok[idx] |= ray_edge_distance(tris12, prim[idx], rays[idx]) <= eps[idx]
    both = (prim_a >= 0) & (prim_b >= 0)
    ok |= both & (np.abs(t_a - t_b) <= DIST_REL * np.maximum(np.abs(t_a), 1e-30))
    return ok


def to_f32_rays(rays64):
    """Round FP64 rays to FP32-representable values (kept as float64), so that an FP32 tracer and
    an FP64 one see bit-identical rays."""
    with np.errstate(over="ignore"):
        r = rays64.astype(np.float32).astype(np.float64)
    r[:, 7] = np.where(rays64[:, 7] > 3.0e38, np.finfo(np.float64).max, r[:, 7])
    return r


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
