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


class TriIndex:
    """Uniform-grid index of a scene's triangles (FP64 rows p0, e1, e2, n) for edge queries at points:
    each triangle sits in the cell of its box centre, cells as large as the largest box, so a box
    that reaches a point lies in the 3 x 3 x 3 cells around the point's cell."""

    def __init__(self, tris12):
        self.tris = tris12
        self.v = tri_vertices(tris12)
        p0, p1, p2 = self.v
        self.lo = np.minimum(np.minimum(p0, p1), p2)
        self.hi = np.maximum(np.maximum(p0, p1), p2)
        self.extent = scene_extent(tris12) if len(tris12) else 0.0
        self.origin = self.lo.min(0) if len(tris12) else np.zeros(3)
        self.cell = max(float((self.hi - self.lo).max()) if len(tris12) else 1.0, 1e-9)
        keys = self._key(np.floor(((self.lo + self.hi) * 0.5 - self.origin) / self.cell).astype(np.int64))
        self.order = np.argsort(keys, kind="stable")
        self.keys = keys[self.order]

    @staticmethod
    def _key(c):
        c = c + (1 << 20)
        return c[..., 0] + (c[..., 1] << 21) + (c[..., 2] << 42)

    def near(self, x, e):
        """Indices of triangles whose box, enlarged by e, contains point x."""
        c = np.floor((x - self.origin) / self.cell).astype(np.int64)
        r = 1 + int(np.ceil(e / self.cell))
        off = np.arange(-r, r + 1)
        cells = np.stack(np.meshgrid(off, off, off, indexing="ij"), -1).reshape(-1, 3) + c
        k = self._key(cells)
        lo = np.searchsorted(self.keys, k, "left")
        hi = np.searchsorted(self.keys, k, "right")
        cand = np.concatenate([self.order[a:b] for a, b in zip(lo, hi)]) if len(k) else np.zeros(0, np.int64)
        if len(cand) == 0:
            return cand
        ok = ((self.lo[cand] - e) <= x).all(1) & (x <= (self.hi[cand] + e)).all(1)
        return cand[ok]

    def ray_near_edge(self, ray, prims, e):
        """Whether the ray's line passes within e of an edge of one of the triangles `prims`."""
        if len(prims) == 0:
            return False
        p0, p1, p2 = (a[prims] for a in self.v)
        o = np.broadcast_to(ray[0:3], p0.shape)
        d = np.broadcast_to(ray[3:6], p0.shape)
        dist = np.minimum(np.minimum(line_segment_distance(o, d, p0, p1), line_segment_distance(o, d, p1, p2)),
                          line_segment_distance(o, d, p2, p0))
        return bool((dist <= e).any())


def edge_eps(rays, extent):
    """Per-ray edge distance of the ID rule: EDGE_REL * (|origin| + scene extent)."""
    return EDGE_REL * (np.linalg.norm(rays[:, 0:3], axis=1) + extent)


def unexcused(index, rays, eps, prims=(), points=()):
    """Indices of the rays that the edge rule does not excuse.  A ray is excused when its line passes
    within eps of an edge of one of its triangles prims[j][k] (>= 0), or of a triangle reaching one of
    its points points[j][k] (finite rows: a hit point reported by either side, which lies on the
    triangle that side hit)."""
    n = len(rays)
    ok = np.zeros(n, dtype=bool)
    for prim in prims:
        prim = np.asarray(prim)
        idx = np.nonzero(~ok & (prim >= 0))[0]
        if len(idx):
            ok[idx] |= ray_edge_distance(index.tris, prim[idx], rays[idx]) <= eps[idx]
    for k in np.nonzero(~ok)[0]:
        for pts in points:
            x = pts[k]
            if np.all(np.isfinite(x)) and index.ray_near_edge(rays[k], index.near(x, eps[k]), eps[k]):
                ok[k] = True
                break
    return np.nonzero(~ok)[0]


def check_passes(index, rays, gpu, ref, gprim=None, what="passes"):
    """Intersection / instance / normal passes of the GPU against the FP64 oracle (or the reference):
    every pixel agrees (same instance id, point within DIST_REL of max(|point|, hit distance), normal
    within DIST_REL) or is excused by the edge rule (unexcused): its ray passes within
    EDGE_REL * (|origin| + extent) of an edge of the triangle either side hit.  Pixels both sides
    miss are exactly zero.  Returns counts."""
    gx, gi, gn = (np.asarray(a) for a in gpu)
    ox, oi, on = (np.asarray(a) for a in ref[:3])
    oprim = np.asarray(ref[3]).ravel() if len(ref) > 3 and ref[3] is not None else None
    gx, gn, ox, on = (a.reshape(-1, 3) for a in (gx, gn, ox, on))
    gi, oi = gi.ravel().astype(np.int64), oi.ravel().astype(np.int64)
    miss = (gi == 0) & (oi == 0)
    assert (gx[miss] == 0).all() and (gn[miss] == 0).all(), f"{what}: non-zero outputs on pixels both sides miss"
    scale = np.maximum(np.linalg.norm(ox, axis=1), np.linalg.norm(ox - rays[:, 0:3], axis=1))
    relx = np.linalg.norm(gx - ox, axis=1) / np.maximum(scale, 1e-30)
    nerr = np.abs(gn - on).max(1)
    same = (gi == oi) & (oi > 0)
    suspect = (gi != oi) | (same & ((relx > DIST_REL) | (nerr > DIST_REL)))
    idx = np.nonzero(suspect)[0]
    eps = edge_eps(rays[idx], index.extent)
    pts = [np.where((gi[idx] > 0)[:, None], gx[idx], np.nan), np.where((oi[idx] > 0)[:, None], ox[idx], np.nan)]
    prims = [p[idx] for p in (oprim, gprim) if p is not None]
    bad = idx[unexcused(index, rays[idx], eps, prims=prims, points=pts)]
    assert len(bad) == 0, (f"{what}: {len(bad)} of {len(gi)} pixels disagree away from triangle edges (first "
                           f"{bad[:5]}: ids {gi[bad[:5]]} vs {oi[bad[:5]]}, rel point err {relx[bad[:5]]}, "
                           f"normal err {nerr[bad[:5]]})")
    return {"pixels": int(len(gi)), "hit": int((oi > 0).sum()), "suspect": int(len(idx)),
            "id_mismatch": int((gi != oi).sum()), "max_rel_point": float(relx[same].max()) if same.any() else 0.0}


def check_hits(index, rays, g_prim, g_t, o_prim, o_t, what="closest hits"):
    """Closest hits of the GPU (prim, t; CRT_MISS -> -1) against the oracle: the same triangle with t
    within DIST_REL of max(t, |origin|) (FP32 rounds coordinates, so the error of a hit distance
    scales with the coordinates, not with the distance when that is much shorter), or excused by
    the edge rule (either side's triangle), or both hit at the same distance (coplanar overlapping
    triangles).  Returns the number of rays whose triangles differ."""
    g_prim = np.asarray(g_prim).astype(np.int64)
    o_prim = np.asarray(o_prim).astype(np.int64)
    g_t, o_t = np.asarray(g_t, np.float64), np.asarray(o_t, np.float64)
    tol = DIST_REL * np.maximum(np.maximum(np.abs(o_t), np.linalg.norm(rays[:, 0:3], axis=1)), 1e-30)
    same = g_prim == o_prim
    tbad = same & (o_prim >= 0) & (np.abs(g_t - o_t) > tol)
    idx = np.nonzero(~same | tbad)[0]
    tie = (g_prim[idx] >= 0) & (o_prim[idx] >= 0) & (np.abs(g_t[idx] - o_t[idx]) <= tol[idx])
    idx = idx[~tie]
    eps = edge_eps(rays[idx], index.extent)
    bad = idx[unexcused(index, rays[idx], eps, prims=[g_prim[idx], o_prim[idx]])]
    assert len(bad) == 0, (f"{what}: {len(bad)} of {len(rays)} rays disagree away from triangle edges (first "
                           f"{bad[:5]}: prim {g_prim[bad[:5]]} vs {o_prim[bad[:5]]}, t {g_t[bad[:5]]} vs {o_t[bad[:5]]})")
    return int((~same).sum())


def check_occlusion(index, rays, g_occ, o_occ, occluders, what="any hits"):
    """Any-hit flags of the GPU against the oracle.  A ray on which they differ is excused when its
    line passes within the edge distance of an edge of a triangle it meets before tmax on the side
    that reports the occlusion (`occluders`: per ray, the closest-hit triangle found by that side's
    closest-hit traversal of the same ray, or its hit point), or meets it within DIST_REL of tmax."""
    g_occ, o_occ = np.asarray(g_occ).astype(bool), np.asarray(o_occ).astype(bool)
    idx = np.nonzero(g_occ != o_occ)[0]
    if len(idx) == 0:
        return 0
    prims, pts, ts = occluders(idx)
    eps = edge_eps(rays[idx], index.extent)
    at_end = np.zeros(len(idx), dtype=bool)
    for t in ts:
        at_end |= np.abs(t - rays[idx, 7]) <= DIST_REL * np.abs(rays[idx, 7])
    sub = np.nonzero(~at_end)[0]
    bad = idx[sub[unexcused(index, rays[idx[sub]], eps[sub], prims=[p[sub] for p in prims],
                            points=[p[sub] for p in pts])]]
    assert len(bad) == 0, f"{what}: {len(bad)} of {len(rays)} rays differ away from triangle edges (first {bad[:5]})"
    return int(len(idx))


def check_direct_render(index, rays, g_rad, o_rad, o_x, o_prim, g_x, g_prim, lights, trace_o, trace_g,
                        what="render"):
    """Deterministic radiance (1 spp at pixel centres, 1 bounce, point lights: no random draws) of the
    GPU against the oracle.  Pixel values agree within FP32 rounding (1e-4 relative + 1e-6 of the
    image maximum) unless the pixel is excused:
      1. its camera ray is excused by the edge rule (unexcused) at either side's triangle or hit point;
      2. for some light, its shadow ray is: the ray from the oracle's surface point toward the light
         passes within the edge distance of an edge of the triangle that occludes it on either side
         (trace_o / trace_g: closest hits of [k, 8] FP64 rays -> (prim, t));
      3. for some light, its shadow ray points into the surface it leaves and crosses that triangle's
         plane near the triangle's edge: within twice a bound on the FP32 error of the surface point,
         4e-6 x ((|origin| + range) / cos(incidence) + |x|), plus the edge distance and the FP32 error
         of the crossing's shift: the reference then stops the ray on its own triangle or not by a
         hair, and the device decides that case from its FP32 surface point.
    Returns counts."""
    g = np.asarray(g_rad, np.float64).reshape(-1, np.asarray(g_rad).shape[-1])[:, :3]
    r = np.asarray(o_rad, np.float64).reshape(-1, np.asarray(o_rad).shape[-1])[:, :3]
    tol = 1e-4 * np.abs(r) + 1e-6 * max(np.abs(r).max(), 1e-30)
    idx = np.nonzero((np.abs(g - r) > tol).any(1))[0]
    rays = rays[idx]
    ox, oprim = np.asarray(o_x).reshape(-1, 3)[idx], np.asarray(o_prim).ravel()[idx]
    gx, gprim = np.asarray(g_x).reshape(-1, 3)[idx], np.asarray(g_prim).ravel()[idx]
    eps = edge_eps(rays, index.extent)
    left = unexcused(index, rays, eps, prims=[oprim, gprim],
                     points=[np.where(gprim[:, None] >= 0, gx, np.nan), np.where(oprim[:, None] >= 0, ox, np.nan)])
    k = left[oprim[left] >= 0]
    tris = index.tris
    n_in = tris[oprim[k], 9:12] / np.linalg.norm(tris[oprim[k], 9:12], axis=1)[:, None]
    excused = np.zeros(len(k), dtype=bool)
    n_shadow = n_reentry = 0
    for light in lights:
        if not len(k) or excused.all():
            break
        lp = np.asarray(light["position"], dtype=np.float64)
        s = ox[k] - 1e-4 * n_in                      # the reference's shadow-ray origin
        L = lp[None, :] - s
        dist = np.linalg.norm(L, axis=1)
        sr = np.zeros((len(k), 8))
        sr[:, 0:3], sr[:, 3:6], sr[:, 7] = s, L / dist[:, None], dist
        po, to = trace_o(sr)
        gs = sr.copy()
        off = np.maximum(1e-4, 4.0 * np.spacing(np.abs(ox[k]).max(1).astype(np.float32)).astype(np.float64))
        gs[:, 0:3] = ox[k] - off[:, None] * n_in    # the device's origin (max(1e-4, 4 ulp) off the surface)
        pg, tg = trace_g(gs)
        pts_o = np.where((po >= 0)[:, None], sr[:, 0:3] + to[:, None] * sr[:, 3:6], np.nan)
        pts_g = np.where((pg >= 0)[:, None], gs[:, 0:3] + tg[:, None] * gs[:, 3:6], np.nan)
        s_eps = edge_eps(sr, index.extent)
        still = np.zeros(len(k), dtype=bool)
        still[unexcused(index, sr, s_eps, prims=[po, pg], points=[pts_o, pts_g])] = True
        n_shadow += int((~still & ~excused).sum())
        excused |= ~still
        # re-entry into the surface it leaves
        d = sr[:, 3:6]
        c = (d * n_in).sum(1)
        q = sr[:, 0:3] + (1e-4 / np.where(c > 0, c, 1.0))[:, None] * d
        de = edge_distance(tris, oprim[k], q)
        v_in = ox[k] - rays[k, 0:3]
        t_in = np.linalg.norm(v_in, axis=1)
        cos_in = np.abs((v_in * n_in).sum(1)) / t_in
        margin = 4e-6 * ((np.abs(rays[k, 0:3]).max(1) + t_in) / np.maximum(cos_in, 1e-3) + np.abs(ox[k]).max(1))
        shift = 1e-4 * np.sqrt(np.maximum(0.0, 1.0 - c * c)) / np.where(c > 0, c, 1.0)
        re = (c > 0) & (de <= 2 * margin + s_eps + shift * 4e-6 / np.where(c > 0, c, 1.0))
        n_reentry += int((re & ~excused).sum())
        excused |= re
    bad = np.concatenate([left[oprim[left] < 0], k[~excused]])
    assert len(bad) == 0, (f"{what}: {len(bad)} of {len(g)} pixels differ away from triangle edges (first "
                           f"pixels {idx[bad[:5]]}: gpu {g[idx[bad[:5]]]} oracle {r[idx[bad[:5]]]})")
    return {"pixels": int(len(g)), "not_equal": int(len(idx)), "primary_edge": int(len(idx) - len(left)),
            "shadow_edge": n_shadow, "reentry": n_reentry}


def radiance_z(g, r, m2, n):
    """z-scores of GPU minus oracle radiance values (per pixel and channel): both are means of n samples
    of the same estimator, so their difference has variance 2 s^2 / n with s^2 = M2 / (n - 1) the
    oracle's per-pixel sample variance; a floor of 1e-4 of the value plus 1e-6 covers the FP32
    rounding of paths that agree."""
    n = np.asarray(n, np.float64)
    if n.ndim:
        n = n[..., None]
    se = np.sqrt(2.0 * np.asarray(m2) / np.maximum(n - 1, 1) / n) + 1e-4 * np.abs(r) + 1e-6
    return np.abs(np.asarray(g, np.float64) - np.asarray(r, np.float64)) / se


def check_mc_radiance(g, r, m2, n, what="render", budget=1e-3, mean_tol=5e-3):
    """Monte-Carlo radiance (same random streams on both sides): at most `budget` of the pixel values
    beyond 4 sigma, image mean within mean_tol.  Returns counts."""
    g = np.asarray(g, np.float64)[..., :3]
    r = np.asarray(r, np.float64)[..., :3]
    z = radiance_z(g, r, m2, n)
    frac = float((z > 4).mean())
    ratio = float(g.mean() / r.mean()) if r.mean() != 0 else 1.0
    assert frac <= budget, f"{what}: {int((z > 4).sum())} of {z.size} values beyond 4 sigma (max z {z.max():.1f})"
    assert abs(ratio - 1) < mean_tol, f"{what}: image mean ratio {ratio}"
    return {"values": int(z.size), "beyond_4sigma": int((z > 4).sum()), "equal": float((g == r).mean()),
            "mean_ratio": ratio}


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
