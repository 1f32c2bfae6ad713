"""BVH topology builders: the binned-SAH tree (default) and the radix tree over the Morton order
(crt_tuning.build_sah = 0) must answer every query the same way — closest hits may differ only on
exact ties, at the same distance — and both must be exact on degenerate inputs (coincident
triangles, identical centroids, slivers, sizes around the 4-triangle segment limit)."""
import numpy as np
import pytest

import oracle
from crt_gb300 import lib, scenes
from helpers import TriIndex, check_hits, check_occlusion, to_f32_rays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


def random_rays(rng, n, spread=3.0, center=(0.0, 0.0, 0.0)):
    org = rng.normal(size=(n, 3)) * spread + np.asarray(center)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    rays = np.zeros((n, 8))
    rays[:, :3], rays[:, 3:6], rays[:, 7] = org, dirs, 3.0e38
    return to_f32_rays(rays)


def as32(rays64):
    return lib.make_rays(rays64[:, 0:3], rays64[:, 3:6])


def build_both(ctx, ents):
    ctx.set_tuning(build_sah=True)
    a = ctx.scene(ents)
    ctx.set_tuning(build_sah=False)
    b = ctx.scene(ents)
    ctx.set_tuning()
    return a, b


@pytest.mark.parametrize("other", ["radix", "leaf_cost_0.5"])
def test_sah_and_radix_trees_agree_on_asteroid(ctx, other):
    ents = [scenes.EntitySpec("a", scenes.asteroid(100_000, seed=11), (0.1, 0.1, 0.1))]
    if other == "radix":
        sah, radix = build_both(ctx, ents)
    else:   # the same topology collapsed with a larger triangle cost (smaller leaves)
        sah = ctx.scene(ents)
        ctx.set_tuning(collapse_tri_cost=0.5)
        radix = ctx.scene(ents)
        ctx.set_tuning()
        assert radix.stats()["n_nodes"] > sah.stats()["n_nodes"]
    assert sah.stats()["n_tris"] == radix.stats()["n_tris"] == 100_000
    rng = np.random.Generator(np.random.PCG64(5))
    rays = as32(random_rays(rng, 200_000, spread=1500.0))
    h1, h2 = sah.trace_closest(rays), radix.trace_closest(rays)
    same = h1["prim"] == h2["prim"]
    assert same.mean() > 0.9999
    # where they differ, both report a hit at the same distance (an exact tie on a shared edge)
    diff = ~same
    assert ((h1["prim"][diff] != lib.CRT_MISS) & (h2["prim"][diff] != lib.CRT_MISS)).all()
    np.testing.assert_array_equal(h1["t"][diff], h2["t"][diff])
    np.testing.assert_array_equal(h1["t"][same], h2["t"][same])
    np.testing.assert_array_equal(sah.trace_any(rays), radix.trace_any(rays))


@pytest.mark.parametrize("case", ["coincident", "same_centroid", "slivers", "n5", "n8", "n9", "n33"])
def test_degenerate_inputs_vs_oracle(ctx, case):
    rng = np.random.Generator(np.random.PCG64(len(case)))
    if case == "coincident":          # 200 copies of one triangle plus scattered ones
        base = rng.uniform(-1, 1, size=(1, 3, 3))
        tris = np.concatenate([np.repeat(base, 200, axis=0), rng.uniform(-1, 1, size=(50, 3, 3))])
    elif case == "same_centroid":     # triangles rotated about a common centroid
        ang = rng.uniform(0, 2 * np.pi, size=300)
        r = rng.uniform(0.1, 1.0, size=300)[:, None]
        v0 = np.stack([np.cos(ang), np.sin(ang), np.zeros(300)], 1) * r
        v1 = np.stack([np.cos(ang + 2.1), np.sin(ang + 2.1), 0.3 * np.ones(300)], 1) * r
        v2 = -(v0 + v1)
        tris = np.stack([v0, v1, v2], 1)
    elif case == "slivers":           # long thin triangles along one line
        x = np.sort(rng.uniform(-5, 5, size=(400, 2)), axis=1)
        tris = np.zeros((400, 3, 3))
        tris[:, 0, 0], tris[:, 1, 0], tris[:, 2, 0] = x[:, 0], x[:, 1], x[:, 1]
        tris[:, 2, 1] = 1e-3
        tris[:, :, 2] = rng.uniform(-0.01, 0.01, size=(400, 1))
    else:                             # sizes around the segment limit
        k = int(case[1:])
        tris = rng.uniform(-1, 1, size=(k, 3, 3))
    v = tris.reshape(-1, 3).astype(np.float32)
    f = np.arange(len(v), dtype=np.int32).reshape(-1, 3)
    ents = [scenes.EntitySpec("t", scenes.Mesh(v, f))]
    sah, radix = build_both(ctx, ents)
    rays = random_rays(rng, 4096, spread=2.0)
    o = oracle.Scene(ents)
    prim_o, t_o, _, _ = o.trace_closest(rays)
    index = TriIndex(o.tris())
    for sc in (sah, radix):
        # closest hits: the same triangle, or the same distance (coincident triangles tie exactly; any
        # of them is a correct closest hit), or a ray at a triangle edge (helpers.check_hits)
        h = sc.trace_closest(as32(rays))
        gp = np.where(h["prim"] == lib.CRT_MISS, -1, h["prim"].astype(np.int64))
        check_hits(index, rays, gp, h["t"], prim_o, t_o, what=f"{case} closest hits")
        occ = sc.trace_any(as32(rays))
        check_occlusion(index, rays, occ, prim_o >= 0,
                        lambda idx: ([gp[idx], prim_o[idx]], [], [h["t"][idx].astype(np.float64), t_o[idx]]),
                        what=f"{case} any hits")
