"""Workload generators (host C++ / numpy, no GPU) against the workload definitions they stand for:
the procedural asteroid (icosphere of 20 * 4^level faces decimated to the target count, radius
1000 m, 5 % radial noise, seeded), the radiation-pressure spacecraft (2 x 2 x 3 m bus, two 1 x 6 m
panels, a 2 m parabolic dish as a 64 x 64 radial mesh; about 50k triangles) and the Cornell box
(36 triangles, 40 degree field of view, 0.25 m area light of intensity 15)."""
import numpy as np

from crt_gb300 import scenes


def edges(f, directed):
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    if not directed:
        e = np.sort(e, axis=1)
    return np.unique(e, axis=0, return_counts=True)[1]


def test_asteroid_closed_oriented_and_seeded():
    m = scenes.asteroid(20000, seed=3)
    v, f = m.vertices.astype(np.float64), m.faces
    assert f.shape == (20000, 3) and v.shape == (20000 // 2 + 2, 3)     # genus 0: V = F / 2 + 2
    assert (edges(f, False) == 2).all() and (edges(f, True) == 1).all()  # watertight, consistent winding
    vol = np.einsum("ij,ij->i", v[f[:, 0]], np.cross(v[f[:, 1]], v[f[:, 2]])).sum() / 6
    assert abs(vol / (4 / 3 * np.pi * 1000.0 ** 3) - 1) < 0.02        # outward winding, radius 1000 m
    r = np.linalg.norm(v, axis=1)
    assert 950.0 < r.min() and r.max() < 1050.0                           # 5 % radial noise
    again = scenes.asteroid(20000, seed=3)
    assert np.array_equal(again.vertices, m.vertices) and np.array_equal(again.faces, m.faces)
    assert not np.array_equal(scenes.asteroid(20000, seed=4).vertices, m.vertices)


def test_asteroid_levels_for_the_workload_sizes():
    # 2M triangles from a 9-subdivision icosphere (5,242,880 faces), 8M from 10 (20,971,520)
    assert scenes.asteroid_level_for(2_000_000) == 9 and 20 * 4 ** 9 == 5_242_880
    assert scenes.asteroid_level_for(8_000_000) == 10 and 20 * 4 ** 10 == 20_971_520
    full = scenes.asteroid(0, level=3)
    assert full.faces.shape == (20 * 4 ** 3, 3)


def test_spacecraft_parts():
    sc = {e.name: e for e in scenes.spacecraft()}
    assert set(sc) == {"bus", "panel_a", "panel_b", "dish"}
    assert sum(e.mesh.n_tris for e in sc.values()) == 48_728
    assert (sc["bus"].rho_s, sc["bus"].rho_d) == (0.1, 0.5) and (sc["dish"].rho_s, sc["dish"].rho_d) == (0.1, 0.5)
    for p in ("panel_a", "panel_b"):
        assert (sc[p].rho_s, sc[p].rho_d) == (0.3, 0.2)
        ext = sc[p].mesh.vertices.max(0) - sc[p].mesh.vertices.min(0)
        np.testing.assert_allclose(ext, [1.0, 6.0, 0.0], atol=1e-6)
    np.testing.assert_allclose(sc["bus"].mesh.vertices.max(0) - sc["bus"].mesh.vertices.min(0), [2.0, 2.0, 3.0])
    dish = sc["dish"].mesh
    assert dish.n_tris == 64 + 2 * 63 * 64                                 # apex fan + 63 rings of quads
    np.testing.assert_allclose(dish.vertices[:, :2].max(0) - dish.vertices[:, :2].min(0), [2.0, 2.0], atol=1e-6)


def test_cornell_box():
    ents, cam, lights = scenes.cornell()
    assert sum(e.mesh.n_tris for e in ents) == 36 and len(ents) == 6
    colors = {e.name: e.color for e in ents}
    assert colors["left"] == (0.65, 0.05, 0.05) and colors["right"] == (0.12, 0.45, 0.15)
    assert colors["walls"] == (0.73, 0.73, 0.73)
    heights = {n: float(np.asarray(e.mesh.vertices)[:, 1].max()) for n, e in ((e.name, e) for e in ents)}
    assert abs(heights["short_box"] - 0.3) < 1e-6 and abs(heights["tall_box"] - 0.6) < 1e-6
    assert cam["resolution"] == [256, 256]
    assert abs(cam["sensor_size"][0] / (2 * cam["focal_length"]) - np.tan(np.deg2rad(20.0))) < 1e-12
    (light,) = lights
    assert light["type"] == "area" and light["intensity"] == 15.0 and list(light["size"]) == [0.25, 0.25]
