"""The oracle's radiation-pressure restatement (no GPU) against closed forms.

The reference has no SRP code, so the oracle that checks the GPU's SRP is pinned here by the
published flat-plate and cannonball results (Montenbruck & Gill, Satellite Orbits, sec. 3.4):
    plate:  F = -P A cos(t) [(1 - rs) s + 2 (rs cos(t) + rd / 3) n],  absorbed (1 - rs - rd) flux A cos(t)
    sphere: F = -P pi R^2 (1 + 4 rd / 9) s,  no torque about the centre
with P = flux / c and s the unit vector toward the sun."""
import numpy as np

import oracle
from crt_gb300 import scenes

C = 299792458.0
FLUX = 1361.0


def params(mesh, sun, grid, nb=0):
    v = np.asarray(mesh.vertices, dtype=np.float64)
    lo, hi = v.min(0), v.max(0)
    p = oracle.SrpParams()
    p.sun_dir[:] = [float(x) for x in sun]
    p.flux, p.c = FLUX, C
    p.center[:] = list(0.5 * (lo + hi))
    p.half_extent = 0.5 * float(np.sqrt(((hi - lo) ** 2).sum()))
    p.center_of_mass[:] = [0.0, 0.0, 0.0]
    p.grid, p.num_bounces = grid, nb
    return p


def test_oracle_flat_plate_closed_form():
    rs, rd = 0.3, 0.2
    plate = scenes.quad_mesh((-0.5, -0.5, 0.0), (0.5, -0.5, 0.0), (0.5, 0.5, 0.0), (-0.5, 0.5, 0.0))
    o = oracle.Scene([scenes.EntitySpec("p", plate, rho_s=rs, rho_d=rd)])
    theta = np.deg2rad(35.0)
    s = np.array([np.sin(theta), 0.0, np.cos(theta)])
    f, t, fp = o.srp(params(plate, s, 2048))
    P, cs, n = FLUX / C, np.cos(theta), np.array([0.0, 0.0, 1.0])
    expect = -P * cs * ((1 - rs) * s + 2 * (rs * cs + rd / 3) * n)
    np.testing.assert_allclose(f, expect, rtol=3e-3, atol=3e-3 * np.abs(expect).max())
    assert abs(fp.sum() / ((1 - rs - rd) * FLUX * cs) - 1) < 3e-3
    assert np.abs(t).max() < 1e-3 * np.abs(expect).max()


def test_oracle_sphere_closed_form():
    rd = 0.4
    sph = scenes.asteroid(target_faces=0, level=6, radius=1.0, amplitude=0.0)
    o = oracle.Scene([scenes.EntitySpec("s", sph, rho_s=0.0, rho_d=rd)])
    s = scenes.unit_vector(4)
    f, t, _ = o.srp(params(sph, s, 1024))
    expect = -(FLUX / C) * np.pi * (1 + 4 * rd / 9) * s   # tessellation: projected area slightly < pi
    np.testing.assert_allclose(f, expect, rtol=0.01, atol=0.01 * np.abs(expect).max())
    assert np.linalg.norm(t) < 1e-3 * np.linalg.norm(expect)
