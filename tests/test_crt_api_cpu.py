"""Host-side logic of the drop-in `crt` package (no GPU): body-frame transforms, LiDAR pose batches,
the `_crt` module surface and argument handling."""
import numpy as np
import pytest

from crt_gb300 import scenes


def reference_transform_to_body(group_pos, group_rot, scale, position, rotation):
    # crt/body_fixed.py:87-101 of the reference, written out
    relative_position = scale * np.matmul(group_rot, position - group_pos)
    relative_rotation = np.matmul(group_rot, rotation.T).T
    return relative_position, relative_rotation


class FakeCpp:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def f(*a, **k):
            self.calls.append((name, a, k))
            return np.zeros((1, 3))
        return f


def make_group(pos, rot, scale=1.0):
    import crt
    g = crt.BodyFixedGroup.__new__(crt.BodyFixedGroup)
    g.position, g.rotation, g.scale = np.asarray(pos, float), np.asarray(rot, float), scale
    g._cpp = FakeCpp()
    return g


def test_module_surface_matches_reference():
    import _crt
    names = {n for n in dir(_crt) if not n.startswith("_")}
    assert {"AreaLight", "BodyFixedEntity", "BodyFixedGroup", "Entity", "PointLight", "SimpleCamera", "SimpleLidar",
            "instance_pass", "intersection_pass", "normal_pass", "render", "simulate_lidar"} <= names
    import crt
    assert set(crt.__all__) == {"Entity", "RigidBody", "BodyFixedGroup", "BodyFixedEntity"}


def test_transform_to_body_matches_reference_formula():
    rng = np.random.Generator(np.random.PCG64(3))
    R = scenes.quaternion_to_matrix(scenes.random_quaternions(1, 5)[0])
    g = make_group(rng.normal(size=3), R, scale=2.5)
    p, r = rng.normal(size=3), scenes.quaternion_to_matrix(scenes.random_quaternions(1, 6)[0])
    a = g.transform_to_body(p, r)
    b = reference_transform_to_body(g.position, g.rotation, g.scale, p, r)
    np.testing.assert_allclose(a[0], b[0], rtol=1e-14)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-14, atol=1e-15)


def test_batch_lidar_poses_match_per_pose_transform():
    from crt.lidars import SimpleLidar
    rng = np.random.Generator(np.random.PCG64(4))
    R = scenes.quaternion_to_matrix(scenes.random_quaternions(1, 7)[0])
    g = make_group(rng.normal(size=3), R, scale=0.5)
    n = 17
    pos = rng.normal(size=(n, 3)) * 100
    rots = np.stack([scenes.quaternion_to_matrix(q) for q in scenes.random_quaternions(n, 8)], axis=2)
    lid = SimpleLidar()
    lid.batch_set_pose(pos, rots)
    g.batch_simulate_lidar(lid)
    # the lidar now holds body-frame poses; compare with the reference's per-pose loop (body_fixed.py:152-162)
    for k in range(n):
        p_ref, r_ref = reference_transform_to_body(g.position, g.rotation, g.scale, pos[k], rots[:, :, k])
        np.testing.assert_allclose(lid.batch_positions[k], p_ref, rtol=1e-13, atol=1e-12)
        np.testing.assert_allclose(lid.batch_rotations[:, :, k], r_ref, rtol=1e-13, atol=1e-14)


def test_render_moves_camera_and_lights_into_body_frame():
    from crt.cameras import SimpleCamera
    from crt.lights import AreaLight, PointLight
    R = scenes.quaternion_to_matrix(scenes.random_quaternions(1, 9)[0])
    g = make_group([1.0, 2.0, 3.0], R)
    cam = SimpleCamera(1.0, [8, 8], [1.0, 1.0], position=[10.0, 0.0, 0.0])
    p_exp, r_exp = g.transform_to_body(cam.position, cam.rotation)
    lights = [PointLight(5.0, position=[0.0, 9.0, 0.0]), AreaLight(2.0, [1.0, 2.0])]
    g.render(cam, lights, 1, 2, 0.5, 3)
    np.testing.assert_allclose(cam.position, p_exp)
    np.testing.assert_allclose(cam.rotation, r_exp)
    name, args, kw = g._cpp.calls[-1]
    assert name == "render" and args[2:] == (1, 2, 0.5, 3) and len(args[1]) == 2


def test_lidar_batch_limit_and_shapes():
    from crt.lidars import SimpleLidar
    lid = SimpleLidar()
    with pytest.raises(ValueError):
        lid.batch_set_pose(np.zeros((100001, 3)), np.zeros((3, 3, 100001)))
    with pytest.raises(ValueError):
        SimpleLidar(position=[1.0, 2.0])


def test_rotations_module():
    from crt.rotations import euler_to_rotmat
    R = euler_to_rotmat("123", [10, 20, 30], degrees=True)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-14)
    with pytest.raises(Exception):
        euler_to_rotmat("124", [0, 0, 0])


def test_srp_request_packing():
    """An SRP query of a mixed batch / server request fills crt_server_request as the C side reads it
    (kind SRP, the scene handle, the descriptor, n_att quaternions and the two output buffers)."""
    import ctypes
    from crt_gb300 import lib

    class FakeScene:
        h = ctypes.c_void_p(0x1234)

    q = dict(kind="srp", scene=FakeScene(), sun_dir=[0.0, 2.0, 0.0], quaternions=np.eye(4)[:3], grid=640,
             num_bounces=1, flux=1000.0, center_of_mass=(0.1, 0.2, 0.3))
    sr, keep = lib.ServerRequest(), []
    force, torque = lib.fill_srp_request(q, sr, None, keep)
    assert sr.base.kind == lib.REQUEST_SRP and sr.base.scene == 0x1234
    assert sr.n_att == 3 and force.shape == (3, 3) and torque.shape == (3, 3)
    assert sr.force == force.ctypes.data and sr.torque == torque.ctypes.data
    d = sr.srp.contents
    assert list(d.sun_dir_inertial) == [0.0, 2.0, 0.0] and d.grid == 640 and d.num_bounces == 1
    assert d.flux == 1000.0 and abs(d.c - 299792458.0) < 1 and list(d.center_of_mass) == [0.1, 0.2, 0.3]
    quats = np.ctypeslib.as_array(ctypes.cast(sr.quaternions, ctypes.POINTER(ctypes.c_double)), shape=(3, 4))
    np.testing.assert_array_equal(quats, np.eye(4)[:3])
    # the request struct the C ABI reads: base request, then the SRP fields
    assert ctypes.sizeof(lib.ServerRequest) == ctypes.sizeof(lib.Request) + 5 * 8


def test_spice_pose_helpers_call_spice_as_the_reference(monkeypatch):
    """spice_position / spice_rotation / spice_pose pass (name, et, ref, abcorr, origin) to spkpos and
    (ref, frame, et) to pxform (crt/rigid_body.py:191, 206, 229-230 of the reference); spiceypy itself
    is replaced by a recording fake (it is not installed)."""
    import sys
    import types
    R = scenes.quaternion_to_matrix(scenes.random_quaternions(1, 11)[0])
    calls = []
    fake = types.ModuleType("spiceypy")

    def spkpos(targ, et, ref, abcorr, obs):
        calls.append(("spkpos", targ, et, ref, abcorr, obs))
        return np.array([1.0, -2.0, 3.5]), 0.25

    def pxform(frm, to, et):
        calls.append(("pxform", frm, to, et))
        return R

    fake.spkpos, fake.pxform = spkpos, pxform
    monkeypatch.setitem(sys.modules, "spiceypy", fake)
    from crt.rigid_body import RigidBody
    b = RigidBody(name="EROS", frame="IAU_EROS", origin="SUN", ref="ECLIPJ2000", abcorr="LT+S")
    b._cpp = FakeCpp()
    b.spice_pose(12.5)
    assert calls == [("spkpos", "EROS", 12.5, "ECLIPJ2000", "LT+S", "SUN"),
                     ("pxform", "ECLIPJ2000", "IAU_EROS", 12.5)]
    np.testing.assert_array_equal(b.position, [1.0, -2.0, 3.5])
    np.testing.assert_array_equal(b.rotation, R)
    assert b._cpp.calls[-1][0] == "set_pose"
    calls.clear()
    b.spice_position(1.0)
    b.spice_rotation(2.0)
    assert calls == [("spkpos", "EROS", 1.0, "ECLIPJ2000", "LT+S", "SUN"), ("pxform", "ECLIPJ2000", "IAU_EROS", 2.0)]
    assert [c[0] for c in b._cpp.calls[-2:]] == ["set_position", "set_rotation"]


def test_lidar_batch_spice_pose(monkeypatch):
    """batch_spice_pose: one vectorised spkpos over the epochs and one pxform per epoch
    (crt/lidars.py:32-44 of the reference), then the batch pose arrays the extension receives."""
    import sys
    import types
    from crt.lidars import SimpleLidar
    ets = np.array([0.0, 60.0, 120.0])
    pos = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.5]])
    rots = [scenes.quaternion_to_matrix(q) for q in scenes.random_quaternions(3, 12)]
    calls = []
    fake = types.ModuleType("spiceypy")

    def spkpos(targ, et, ref, abcorr, obs):
        calls.append(("spkpos", targ, tuple(np.atleast_1d(et)), ref, abcorr, obs))
        return pos, np.zeros(3)

    def pxform(frm, to, et):
        calls.append(("pxform", frm, to, float(et)))
        return rots[int(et // 60)]

    fake.spkpos, fake.pxform = spkpos, pxform
    monkeypatch.setitem(sys.modules, "spiceypy", fake)
    lid = SimpleLidar(name="SC", frame="SC_LIDAR", origin="EROS", ref="J2000", abcorr="NONE")
    lid._cpp = FakeCpp()
    lid.batch_spice_pose(ets)
    assert calls[0] == ("spkpos", "SC", (0.0, 60.0, 120.0), "J2000", "NONE", "EROS")
    assert calls[1:] == [("pxform", "J2000", "SC_LIDAR", e) for e in (0.0, 60.0, 120.0)]
    np.testing.assert_array_equal(lid.batch_positions, pos)
    name, args, _ = lid._cpp.calls[-1]
    assert name == "batch_set_pose" and args[2] == 3 and args[1].shape == (3, 3, 100000)
    for k in range(3):
        np.testing.assert_array_equal(args[1][:, :, k], rots[k])
    assert not args[1][:, :, 3:].any()


def test_dynamic_passes_return_images(monkeypatch):
    """crt.rendering's passes hand the entities' C++ objects to _crt and, with return_image, add the
    reference's images (crt/rendering.py:54-144): 255 |n| for normals, the distance to the origin
    shifted to 0 and scaled to 255 for intersections, one colour per instance id."""
    import types
    import crt.rendering as rendering
    rng = np.random.Generator(np.random.PCG64(13))
    pts = rng.normal(size=(6, 5, 3))
    nrm = rng.normal(size=(6, 5, 3))
    ids = rng.integers(0, 4, size=(6, 5)).astype(np.uint32)
    seen = []

    def rec(out):
        def f(cam, ents):
            seen.append((cam, list(ents)))
            return out
        return f

    fake = types.SimpleNamespace(normal_pass=rec(nrm), intersection_pass=rec(pts), instance_pass=rec(ids))
    monkeypatch.setattr(rendering, "_crt", fake)
    cam = types.SimpleNamespace(_cpp="camera")
    ents = [types.SimpleNamespace(_cpp="e0"), types.SimpleNamespace(_cpp="e1")]
    n, img = rendering.normal_pass(cam, ents, return_image=True)
    assert n is nrm and np.array_equal(img, 255 * np.abs(nrm))
    p, img = rendering.intersection_pass(cam, ents, return_image=True)
    dist = np.sqrt(pts[:, :, 0] ** 2 + pts[:, :, 1] ** 2 + pts[:, :, 2] ** 2)
    np.testing.assert_allclose(img, 255 * (dist - dist.min()) / (dist - dist.min()).max(), rtol=1e-15)
    i, img = rendering.instance_pass(cam, ents, return_image=True)
    assert img.shape == (6, 5, 3)
    for k in np.unique(ids):
        assert len(np.unique(img[ids == k], axis=0)) == 1
    assert all(s == ("camera", ["e0", "e1"]) for s in seen) and len(seen) == 3
    assert rendering.normal_pass(cam, ents) is nrm
