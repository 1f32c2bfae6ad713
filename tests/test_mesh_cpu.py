"""OBJ ingest (crt_mesh_load_obj, host C++; no GPU) against the rules of the reference's loader
(lib/model_loaders/obj.hpp:59-117): comments and blank lines skipped, `vt` / `vn` lines ignored,
faces fan-triangulated from their first vertex, negative indices relative to the vertices read so
far, `/vt/vn` parts of a face index ignored, vertex normals the normalised sums of the incident
triangles' unnormalised left-handed normals (p0 - p1) x (p2 - p0)."""
import ctypes

import numpy as np

from crt_gb300 import lib

OBJ = """# two faces and a quad
v 0 0 0
v 1 0 0

v 1 1 0
v 0 1 0
v 0.25 0.5 1
vt 0 0
vn 0 0 1
f 1 2 3 4
f -5/1/1 -4//1 -1
   f 2/1 3/1 5/1
"""


def expected():
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.25, 0.5, 1]], dtype=np.float64)
    tris = [(0, 1, 2), (0, 2, 3), (0, 1, 4), (1, 2, 4)]
    acc = np.zeros_like(v)
    for a, b, c in tris:
        n = np.cross(v[a] - v[b], v[c] - v[a])
        for k in (a, b, c):
            acc[k] += n
    vn = acc / np.linalg.norm(acc, axis=1)[:, None]
    xyz = np.array([np.concatenate([v[a], v[b], v[c]]) for a, b, c in tris])
    nrm = np.array([np.concatenate([vn[a], vn[b], vn[c]]) for a, b, c in tris])
    return xyz, nrm


def load(path):
    L = lib.load()
    h = ctypes.c_void_p()
    rc = L.crt_mesh_load_obj(str(path).encode(), ctypes.byref(h))
    if rc != 0:
        return rc, None, None
    n = L.crt_mesh_num_tris(h)
    if n == 0:   # no triangles: the data pointers may be null
        L.crt_mesh_destroy(h)
        return rc, np.zeros((0, 9), np.float32), np.zeros((0, 9), np.float32)
    xyz = np.ctypeslib.as_array((ctypes.c_float * (9 * n)).from_address(L.crt_mesh_xyz(h))).copy()
    nrm = np.ctypeslib.as_array((ctypes.c_float * (9 * n)).from_address(L.crt_mesh_normals(h))).copy()
    L.crt_mesh_destroy(h)
    return rc, xyz.reshape(-1, 9), nrm.reshape(-1, 9)


def test_obj_faces_indices_and_vertex_normals(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text(OBJ)
    rc, xyz, nrm = load(p)
    assert rc == 0
    exyz, enrm = expected()
    np.testing.assert_array_equal(xyz, exyz.astype(np.float32))
    np.testing.assert_allclose(nrm, enrm, atol=1e-7)


def test_obj_missing_file_and_no_faces(tmp_path):
    assert load(tmp_path / "missing.obj")[0] == -5   # CRT_ERR_IO
    p = tmp_path / "v.obj"
    p.write_text("v 0 0 0\nv 1 0 0\n# no faces\n")
    rc, xyz, _ = load(p)
    assert rc == 0 and xyz.shape == (0, 9)


def test_obj_index_out_of_range(tmp_path):
    """A face index of 0, past the last vertex read so far, or a negative index reaching before the
    first vertex is refused (CRT_ERR_IO, the file is malformed) and no mesh is returned; the same
    file without that face loads."""
    head = "v 0 0 0\nv 1 0 0\nv 0 1 0\n"
    for bad in ("f 0 1 2", "f 1 2 4", "f -4 -2 -1", "f 1 2 3\nf 1 2 9"):
        p = tmp_path / "bad.obj"
        p.write_text(head + bad + "\n")
        rc, xyz, _ = load(p)
        assert rc == -5 and xyz is None, bad
    p = tmp_path / "ok.obj"
    p.write_text(head + "f -3 -2 -1\n")
    rc, xyz, _ = load(p)
    assert rc == 0 and xyz.shape == (1, 9)
    np.testing.assert_array_equal(xyz[0], [0, 0, 0, 1, 0, 0, 0, 1, 0])


def test_obj_long_lines_and_crlf(tmp_path):
    """A line longer than the 1024-byte read buffer is cut there and parsing continues with the next
    line (a deliberate difference: the reference's getline fails on it and stops reading the file,
    which would drop the face below), and CR LF line ends parse as LF."""
    p = tmp_path / "m.obj"
    p.write_text("v 0 0 0\r\nv 1 0 0\r\nv 0 1 0\r\n# " + "x" * 3000 + "\r\nf 1 2 3\r\n", newline="")
    rc, xyz, _ = load(p)
    assert rc == 0 and xyz.shape == (1, 9)
