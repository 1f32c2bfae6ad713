"""The C-ABI library loads without a GPU, exports every function declared in include/*.h, and the
ctypes binding lays out every struct of the header as the C compiler does."""
import ctypes
import glob
import os
import re

import pytest

from helpers import REPO

from crt_gb300 import lib

DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(crt_[a-z0-9_]+)\s*\(", re.M)


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(DECL.findall(src))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("crt_context_create", "crt_scene_create", "crt_trace_closest", "crt_trace_any", "crt_passes",
                 "crt_lidar_batch", "crt_lidar_grid", "crt_render", "crt_srp", "crt_mesh_load_obj"):
        assert must in names


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    L = ctypes.CDLL(lib.LIB_PATH)
    assert hasattr(L, name), f"{name} declared in include/ but not exported by libcrt_gpu.so"


def test_binding_covers_header():
    """Every declared entry point has a ctypes signature in crt_gb300.lib (used by the tests)."""
    assert set(declared_functions()) <= set(lib.SIGNATURES)


def test_abi_version_without_gpu():
    L = lib.load()
    assert L.crt_abi_version() == 3
    assert L.crt_status_string(-4) == b"timeout"


def test_context_create_reports_no_device_on_cpu_host():
    """On a host without a GPU the library refuses cleanly (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.load().crt_context_create(0, ctypes.byref(h))
    assert rc == -7 and not h.value


STRUCTS = {"EntityDesc": "crt_entity_desc", "CameraDesc": "crt_camera_desc", "LightDesc": "crt_light_desc",
           "RenderParams": "crt_render_params", "LidarGridDesc": "crt_lidar_grid_desc", "SrpDesc": "crt_srp_desc",
           "Request": "crt_request", "BatchStats": "crt_batch_stats", "Tuning": "crt_tuning",
           "ServerConfig": "crt_server_config", "ServerRequest": "crt_server_request",
           "ServerResult": "crt_server_result", "ServerStats": "crt_server_stats", "SceneStats": "crt_scene_stats",
           "Counters": "crt_counters"}
DTYPES = {"RAY_DTYPE": ("crt_ray", {"o": "o", "tmin": "tmin", "d": "d", "tmax": "tmax"}),
          "HIT_DTYPE": ("crt_hit", {"t": "t", "u": "u", "v": "v", "prim": "prim"})}


def test_struct_layouts_match_header(tmp_path):
    """The ctypes structures and numpy dtypes of the binding have the size and field offsets the C
    compiler gives the structs of include/crt_gpu.h (a mismatch would corrupt every request)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "crt_gpu.h"', "int main(void) {"]
    expect = {}
    for py, c in STRUCTS.items():
        cls = getattr(lib, py)
        lines.append(f'printf("{c} %zu\\n", sizeof({c}));')
        expect[c] = ctypes.sizeof(cls)
        for name, _ in cls._fields_:
            lines.append(f'printf("{c}.{name} %zu\\n", offsetof({c}, {name}));')
            expect[f"{c}.{name}"] = getattr(cls, name).offset
    for py, (c, fields) in DTYPES.items():
        dt = getattr(lib, py)
        lines.append(f'printf("{c} %zu\\n", sizeof({c}));')
        expect[c] = dt.itemsize
        for f_py, f_c in fields.items():
            lines.append(f'printf("{c}.{f_c} %zu\\n", offsetof({c}, {f_c}));')
            expect[f"{c}.{f_c}"] = dt.fields[f_py][1]
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                             text=True).stdout.splitlines())
    got = {k: int(v) for k, v in got.items()}
    assert got == expect
