"""The C-ABI library loads without a GPU and exports every function declared in include/*.h."""
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
    assert L.crt_abi_version() == 2
    assert L.crt_status_string(-4) == b"timeout"


def test_context_create_reports_no_device_on_cpu_host():
    """On a host without a GPU the library refuses cleanly (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.load().crt_context_create(0, ctypes.byref(h))
    assert rc == -7 and not h.value
