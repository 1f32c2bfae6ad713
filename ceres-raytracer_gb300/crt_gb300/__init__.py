"""Helpers around the GB300 ray-query library: build recipe, raw C-ABI binding, synthetic scenes.

The user-facing drop-in API is the `crt` package next to this one (same classes and functions
as the reference's `crt`), backed by the `_crt` extension module.  This package holds what the
tests and the benchmark need in addition: `lib` (ctypes binding of every entry point declared in
include/crt_gpu.h), `scenes` (seeded synthetic scenes) and `build`.
"""
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_DIR = os.path.dirname(PKG_DIR)
