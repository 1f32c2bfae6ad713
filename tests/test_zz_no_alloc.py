"""crt_srp_static: the allocation-free radiation-pressure entry point, through the C ABI.

Some callers cannot allocate device memory while they run: an attitude or orbit propagator that
evaluates radiation pressure every integration step under a fixed memory budget, or a component
embedded in a host application that owns the CUDA allocator.  crt_srp_static gives them the same
force and torque as crt_srp with all scratch in a static 16 MiB device array.  This test checks, on
two calls in a row, that its results equal crt_srp's within the radiation-pressure tolerance
(1e-4 relative) and that the second call changes the device's free memory by nothing.
"""
import ctypes

import numpy as np
import pytest

from crt_gb300 import lib, scenes

pytestmark = pytest.mark.gpu


def test_static_scratch_matches_allocating_entry_point():
    import torch
    ctx = lib.Context(0)
    try:
        sc = ctx.scene(scenes.spacecraft(bus_cell=0.25, panel_cell=0.2, dish_rings=16, dish_segments=16))
        q = scenes.random_quaternions(5, seed=31)
        d = lib.SrpDesc()
        d.sun_dir_inertial[:] = [0.3, -0.2, 0.93]
        d.flux, d.c = 1361.0, 299792458.0
        d.center_of_mass[:] = [0.05, 0.1, -0.2]
        d.grid, d.num_bounces = 512, 2
        f_ref, t_ref = np.empty((5, 3)), np.empty((5, 3))
        ctx._check(ctx.L.crt_srp(sc.h, ctypes.byref(d), q.ctypes.data, 5, f_ref.ctypes.data, t_ref.ctypes.data, None))
        free = []
        for call in range(2):
            f, t = np.full((5, 3), np.nan), np.full((5, 3), np.nan)
            ctx._check(ctx.L.crt_srp_static(sc.h, ctypes.byref(d), q.ctypes.data, 5, f.ctypes.data, t.ctypes.data))
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
            for a in range(5):
                assert np.linalg.norm(f[a] - f_ref[a]) <= 1e-4 * np.linalg.norm(f_ref[a]), (call, a)
                assert np.linalg.norm(t[a] - t_ref[a]) <= 1e-4 * max(np.linalg.norm(t_ref[a]),
                                                                    1e-3 * np.linalg.norm(f_ref[a])), (call, a)
        assert free[0] == free[1]
        # sizes beyond the static scratch are refused with a clear error
        d.grid = 20000
        rc = ctx.L.crt_srp_static(sc.h, ctypes.byref(d), q.ctypes.data, 5, f.ctypes.data, t.ctypes.data)
        assert rc == -1 and b"static scratch" in ctx.L.crt_context_last_error(ctx.h)
    finally:
        ctx.close()
