"""crt_srp_static: the allocation-free radiation-pressure entry point, through the C ABI.

Some callers cannot allocate device memory while they run: an attitude or orbit propagator that
evaluates radiation pressure at every integration step under a fixed memory budget, or a component
embedded in a host application that owns the CUDA allocator.  crt_srp_static gives them the force
and torque of crt_srp from the same wavefront stages, with all scratch in a static 64 MiB device
array.  These tests check, on two calls in a row, that its results equal crt_srp's bit for bit (the
same additions in the same order) and that the second call changes the device's free memory by
nothing; they cover waves of whole attitudes, attitudes spread over several waves, attitude tables
uploaded in several chunks, and host and device outputs and quaternions.
"""
import ctypes

import numpy as np
import pytest

from crt_gb300 import lib, scenes

pytestmark = pytest.mark.gpu

CRT_ERR_INVALID = -1


@pytest.fixture(scope="module")
def craft():
    ctx = lib.Context(0)
    sc = ctx.scene(scenes.spacecraft(bus_cell=0.25, panel_cell=0.2, dish_rings=16, dish_segments=16))
    yield ctx, sc
    ctx.close()


def desc(grid, nb=2):
    d = lib.SrpDesc()
    d.sun_dir_inertial[:] = [0.3, -0.2, 0.93]
    d.flux, d.c = 1361.0, 299792458.0
    d.center_of_mass[:] = [0.05, 0.1, -0.2]
    d.grid, d.num_bounces = grid, nb
    return d


def ptr(a):
    return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data


def reference(ctx, sc, d, q):
    n = len(q)
    f, t = np.empty((n, 3)), np.empty((n, 3))
    ctx._check(ctx.L.crt_srp(sc.h, ctypes.byref(d), q.ctypes.data, n, f.ctypes.data, t.ctypes.data, None))
    return f, t


# grid 384: 147,456 items per attitude, 7 attitudes per wave of 2^20 items (100 attitudes: 15 waves of
# whole attitudes, tables uploaded in 2 chunks); grid 512: 4 attitudes per wave; grid 2048: 4 Mi items
# per attitude, four waves each (running totals across waves)
@pytest.mark.parametrize("grid,n_att,where", [(384, 100, "host"), (2048, 3, "host"), (2048, 3, "device"),
                                              (512, 70, "mixed")])
def test_static_scratch_equals_allocating_entry_point(craft, grid, n_att, where):
    import torch
    ctx, sc = craft
    d = desc(grid)
    q = scenes.random_quaternions(n_att, seed=31 + grid)
    f_ref, t_ref = reference(ctx, sc, d, q)
    assert np.abs(f_ref).max() > 0
    free = []
    for call in range(2):
        if where == "host":
            qin, f, t = q, np.full((n_att, 3), np.nan), np.full((n_att, 3), np.nan)
        elif where == "device":
            qin = torch.from_numpy(q).cuda()
            f = torch.full((n_att, 3), float("nan"), dtype=torch.float64, device="cuda")
            t = torch.full((n_att, 3), float("nan"), dtype=torch.float64, device="cuda")
        else:   # device force, host torque, host quaternions
            qin = q
            f = torch.full((n_att, 3), float("nan"), dtype=torch.float64, device="cuda")
            t = np.full((n_att, 3), np.nan)
        torch.cuda.synchronize()
        ctx._check(ctx.L.crt_srp_static(sc.h, ctypes.byref(d), ptr(qin), n_att, ptr(f), ptr(t)))
        ctx.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        f_np = f.cpu().numpy() if hasattr(f, "cpu") else f
        t_np = t.cpu().numpy() if hasattr(t, "cpu") else t
        np.testing.assert_array_equal(f_np, f_ref, err_msg=f"force, call {call}")
        np.testing.assert_array_equal(t_np, t_ref, err_msg=f"torque, call {call}")
    assert free[0] == free[1]


def test_static_limits_are_refused(craft):
    ctx, sc = craft
    q = scenes.random_quaternions(4097, seed=3)
    f, t = np.empty((4097, 3)), np.empty((4097, 3))
    rc = ctx.L.crt_srp_static(sc.h, ctypes.byref(desc(64)), q.ctypes.data, 4097, f.ctypes.data, t.ctypes.data)
    assert rc == CRT_ERR_INVALID and b"static scratch" in ctx.L.crt_context_last_error(ctx.h)
    rc = ctx.L.crt_srp_static(sc.h, ctypes.byref(desc(32769)), q.ctypes.data, 1, f.ctypes.data, t.ctypes.data)
    assert rc == CRT_ERR_INVALID
    # a zero quaternion is refused before any launch
    q0 = np.zeros((1, 4))
    rc = ctx.L.crt_srp_static(sc.h, ctypes.byref(desc(64)), q0.ctypes.data, 1, f.ctypes.data, t.ctypes.data)
    assert rc == CRT_ERR_INVALID
