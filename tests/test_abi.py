"""The C ABI on the CPU: libgfs.so builds for sm_103a, loads, and exports every
entry point include/gfs.h declares; host-only calls behave (no GPU needed)."""
import ctypes
import os
import re
import shutil

import pytest

from gridfluidsim3d_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gfs.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s*(gfs_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no CUDA toolkit")
    from gridfluidsim3d_gb300 import build
    build.build()
    return _lib.load()


def test_header_and_binding_agree():
    assert _declared() == sorted(_lib.EXPORTS)


def test_every_declared_symbol_is_exported(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_host_only_calls(lib):
    assert lib.gfs_version().decode().startswith("gfs-gb300")
    p = _lib.SimParams()
    lib.gfs_sim_default_params(ctypes.byref(p))
    assert p.density == 20.0 and p.max_cg_iterations == 200 and abs(p.ratio_pic - 0.05) < 1e-8
    assert p.tol == 1e-6 and p.max_particles_per_cell == 100 and tuple(p.gravity) == (0.0, -25.0, 0.0)


def test_errors_are_reported_not_raised(lib):
    # a NULL out-pointer is rejected with a message, whatever the device situation
    with pytest.raises(_lib.GFSError) as e:
        lib.gfs_ctx_create(0, None)
    assert "NULL" in str(e.value)
    with pytest.raises(_lib.GFSError):
        lib.gfs_sim_default_params(None)


def test_fluid_cell_queue_arguments(lib):
    # gfs_sim_add_fluid_cells / gfs_sim_remove_fluid_cells validate before any device work
    cells = (ctypes.c_int32 * 3)(1, 2, 3)
    with pytest.raises(_lib.GFSError) as e:
        lib.gfs_sim_add_fluid_cells(None, cells, 1, None)
    assert "invalid arguments" in str(e.value)
    with pytest.raises(_lib.GFSError):
        lib.gfs_sim_remove_fluid_cells(None, cells, 1)
    with pytest.raises(_lib.GFSError):
        lib.gfs_sim_update_fluid_sources(None, None, None)


def test_noalloc_rejects_overflowing_dims_before_any_device_work(lib):
    # dims whose padded extents would overflow int are rejected before the grids
    # are formed; dummy non-NULL pointers are never dereferenced on this path
    dummy = ctypes.c_void_p(16)
    big = 2 ** 31 - 4
    for dims in ((big, big, 1), (1, big, 1), (70000, 70000, 1)):
        with pytest.raises(_lib.GFSError) as e:
            lib.gfs_tricubic_interpolate_noalloc(*dims, 0.1, dummy, dummy, dummy, dummy, 1, dummy, None)
        assert e.value.code == _lib.GFS_ERR_INVALID
        assert "too large" in str(e.value) or "scratch" in str(e.value)


# ---- the reference's FluidSimulation C exports (include/gfs_fluidsimulation_c.h)

FSIM_HEADER = os.path.join(ROOT, "include", "gfs_fluidsimulation_c.h")


def _fsim_declared():
    src = open(FSIM_HEADER).read()
    return sorted(set(re.findall(r"\b((?:FluidSimulation|CBindings)_\w+)\s*\(", src)))


def test_fluidsimulation_exports(lib):
    names = _fsim_declared()
    assert "FluidSimulation_update" in names and "CBindings_get_error_message" in names
    for name in names:
        assert hasattr(lib, name), name


def test_fluidsimulation_exports_host_only(lib):
    """The reference's error convention (int *err: 1 success, 0 failure, message
    from CBindings_get_error_message) on calls that need no GPU."""
    c_int, c_double, c_void_p, byref = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.byref
    lib.CBindings_get_error_message.restype = ctypes.c_char_p
    lib.FluidSimulation_new_from_empty.restype = c_void_p
    lib.FluidSimulation_new_from_empty.argtypes = [c_void_p]
    err = c_int(-1)
    obj = lib.FluidSimulation_new_from_empty(byref(err))
    assert err.value == 1 and obj
    i, j, k = c_int(7), c_int(7), c_int(7)
    lib.FluidSimulation_get_grid_dimensions.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.FluidSimulation_get_grid_dimensions(obj, byref(i), byref(j), byref(k), byref(err))
    assert err.value == 1 and (i.value, j.value, k.value) == (0, 0, 0)
    # an empty simulation has no grid to step
    lib.FluidSimulation_update.argtypes = [c_void_p, c_double, c_void_p]
    lib.FluidSimulation_update(obj, 0.01, byref(err))
    assert err.value == 0 and b"no grid" in lib.CBindings_get_error_message()
    lib.FluidSimulation_destroy.argtypes = [c_void_p]
    lib.FluidSimulation_destroy(obj)
    # bad dimensions are refused before any device work
    lib.FluidSimulation_new_from_dimensions.restype = c_void_p
    lib.FluidSimulation_new_from_dimensions.argtypes = [c_int, c_int, c_int, c_double, c_void_p]
    assert not lib.FluidSimulation_new_from_dimensions(0, 8, 8, 0.1, byref(err))
    assert err.value == 0 and b"positive" in lib.CBindings_get_error_message()
