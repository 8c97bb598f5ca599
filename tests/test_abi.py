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
