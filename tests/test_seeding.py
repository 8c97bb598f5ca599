"""FluidSimulation::initialize's fluid seeding against the reference's own.

The fixtures tests/golden/initialize_*.npz were written by the reference's
FluidSimulation::initialize (fluidsimulation.cpp:48-55, 1383-1434), compiled
unchanged on the CPU, with the marker-particle jitter factor 0
(tests/golden/make_initialize_golden.py): the hello-world ball (one implicit
point) and a scene of two implicit points, a cuboid and added solid cells.
libgfs's host seeding (gfs_seed_fluid_particles, the seeding step of
gfs_sim_initialize) must give the same particle positions, bit for bit and in
the same creation order, on the CPU alone.
"""
import ctypes
import os

import numpy as np
import pytest

from gridfluidsim3d_gb300 import _lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    from gridfluidsim3d_gb300 import build
    build.build()
    return _lib.load()


def _seed(lib, f, jitter=0.0, seed=0):
    ni, nj, nk = (int(x) for x in f["grid"])
    mat = np.zeros((nk, nj, ni), np.uint8)
    for i, j, k in f["solids"]:
        mat[k, j, i] = 2
    pts = np.ascontiguousarray(f["points"], np.float64)
    cub = np.ascontiguousarray(f["cuboids"], np.float64)
    n = ctypes.c_int64(0)
    args = (ni, nj, nk, float(f["dx"]), mat.ctypes.data_as(ctypes.c_void_p), pts.ctypes.data_as(ctypes.c_void_p),
            len(pts), cub.ctypes.data_as(ctypes.c_void_p), len(cub), jitter, seed)
    lib.gfs_seed_fluid_particles(*args, None, 0, ctypes.byref(n))
    out = np.zeros((max(n.value, 1), 3), np.float32)
    lib.gfs_seed_fluid_particles(*args, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
    return out[:n.value]


@pytest.mark.parametrize("name", ["initialize_ball", "initialize_mixed"])
def test_seeding_matches_reference(lib, name):
    f = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    got = _seed(lib, f)
    want = f["positions"]
    assert got.shape == want.shape, (got.shape, want.shape)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_seeding_jitter_is_bounded_and_reproducible(lib):
    f = dict(np.load(os.path.join(GOLDEN, "initialize_mixed.npz")))
    a = _seed(lib, f, jitter=0.1, seed=7)
    b = _seed(lib, f, jitter=0.1, seed=7)
    c = _seed(lib, f, jitter=0.1, seed=8)
    want = f["positions"]
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.shape == want.shape
    j = 0.25 * 0.1 * float(f["dx"])
    assert np.abs(a - want).max() <= j * (1 + 1e-6)


def test_seeding_rejects_bad_input(lib):
    mat = np.zeros((8, 8, 8), np.uint8)
    bad = np.array([[0.4, 0.4, 0.4, -1.0]])
    n = ctypes.c_int64(0)
    with pytest.raises(_lib.GFSError):
        lib.gfs_seed_fluid_particles(8, 8, 8, 0.1, mat.ctypes.data_as(ctypes.c_void_p),
                                     bad.ctypes.data_as(ctypes.c_void_p), 1, None, 0, 0.0, 0, None, 0,
                                     ctypes.byref(n))
