"""GPU: the reference's FluidSimulation C exports (include/gfs_fluidsimulation_c.h),
called the way pyfluid calls them (ctypes, trailing int *err, 1 = success; the
message from CBindings_get_error_message), run the device-resident substep.

The scene (body force, implicit fluid point, fluid cuboid, solid cells,
initialize, three updates) is also run through the Python FluidSimulation on the
same library: both paths must give the same particles bit for bit, and the
exports must answer the queries pyfluid makes (dimensions, density, frame,
particle ranges) and report misuse through err.
"""
import ctypes
from ctypes import byref, c_double, c_int, c_void_p

import numpy as np
import pytest

from gridfluidsim3d_gb300 import FluidSimulation, GridIndex, _lib

pytestmark = pytest.mark.gpu


class Vector3_t(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class AABB_t(ctypes.Structure):
    _fields_ = [("position", Vector3_t), ("width", ctypes.c_float), ("height", ctypes.c_float),
                ("depth", ctypes.c_float)]


class GridIndex_t(ctypes.Structure):
    _fields_ = [("i", c_int), ("j", c_int), ("k", c_int)]


class MarkerParticle_t(ctypes.Structure):
    _fields_ = [("position", Vector3_t), ("velocity", Vector3_t)]


DIMS, DX, DT = (24, 20, 22), 0.25, 1.0 / 30.0
POINT = (3.0, 2.5, 2.75, 1.4)
CUBOID = ((0.5, 0.25, 0.5), 5.0, 1.0, 4.5)
SOLIDS = [(10, 3, 10), (11, 3, 10), (10, 4, 11)]


def _api():
    lib = _lib.lib()
    sig = {
        "FluidSimulation_new_from_dimensions": ([c_int, c_int, c_int, c_double, c_void_p], c_void_p),
        "FluidSimulation_destroy": ([c_void_p], None),
        "FluidSimulation_initialize": ([c_void_p, c_void_p], None),
        "FluidSimulation_is_initialized": ([c_void_p, c_void_p], c_int),
        "FluidSimulation_update": ([c_void_p, c_double, c_void_p], None),
        "FluidSimulation_get_current_frame": ([c_void_p, c_void_p], c_int),
        "FluidSimulation_get_cell_size": ([c_void_p, c_void_p], c_double),
        "FluidSimulation_get_simulation_width": ([c_void_p, c_void_p], c_double),
        "FluidSimulation_get_density": ([c_void_p, c_void_p], c_double),
        "FluidSimulation_set_density": ([c_void_p, c_double, c_void_p], None),
        "FluidSimulation_add_body_force": ([c_void_p, c_double, c_double, c_double, c_void_p], None),
        "FluidSimulation_get_constant_body_force": ([c_void_p, c_void_p], Vector3_t),
        "FluidSimulation_add_implicit_fluid_point": ([c_void_p, c_double, c_double, c_double, c_double, c_void_p],
                                                     None),
        "FluidSimulation_add_fluid_cuboid": ([c_void_p, AABB_t, c_void_p], None),
        "FluidSimulation_add_solid_cells": ([c_void_p, c_void_p, c_int, c_void_p], None),
        "FluidSimulation_get_num_marker_particles": ([c_void_p, c_void_p], c_int),
        "FluidSimulation_get_marker_particles": ([c_void_p, c_int, c_int, c_void_p, c_void_p], None),
        "FluidSimulation_get_marker_particle_positions": ([c_void_p, c_int, c_int, c_void_p, c_void_p], None),
        "FluidSimulation_get_marker_particle_velocities": ([c_void_p, c_int, c_int, c_void_p, c_void_p], None),
        "CBindings_get_error_message": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes, f.restype = args, res
    return lib


def _call(lib, name, *args):
    """pyfluid's execute_lib_func: append &success, raise on failure."""
    err = c_int(-1)
    out = getattr(lib, name)(*args, byref(err))
    if err.value != 1:
        raise RuntimeError(name + " - " + lib.CBindings_get_error_message().decode())
    return out


def test_c_exports_run_the_core(gpu_ctx):
    lib = _api()
    obj = _call(lib, "FluidSimulation_new_from_dimensions", *DIMS, DX)
    try:
        assert _call(lib, "FluidSimulation_get_cell_size", obj) == DX
        assert _call(lib, "FluidSimulation_get_simulation_width", obj) == DIMS[0] * DX
        assert _call(lib, "FluidSimulation_get_density", obj) == 20.0
        f = _call(lib, "FluidSimulation_get_constant_body_force", obj)
        assert (f.x, f.y, f.z) == (0.0, 0.0, 0.0)                    # none until added
        _call(lib, "FluidSimulation_add_body_force", obj, 0.0, -25.0, 0.0)
        _call(lib, "FluidSimulation_add_implicit_fluid_point", obj, *POINT)
        (px, py, pz), w, h, d = CUBOID
        _call(lib, "FluidSimulation_add_fluid_cuboid", obj, AABB_t(Vector3_t(px, py, pz), w, h, d))
        cells = (GridIndex_t * len(SOLIDS))(*[GridIndex_t(*c) for c in SOLIDS])
        _call(lib, "FluidSimulation_add_solid_cells", obj, cells, len(SOLIDS))
        # update before initialize fails through err, as the reference's asserts would stop it
        with pytest.raises(RuntimeError, match="initialized"):
            _call(lib, "FluidSimulation_update", obj, DT)
        assert _call(lib, "FluidSimulation_is_initialized", obj) == 0
        _call(lib, "FluidSimulation_initialize", obj)
        assert _call(lib, "FluidSimulation_is_initialized", obj) == 1
        n0 = _call(lib, "FluidSimulation_get_num_marker_particles", obj)
        assert n0 > 1000
        for _ in range(3):
            _call(lib, "FluidSimulation_update", obj, DT)
        assert _call(lib, "FluidSimulation_get_current_frame", obj) == 3
        n = _call(lib, "FluidSimulation_get_num_marker_particles", obj)
        mps = (MarkerParticle_t * n)()
        _call(lib, "FluidSimulation_get_marker_particles", obj, 0, n, mps)
        c_pos = np.array([(m.position.x, m.position.y, m.position.z) for m in mps], np.float32)
        c_vel = np.array([(m.velocity.x, m.velocity.y, m.velocity.z) for m in mps], np.float32)
        part = (Vector3_t * 10)()
        _call(lib, "FluidSimulation_get_marker_particle_positions", obj, 5, 15, part)
        assert np.array_equal(np.array([(v.x, v.y, v.z) for v in part], np.float32), c_pos[5:15])
        _call(lib, "FluidSimulation_get_marker_particle_velocities", obj, n - 10, n, part)
        assert np.array_equal(np.array([(v.x, v.y, v.z) for v in part], np.float32), c_vel[n - 10:])
        with pytest.raises(RuntimeError, match="out of bounds"):
            _call(lib, "FluidSimulation_get_marker_particle_positions", obj, 0, n + 1, part)
        with pytest.raises(RuntimeError, match="density"):
            _call(lib, "FluidSimulation_set_density", obj, 0.0)
    finally:
        lib.FluidSimulation_destroy(obj)

    # the same scene through the Python FluidSimulation on the same library
    sim = FluidSimulation(*DIMS, DX, ctx=gpu_ctx)
    sim.reset_body_force()
    sim.add_body_force(0.0, -25.0, 0.0)
    sim.add_implicit_fluid_point(*POINT)
    sim.add_fluid_cuboid(*CUBOID[0], *CUBOID[1:])
    sim.add_solid_cells([GridIndex(*c) for c in SOLIDS])
    sim.initialize()
    assert sim.get_num_marker_particles() == n0
    for _ in range(3):
        sim.update(DT)
    pos, vel, _ = sim.get_marker_particles()
    sim.close()
    assert np.array_equal(pos, c_pos) and np.array_equal(vel, c_vel)
