"""FluidSimulation.initialize on the device-resident simulation.

The scene set-up API of the reference (addImplicitFluidPoint, addFluidCuboid,
addSolidCells, initialize; fluidsimulation.cpp:48-55, 703-765, 845-861,
1383-1434) through the Python FluidSimulation and gfs_sim_initialize: with the
jitter factor 0 the resident particles, taken in id (= creation) order, are the
reference's own initialize() output bit for bit (tests/golden/initialize_*.npz),
and the material grid -- solid border, added solid cells, fluid where particles
are -- is the reference's.  A step then runs from that state.
"""
import os

import numpy as np
import pytest

from gridfluidsim3d_gb300 import FluidSimulation, GridIndex

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["initialize_ball", "initialize_mixed"])
def test_initialize_matches_reference(gpu_ctx, name):
    f = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    ni, nj, nk = (int(x) for x in f["grid"])
    sim = FluidSimulation(ni, nj, nk, float(f["dx"]), ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.0)
    for x, y, z, r in f["points"]:
        sim.add_implicit_fluid_point(x, y, z, r)
    for x, y, z, w, h, d in f["cuboids"]:
        sim.add_fluid_cuboid(x, y, z, w, h, d)
    sim.add_solid_cells([GridIndex(*c) for c in f["solids"]])
    sim.initialize()
    assert sim.is_initialized()
    pos, vel, ids = sim.get_marker_particles()
    o = np.argsort(ids)
    assert np.array_equal(ids[o], np.arange(len(f["positions"]), dtype=np.uint32))
    assert np.array_equal(pos[o].view(np.uint32), f["positions"].view(np.uint32))
    assert not vel.any()
    assert np.array_equal(sim.get_material_grid(), f["material"])
    st = sim.update(1.0 / 30.0)
    assert st["num_particles"] == len(f["positions"])
    sim.close()
