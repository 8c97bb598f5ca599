"""Savestates read into and written from the device-resident simulation
(gfs_sim_load_state / gfs_sim_save_state through the C ABI), checked against the
oracle's restatement of the FluidSimulationSaveState format and the fixture the
reference's own FluidSimulation wrote (tests/golden/savestate_ref.state).

Bars: the file's particles and solid cells arrive bit for bit (particles by id =
position in the file; cells holding particles become fluid, as after the
reference's load); a written file is byte-identical to the oracle's file of
the simulation's own state (particles in its (cell, id) order); load after save
reproduces the state; a substep after loading equals a substep after setting the
same arrays directly.
"""
import os

import numpy as np
import pytest

from gridfluidsim3d_gb300 import FluidSimulation, FluidSimulationSaveState, GFSError, scenes
from oracle import savestate as S

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FREF = os.path.join(HERE, "golden", "savestate_ref.state")


def _by_id(pos, vel, ids):
    o = np.argsort(ids)
    return pos[o], vel[o], ids[o]


def test_load_reference_fixture(gpu_ctx):
    ref = S.read_state(FREF)
    sim = FluidSimulation.from_save_state(FREF, ctx=gpu_ctx)
    assert (sim.isize, sim.jsize, sim.ksize, sim.dx) == (*ref["dims"], ref["dx"])
    assert sim.current_frame == ref["frame"]
    # the file's solid cells; cells holding particles are fluid, as the reference marks
    # them after loading (_initializeFluidMaterialParticlesFromSaveState)
    want = S.material_from_solid(ref["dims"], ref["solid_cells"])
    g = np.floor(ref["positions"].astype(np.float64) / ref["dx"]).astype(int)
    want[g[:, 2], g[:, 1], g[:, 0]] = 1
    assert np.array_equal(sim.get_material_grid(), want)
    pos, vel, ids = _by_id(*sim.get_marker_particles())
    assert np.array_equal(ids, np.arange(len(ref["positions"]), dtype=np.uint32))
    assert np.array_equal(pos, ref["positions"]) and np.array_equal(vel, ref["velocities"])


def test_save_matches_oracle_bytes(gpu_ctx, tmp_path):
    sc = scenes.random_box(dims=(20, 14, 17), seed=5)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    sim.update(sc.dt)
    out = str(tmp_path / "gpu.state")
    sim.save_state(out, current_frame=11)
    pos, vel, _ = sim.get_marker_particles()            # the device's (cell, id) order
    want = str(tmp_path / "oracle.state")
    S.write_state(want, sc.dims, sc.dx, 11, pos, vel, sim.get_material_grid())
    assert open(out, "rb").read() == open(want, "rb").read()
    st = FluidSimulationSaveState()
    st.load_state(out)
    assert st.get_num_marker_particles() == len(pos) and st.get_current_frame() == 11


def test_round_trip_and_step(gpu_ctx, tmp_path):
    sc = scenes.random_box(dims=(24, 18, 16), seed=8)
    a = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    a.set_material_grid(sc.mat)
    a.set_marker_particles(sc.pos, sc.vel)
    a.update(sc.dt)
    path = str(tmp_path / "rt.state")
    a.save_state(path, current_frame=3)
    pos, vel, _ = a.get_marker_particles()
    b = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    assert b.load_state(path) == 3
    # a savestate holds the solid cells; the others come back as air, or fluid where particles are
    ma, mb = a.get_material_grid(), b.get_material_grid()
    assert np.array_equal(mb == S.SOLID, ma == S.SOLID) and np.all(mb <= S.SOLID)
    bp, bv, bi = _by_id(*b.get_marker_particles())
    assert np.array_equal(bp, pos) and np.array_equal(bv, vel)
    # the loaded state steps exactly like the same arrays set directly
    c = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    c.set_material_grid(mb)
    c.set_marker_particles(pos, vel)
    b.update(sc.dt)
    c.update(sc.dt)
    for x, y in zip(_by_id(*b.get_marker_particles()), _by_id(*c.get_marker_particles())):
        assert np.array_equal(x, y)


def test_load_errors(gpu_ctx, tmp_path):
    sim = FluidSimulation(10, 10, 10, 0.25, max_particles=100, ctx=gpu_ctx)
    with pytest.raises(GFSError, match="does not match"):
        sim.load_state(FREF)                              # 12 x 10 x 9 file
    small = FluidSimulation(12, 10, 9, 0.25, max_particles=10, ctx=gpu_ctx)
    with pytest.raises(GFSError, match="capacity"):
        small.load_state(FREF)                            # 300 particles
    cut = tmp_path / "cut.state"
    cut.write_bytes(open(FREF, "rb").read()[:5000])
    ok = FluidSimulation(12, 10, 9, 0.25, max_particles=400, ctx=gpu_ctx)
    with pytest.raises(GFSError, match="truncated"):
        ok.load_state(str(cut))
    with pytest.raises(GFSError, match="cannot open"):
        ok.load_state(str(tmp_path / "missing.state"))
