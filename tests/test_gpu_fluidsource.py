"""Fluid sources and the fluid-cell queues on the device
(gfs_sim_set_fluid_sources, gfs_sim_add_fluid_cells, gfs_sim_remove_fluid_cells,
gfs_sim_update_fluid_sources and the first stage of gfs_sim_step, through the C
ABI) against the reference's results (tests/golden/fluidsource_ref.state and
fluidcells_ref.state, jitter factor 0) and the oracle's restatement (with
jitter, same counter-based hash).

Bars: with jitter 0 the particle set equals the reference's bit for bit; with
jitter the particles equal the oracle's by id, bit for bit; a substep with
sources matches the oracle's sources followed by the oracle's substep (positions
within 1e-5 of a cell, velocities within 1e-4 of the scene's scale, as the
substep tests); exceeding the capacity fails with GFS_ERR_INVALID.
"""
import json
import os

import numpy as np
import pytest

from gridfluidsim3d_gb300 import CuboidFluidSource, FluidSimulation, GFSError, SphericalFluidSource
from oracle import fluidsource as F
from oracle import savestate as S

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIN = os.path.join(G, "fluidsource_in.state")


def sources():
    out = []
    for s in json.load(open(os.path.join(G, "fluidsource_sources.json"))):
        if s["shape"] == "sphere":
            src = SphericalFluidSource(s["position"], s["radius"], s["velocity"])
        else:
            src = CuboidFluidSource(s["position"], *s["size"], velocity=s["velocity"])
        src.is_inflow = not s.get("outflow", False)
        src.is_active = s.get("active", True)
        out.append(src)
    return out


def with_sources(sim):
    for src in sources():
        if isinstance(src, SphericalFluidSource):
            sim.add_spherical_fluid_source(src)
        else:
            sim.add_cuboid_fluid_source(src)


def oracle_case():
    inp = S.read_state(FIN)
    mat = S.material_from_solid(inp["dims"], inp["solid_cells"])
    g = np.floor(inp["positions"].astype(np.float64) / inp["dx"]).astype(int)
    mat[g[:, 2], g[:, 1], g[:, 0]] = F.FLUID
    return inp, mat, json.load(open(os.path.join(G, "fluidsource_sources.json")))


def rows(p, v):
    return np.sort(np.concatenate([p, v], 1).astype(np.float32).view([("", np.float32)] * 6).ravel())


def by_id(pos, vel, ids):
    o = np.argsort(ids)
    return pos[o], vel[o], ids[o]


def test_sources_match_reference(gpu_ctx):
    ref = S.read_state(os.path.join(G, "fluidsource_ref.state"))
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.0)
    with_sources(sim)
    added, removed = sim.update_fluid_sources()
    pos, vel, ids = sim.get_marker_particles()
    assert len(pos) == len(ref["positions"]) == 4480 + added - removed
    assert np.array_equal(rows(pos, vel), rows(ref["positions"], ref["velocities"]))
    assert len(np.unique(ids)) == len(ids)


def test_jittered_sources_match_oracle(gpu_ctx):
    inp, mat, srcs = oracle_case()
    _, op, ov, oi, _ = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                             np.arange(len(inp["positions"])), srcs, jitter_factor=0.1, seed=11)
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.1, seed=11)
    with_sources(sim)
    sim.update_fluid_sources()
    gp, gv, gi = by_id(*sim.get_marker_particles())
    op, ov, oi = by_id(op, ov, oi)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gp, op) and np.array_equal(gv, ov)


def test_substep_with_sources(gpu_ctx, oracle_lib):
    inp, mat, srcs = oracle_case()
    dt, grav = 1.0 / 30.0, (0.0, -25.0, 0.0)
    _, op, ov, oi, _ = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                             np.arange(len(inp["positions"])), srcs, jitter_factor=0.1, seed=3)
    # the oracle's substep classifies cells from the particles itself
    base = S.material_from_solid(inp["dims"], inp["solid_cells"])
    st = oracle_lib.substep(inp["dims"], inp["dx"], dt, grav, base, op, ov, oi)
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.1, seed=3)
    sim.reset_body_force()
    sim.add_body_force(grav)
    with_sources(sim)
    stats = sim.update(dt)
    gp, gv, gi = by_id(*sim.get_marker_particles())
    rp, rv, ri = by_id(st["pos"], st["vel"], st["ids"])
    assert np.array_equal(gi, ri)
    assert abs(stats["cg_iterations"] - st["cg_iterations"]) <= 1
    assert np.abs(gp - rp).max() / inp["dx"] < 1e-5
    assert np.abs(gv - rv).max() / max(np.abs(rv).max(), 1.0) < 1e-4


def test_edge_sources_match_reference(gpu_ctx):
    """Sources across the grid's faces (clamped bounds, radius 0 and -1, an outflow
    over the pool's edge) against the reference's result, jitter 0."""
    ref = S.read_state(os.path.join(G, "fluidsource_edge_ref.state"))
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.0)
    for s in json.load(open(os.path.join(G, "fluidsource_edge_sources.json"))):
        if s["shape"] == "sphere":
            src = SphericalFluidSource(s["position"], s["radius"], s["velocity"])
            src.is_inflow = not s.get("outflow", False)
            sim.add_spherical_fluid_source(src)
        else:
            src = CuboidFluidSource(s["position"], *s["size"], velocity=s["velocity"])
            src.is_inflow = not s.get("outflow", False)
            sim.add_cuboid_fluid_source(src)
    added, removed = sim.update_fluid_sources()
    pos, vel, _ = sim.get_marker_particles()
    assert len(pos) == len(ref["positions"]) == 4480 + added - removed
    assert np.array_equal(rows(pos, vel), rows(ref["positions"], ref["velocities"]))


def test_capacity_error(gpu_ctx):
    sim = FluidSimulation.from_save_state(FIN, max_particles=4600, ctx=gpu_ctx)
    with_sources(sim)
    with pytest.raises(GFSError, match="capacity"):
        sim.update_fluid_sources()


def test_new_ids_follow_caller_ids(gpu_ctx):
    inp, mat, srcs = oracle_case()
    n = len(inp["positions"])
    ids = (np.arange(n, dtype=np.uint32) * 3 + 1000)   # caller ids, largest 1000 + 3 (n - 1)
    sim = FluidSimulation(*inp["dims"], inp["dx"], max_particles=8000, ctx=gpu_ctx)
    sim.set_material_grid(S.material_from_solid(inp["dims"], inp["solid_cells"]))
    sim.set_marker_particles(inp["positions"], inp["velocities"], ids)
    with_sources(sim)
    added, removed = sim.update_fluid_sources()
    _, _, got = sim.get_marker_particles()
    new = np.setdiff1d(got, ids)
    assert len(new) == added > 0
    assert new.min() == int(ids.max()) + 1 and new.max() == int(ids.max()) + added


def with_queues(sim):
    q = json.load(open(os.path.join(G, "fluidcells_queues.json")))
    for grp in q["added"]:
        if grp["velocity"] is None:
            sim.add_fluid_cells(grp["cells"])
        else:
            sim.add_fluid_cells(grp["cells"], *grp["velocity"])
    sim.remove_fluid_cells(q["removed"])


def oracle_queues(inp, mat, jitter, seed):
    """The oracle's queues then sources on the fixture input; (mat, pos, vel, ids)."""
    dims, dx = inp["dims"], inp["dx"]
    q = json.load(open(os.path.join(G, "fluidcells_queues.json")))
    added = [(F.add_fluid_cells_filter(dims, mat, grp["cells"]), grp["velocity"] or [0.0, 0.0, 0.0])
             for grp in q["added"]]
    srcs = json.load(open(os.path.join(G, "fluidsource_sources.json")))
    m, p, v, i, nid = F.update_fluid_cell_queues(dims, dx, mat, inp["positions"], inp["velocities"],
                                                 np.arange(len(inp["positions"])), added, q["removed"],
                                                 jitter_factor=jitter, seed=seed)
    m, p, v, i, _ = F.update_fluid_sources(dims, dx, m, p, v, i, srcs, jitter_factor=jitter, seed=seed, next_id=nid)
    return m, p, v, i


def test_fluid_cell_queues_match_reference(gpu_ctx):
    """addFluidCells / removeFluidCells, then the sources, against the reference's
    _updateFluidCells on the same state (tests/golden/fluidcells_ref.state)."""
    ref = S.read_state(os.path.join(G, "fluidcells_ref.state"))
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.0)
    with_sources(sim)
    with_queues(sim)
    added, removed = sim.update_fluid_sources()
    pos, vel, ids = sim.get_marker_particles()
    assert len(pos) == len(ref["positions"]) == 4480 + added - removed
    assert np.array_equal(rows(pos, vel), rows(ref["positions"], ref["velocities"]))
    assert len(np.unique(ids)) == len(ids)
    # the queues are consumed: without the sources a second pass changes nothing
    sim.remove_fluid_sources()
    assert sim.update_fluid_sources() == (0, 0)


def test_jittered_queues_match_oracle(gpu_ctx):
    inp, mat, _ = oracle_case()
    _, op, ov, oi = oracle_queues(inp, mat, 0.1, 23)
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.1, seed=23)
    with_sources(sim)
    with_queues(sim)
    sim.update_fluid_sources()
    gp, gv, gi = by_id(*sim.get_marker_particles())
    op, ov, oi = by_id(op, ov, oi)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gp, op) and np.array_equal(gv, ov)


def test_substep_with_queues(gpu_ctx, oracle_lib):
    """The queues applied by update(dt) at the start of the substep."""
    inp, mat, _ = oracle_case()
    dt, grav = 1.0 / 30.0, (0.0, -25.0, 0.0)
    _, op, ov, oi = oracle_queues(inp, mat, 0.1, 9)
    base = S.material_from_solid(inp["dims"], inp["solid_cells"])
    st = oracle_lib.substep(inp["dims"], inp["dx"], dt, grav, base, op, ov, oi)
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    sim.set_marker_particle_jitter(0.1, seed=9)
    sim.reset_body_force()
    sim.add_body_force(grav)
    with_sources(sim)
    with_queues(sim)
    stats = sim.update(dt)
    gp, gv, gi = by_id(*sim.get_marker_particles())
    rp, rv, ri = by_id(st["pos"], st["vel"], st["ids"])
    assert np.array_equal(gi, ri)
    assert abs(stats["cg_iterations"] - st["cg_iterations"]) <= 1
    assert np.abs(gp - rp).max() / inp["dx"] < 1e-5
    assert np.abs(gv - rv).max() / max(np.abs(rv).max(), 1.0) < 1e-4


def test_fluid_cell_out_of_range(gpu_ctx):
    sim = FluidSimulation.from_save_state(FIN, max_particles=8000, ctx=gpu_ctx)
    with pytest.raises(GFSError, match="out of range"):
        sim.add_fluid_cells([[3, 6, 4], [16, 0, 0]])
    with pytest.raises(GFSError, match="out of range"):
        sim.remove_fluid_cells([[-1, 2, 2]])
    assert sim.update_fluid_sources() == (0, 0)     # nothing was queued
