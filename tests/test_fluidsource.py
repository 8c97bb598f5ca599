"""Fluid sources (FluidSimulation::_updateFluidSources, fluidsimulation.cpp:1717-1879)
on the CPU: the oracle's restatement against the result the reference's own
code produced on the same state and sources (tests/golden/make_fluidsource_golden.py,
jitter factor 0), and the jittered form's invariants.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import fluidsource as F  # noqa: E402
from oracle import savestate as S  # noqa: E402

G = os.path.join(HERE, "golden")


def load_case():
    inp = S.read_state(os.path.join(G, "fluidsource_in.state"))
    ref = S.read_state(os.path.join(G, "fluidsource_ref.state"))
    srcs = json.load(open(os.path.join(G, "fluidsource_sources.json")))
    dims, dx = inp["dims"], inp["dx"]
    mat = S.material_from_solid(dims, inp["solid_cells"])
    g = np.floor(inp["positions"].astype(np.float64) / dx).astype(int)
    # fluid where particles are, as the reference marks them after loading
    # (_initializeFluidMaterialParticlesFromSaveState, fluidsimulation.cpp:1466)
    mat[g[:, 2], g[:, 1], g[:, 0]] = F.FLUID
    return inp, ref, srcs, mat


def rows(p, v):
    return np.sort(np.concatenate([p, v], 1).astype(np.float32).view([("", np.float32)] * 6).ravel())


def test_oracle_matches_reference_sources():
    inp, ref, srcs, mat = load_case()
    _, p, v, ids, nid = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                              np.arange(len(inp["positions"])), srcs, jitter_factor=0.0)
    assert len(p) == len(ref["positions"]) == 5382
    assert np.array_equal(rows(p, v), rows(ref["positions"], ref["velocities"]))
    assert len(np.unique(ids)) == len(ids)


def test_jittered_particles_stay_in_their_sub_cells():
    inp, _, srcs, mat = load_case()
    n0 = len(inp["positions"])
    _, p0, _, i0, _ = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                            np.arange(n0), srcs, jitter_factor=0.0)
    _, p1, v1, i1, _ = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                             np.arange(n0), srcs, jitter_factor=0.1, seed=5)
    assert np.array_equal(i0, i1)
    new = i1 >= n0
    d = np.abs(p1[new].astype(np.float64) - p0[new])
    # the default factor 0.1: |jitter| <= 0.025 dx, well inside a sub-cell (half-width 0.25 dx),
    # so the same sub-cells are filled and the ids match
    jmax = 0.25 * 0.1 * inp["dx"]
    assert d.max() <= jmax * (1 + 1e-6) and d.max() > 0.5 * jmax
    assert np.array_equal(p1[~new], p0[~new])


def queue_case(mat, dims):
    """The queued groups of tests/golden/fluidcells_queues.json, filtered as
    addFluidCells filters them when called."""
    q = json.load(open(os.path.join(G, "fluidcells_queues.json")))
    added = [(F.add_fluid_cells_filter(dims, mat, grp["cells"]), grp["velocity"] or [0.0, 0.0, 0.0])
             for grp in q["added"]]
    return added, q["removed"]


def test_oracle_matches_reference_fluid_cell_queues():
    """The queues, then the sources, as the reference's _updateFluidCells
    (fluidsimulation.cpp:1990-1994) ran them."""
    inp, _, srcs, mat = load_case()
    ref = S.read_state(os.path.join(G, "fluidcells_ref.state"))
    dims, dx = inp["dims"], inp["dx"]
    added, removed = queue_case(mat, dims)
    assert [len(c) for c, _ in added] == [5, 3]      # (2,2,2) is fluid and (0,5,5) solid: not queued
    m, p, v, ids, nid = F.update_fluid_cell_queues(dims, dx, mat, inp["positions"], inp["velocities"],
                                                   np.arange(len(inp["positions"])), added, removed,
                                                   jitter_factor=0.0)
    _, p, v, ids, _ = F.update_fluid_sources(dims, dx, m, p, v, ids, srcs, jitter_factor=0.0, next_id=nid)
    assert len(p) == len(ref["positions"]) == 5394
    assert np.array_equal(rows(p, v), rows(ref["positions"], ref["velocities"]))
    assert len(np.unique(ids)) == len(ids)


def test_fluid_cell_index_out_of_range():
    inp, _, _, mat = load_case()
    try:
        F.add_fluid_cells_filter(inp["dims"], mat, [[1, 1, 1], [16, 0, 0]])
    except IndexError:
        return
    raise AssertionError("out-of-range cell accepted")


def test_cell_lists_for_the_queues():
    """FluidSimulation.add_fluid_cells / remove_fluid_cells take pyfluid
    GridIndex objects or (i, j, k) rows; both become int32 triples."""
    from gridfluidsim3d_gb300 import FluidSimulation, GridIndex
    g = [GridIndex(1, 2, 3), GridIndex(GridIndex(4, 5, 6))]
    a = FluidSimulation._cells(g)
    b = FluidSimulation._cells([(1, 2, 3), [4, 5, 6]])
    c = FluidSimulation._cells(np.array([[1, 2, 3], [4, 5, 6]], np.int64))
    for x in (a, b, c):
        assert x.dtype == np.int32 and x.flags.c_contiguous
        assert x.tolist() == [[1, 2, 3], [4, 5, 6]]
    assert FluidSimulation._cells([]).shape == (0, 3)
    assert list(g[1]) == [4, 5, 6] and g[1][2] == 6 and g[0] == GridIndex(1, 2, 3)


def test_oracle_matches_reference_edge_sources():
    """Sources across the grid's faces (tests/golden/fluidsource_edge_sources.json):
    the clamping of fitAABBtoGrid / getGridIndexBounds, radius 0 and -1, and an
    outflow over the pool's edge, against the reference's _updateFluidSources."""
    inp, _, _, mat = load_case()
    ref = S.read_state(os.path.join(G, "fluidsource_edge_ref.state"))
    srcs = json.load(open(os.path.join(G, "fluidsource_edge_sources.json")))
    _, p, v, ids, _ = F.update_fluid_sources(inp["dims"], inp["dx"], mat, inp["positions"], inp["velocities"],
                                            np.arange(len(inp["positions"])), srcs, jitter_factor=0.0)
    assert len(p) == len(ref["positions"]) == 3699
    assert np.array_equal(rows(p, v), rows(ref["positions"], ref["velocities"]))
