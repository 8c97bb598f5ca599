"""The device substep, stage by stage, against the reference's own substep.

The fixtures tests/golden/substep_*.npz hold the state after every stage of one
substep of the reference's FluidSimulation, run on the CPU with fluidsimulation.cpp
and its PressureSolver compiled unchanged (tests/golden/make_substep_golden.py;
the oracle reproduces them bit for bit, tests/test_oracle_substep_reference.py).
Here the device runs the same substep from the same particles through the C ABI
(gfs_sim_step_stages), stopping after each stage:

  stage 1   classification (k_classify)                    equal
  stage 6   splat + 26-neighbour fill + body force (k_splat_gather, k_face_fill),
            saved field + extrapolation                    1e-5 relative
  stage 7   pressure grid (PLAIN, FP64)                    1e-5 of max|p|
  stage 8   apply-pressure (k_apply_pressure)              1e-5 relative
  stage 9   extrapolation                                  1e-5 relative
  stage 12  PIC/FLIP + RK4 + collisions (k_g2p_advect)     positions 1e-5 cell,
            velocities 1e-4 of the scene's scale;
            the per-cell cap (k_cap_counts, k_cap_copy)    per-cell counts equal
            to the reference's, and the survivors the smallest ids of each
            crowded cell (the documented deviation from the reference's rand()
            shuffle)

The relative bars carry an absolute floor of 1e-6 of the field's scale: the
device sums the splat in float in a different order than the reference.
"""
import os

import numpy as np
import pytest

from gridfluidsim3d_gb300 import (FluidSimulation, PRECISION_PLAIN, STAGE_APPLY_PRESSURE, STAGE_BODY_FORCES,
                                  STAGE_EXTRAPOLATE, STAGE_PRESSURE, STAGE_UPDATE_FLUID_CELLS)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["substep_pool", "substep_sparse", "substep_crowd"]


def _load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def _close(got, want, what, rtol=1e-5):
    scale = max(float(np.abs(want).max()), 1e-3)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=1e-6 * scale, err_msg=what)


def _fields(f, tag):
    return f[f"{tag}_u"], f[f"{tag}_v"], f[f"{tag}_w"]


@pytest.fixture(params=SCENES)
def run(request, gpu_ctx):
    f = _load(request.param)
    dims = tuple(int(x) for x in f["dims"])
    sim = FluidSimulation(*dims, float(f["dx"]), max_particles=len(f["pos_in"]), ctx=gpu_ctx)
    sim.precision = PRECISION_PLAIN
    sim.set_material_grid(f["mat_in"])
    sim.set_marker_particles(f["pos_in"], f["vel_in"], np.arange(len(f["pos_in"]), dtype=np.uint32))
    yield request.param, f, sim
    sim.close()


def test_stages_match_the_reference(run):
    name, f, sim = run
    dt = float(f["dt"])
    st = sim.step_stages(dt, STAGE_UPDATE_FLUID_CELLS)
    assert np.array_equal(sim.get_material_grid(), f["mat1"]), "classification"
    assert st["num_fluid_cells"] == int(f["num_fluid_cells"])

    sim.step_stages(dt, STAGE_BODY_FORCES)
    g = sim.get_velocity_field()
    for got, want, c in zip((g.u, g.v, g.w), _fields(f, "body"), "uvw"):
        _close(got, want, f"{name}: field after the splat, fill and body force ({c})")
    s = sim.get_saved_velocity_field()
    for got, want, c in zip((s.u, s.v, s.w), _fields(f, "saved"), "uvw"):
        _close(got, want, f"{name}: saved field ({c})")

    sim.step_stages(dt, STAGE_PRESSURE)
    p = sim.get_pressure_grid()
    want = f["pressure"]
    assert np.abs(p - want).max() <= 1e-5 * np.abs(want).max(), f"{name}: pressure"

    sim.step_stages(dt, STAGE_APPLY_PRESSURE)
    g = sim.get_velocity_field()
    for got, want, c in zip((g.u, g.v, g.w), _fields(f, "applied"), "uvw"):
        _close(got, want, f"{name}: field after apply-pressure ({c})")

    sim.step_stages(dt, STAGE_EXTRAPOLATE)
    g = sim.get_velocity_field()
    for got, want, c in zip((g.u, g.v, g.w), _fields(f, "extrap"), "uvw"):
        _close(got, want, f"{name}: extrapolated field ({c})")


def test_whole_substep_matches_the_reference(run, oracle_lib):
    name, f, sim = run
    dx, dt = float(f["dx"]), float(f["dt"])
    dims = tuple(int(x) for x in f["dims"])
    sim.update(dt)
    pos, vel, ids = sim.get_marker_particles()
    # survivors: the reference's per-cell counts, and the smallest ids of each cell
    cells = np.floor(pos.astype(np.float64) / dx).astype(np.int64)
    counts = np.zeros(f["cap_counts"].shape, np.int32)
    np.add.at(counts, (cells[:, 2], cells[:, 1], cells[:, 0]), 1)
    assert np.array_equal(counts, f["cap_counts"]), f"{name}: per-cell counts after the cap"
    ref_pos, ref_vel = f["pos12"], f["vel11"]
    want_ids = np.arange(len(ref_pos), dtype=np.uint32)   # compacted in place to the survivors
    kept = oracle_lib.lib().gfo_cap_particles_per_cell(*dims, dx, int(f["max_per_cell"]), ref_pos.copy(),
                                                       ref_vel.copy(), want_ids, len(ref_pos))
    assert np.array_equal(np.sort(ids), np.sort(want_ids[:kept])), f"{name}: surviving particles"
    err = np.abs(pos - ref_pos[ids]).max() / dx
    assert err < 1e-5, (name, err)
    vscale = max(float(np.abs(ref_vel).max()), 1e-3)
    assert np.abs(vel - ref_vel[ids]).max() < 1e-4 * vscale, name
