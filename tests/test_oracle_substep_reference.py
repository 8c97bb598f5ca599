"""The oracle's substep stages against the reference's own substep, bit for bit.

The fixtures tests/golden/substep_*.npz were written by the reference itself:
fluidsimulation.cpp and the reference's PressureSolver compiled unchanged on the
CPU, with the OpenCL classes replaced by CPU backends that run the reference's
OpenCL-disabled arithmetic (tests/golden/make_substep_golden.py).  Each test
feeds one stage of the oracle (oracle/gfs_oracle.c) the reference's input of that
stage and requires the reference's output exactly:

  stage 1   _updateFluidCells                 fluidsimulation.cpp:1990-2041
  stage 5   _advectVelocityField (splat + the 26-neighbour fill, U tests a
            nonzero value, V/W the is-set flag)          :2526-2736
            _savedVelocityField + extrapolation           :3306-3307
  stage 6   _applyBodyForcesToVelocityField               :2766-2805
  stage 7   _updatePressureGrid (PressureSolver::solve)   :2870-2889
  stage 8   _applyPressureToVelocityField (ghost pressures next to solids) :2895-3061
  stage 9   _extrapolateFluidVelocities                   :3067
  stage 11  _updateMarkerParticleVelocities (PIC/FLIP)    :3104-3129
  stage 12  _advanceRangeOfMarkerParticles (RK4 + collisions) :3145-3209
  cap       _removeMarkerParticles: per-cell counts min(n, 100) :3221-3243
            (which particles survive is the reference's rand() shuffle; the
            oracle keeps the smallest ids, a documented deviation)
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["substep_pool", "substep_sparse", "substep_crowd"]
RATIO_PIC = float(np.float32(0.05))   # _ratioPICFLIP = 0.05f held in a double (fluidsimulation.h:1161)
LAYERS = 7                            # ceil(CFL 5 + 2) (fluidsimulation.cpp:3067-3070)


def _load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def _mac(f, tag):
    return f[f"{tag}_u"], f[f"{tag}_v"], f[f"{tag}_w"]


def _same(got, want, what):
    for g, w, c in zip(got, want, "uvw"):
        assert g.shape == w.shape, (what, c)
        bad = np.flatnonzero(g.view(np.uint32) != w.view(np.uint32))
        assert bad.size == 0, f"{what} {c}: {bad.size} faces differ (first {bad[:5]})"


@pytest.fixture(params=SCENES)
def fx(request, oracle_lib):
    return _load(request.param)


def _stage1(O, f):
    dims = tuple(int(x) for x in f["dims"])
    mat = f["mat_in"].copy()
    pos, vel = f["pos_in"].copy(), f["vel_in"].copy()
    ids = np.arange(len(pos), dtype=np.uint32)
    n = O.lib().gfo_update_fluid_cells(*dims, float(f["dx"]), mat, pos, vel, ids, len(pos))
    return dims, mat, pos[:n], vel[:n], ids[:n]


def test_stage1_update_fluid_cells(fx, oracle_lib):
    dims, mat, pos, vel, ids = _stage1(oracle_lib, fx)
    assert np.array_equal(mat, fx["mat1"])
    assert int((mat == 1).sum()) == int(fx["num_fluid_cells"])
    assert np.array_equal(pos, fx["pos1"])


def test_stage5_advect_velocity_field_and_saved(fx, oracle_lib):
    O = oracle_lib
    dims, mat, pos, vel, _ = _stage1(O, fx)
    adv = O.advect_velocity_field(dims, float(fx["dx"]), mat, pos, vel)
    _same(adv, _mac(fx, "advected"), "advected field")
    _same(O.extrapolate(dims, fx["mat1"], LAYERS, *_mac(fx, "advected")), _mac(fx, "saved"), "saved field")


def test_stage6_body_force(fx, oracle_lib):
    dims = tuple(int(x) for x in fx["dims"])
    got = oracle_lib.body_force(dims, fx["mat1"], fx["gravity"], float(fx["dt"]), *_mac(fx, "advected"))
    _same(got, _mac(fx, "body"), "field after body force")


def test_stage7_pressure(fx, oracle_lib):
    O = oracle_lib
    dims = tuple(int(x) for x in fx["dims"])
    p, it, _ = O.pressure_solve(dims, float(fx["dx"]), 20.0, float(fx["dt"]), fx["mat1"], *_mac(fx, "body"))
    assert it > 0, "the scene must exercise the PCG loop"
    got = O.pressure_to_grid(dims, fx["mat1"], p)
    assert np.array_equal(got.view(np.uint32), fx["pressure"].view(np.uint32))


def test_stage8_apply_pressure(fx, oracle_lib):
    dims = tuple(int(x) for x in fx["dims"])
    got = oracle_lib.apply_pressure(dims, float(fx["dx"]), 20.0, float(fx["dt"]), fx["mat1"], fx["pressure"],
                                    *_mac(fx, "body"))
    _same(got, _mac(fx, "applied"), "field after apply-pressure")


def test_stage9_extrapolate(fx, oracle_lib):
    dims = tuple(int(x) for x in fx["dims"])
    _same(oracle_lib.extrapolate(dims, fx["mat1"], LAYERS, *_mac(fx, "applied")), _mac(fx, "extrap"),
          "extrapolated field")


def test_stage11_pic_flip(fx, oracle_lib):
    O = oracle_lib
    dims, mat, pos, vel, _ = _stage1(O, fx)
    got = O.flip_update(dims, float(fx["dx"]), RATIO_PIC, _mac(fx, "extrap"), _mac(fx, "saved"), pos, vel)
    assert np.array_equal(got.view(np.uint32), fx["vel11"].view(np.uint32))


def test_stage12_advance_with_collisions(fx, oracle_lib):
    O = oracle_lib
    dims, mat, pos, vel, _ = _stage1(O, fx)
    dx, dt = float(fx["dx"]), float(fx["dt"])
    p1 = O.advect_rk4(dims, dx, *_mac(fx, "extrap"), dt, pos)
    got = O.resolve_collisions(dims, dx, fx["mat1"], pos, p1)
    assert np.array_equal(got.view(np.uint32), fx["pos12"].view(np.uint32))


def test_cap_counts(fx, oracle_lib):
    O = oracle_lib
    dims = tuple(int(x) for x in fx["dims"])
    dx = float(fx["dx"])
    pos = fx["pos12"].copy()
    vel = fx["vel11"].copy()
    ids = np.arange(len(pos), dtype=np.uint32)
    n = O.lib().gfo_cap_particles_per_cell(*dims, dx, int(fx["max_per_cell"]), pos, vel, ids, len(pos))
    cells = np.floor(pos[:n].astype(np.float64) / dx).astype(np.int64)
    counts = np.zeros(fx["cap_counts"].shape, np.int32)
    np.add.at(counts, (cells[:, 2], cells[:, 1], cells[:, 0]), 1)
    assert np.array_equal(counts, fx["cap_counts"])


def test_crowd_scene_crowds_cells():
    f = _load("substep_crowd")
    assert f["cap_counts"].max() == 100
    assert len(f["pos12"]) - int(f["cap_counts"].sum()) == 38    # 37 + 1 + 0 above the cap


def test_sparse_scene_exercises_the_fill_asymmetry(oracle_lib):
    """Faces bordering fluid without splat weight take the 26-neighbour fill, and
    for every one of them the U rule (nonzero neighbours) and the V / W rule (set
    neighbours) would give different values: the fixture tells the two apart."""
    O = oracle_lib
    f = _load("substep_sparse")
    dims = tuple(int(x) for x in f["dims"])
    for d, c in enumerate("uvw"):
        field, mask = O.velocity_scalar_field(d, dims, float(f["dx"]), f["pos1"], f["vel_in"])
        filled = (mask == 0) & (f[f"advected_{c}"] != 0)
        assert filled.sum() >= 5, c
        assert ((mask == 1) & (field == 0)).sum() > 100, c


def test_pool_scene_reaches_every_stage():
    f = _load("substep_pool")
    # gravity changed V only, the pressure solve did work, and particles moved
    adv_u, body_u = f["advected_u"], f["body_u"]
    assert np.array_equal(adv_u, body_u)          # gravity is along y only
    assert not np.array_equal(f["advected_v"], f["body_v"])
    assert np.abs(f["pressure"]).max() > 0
    assert np.abs(f["pos12"] - f["pos1"]).max() > 0.1 * float(f["dx"])
