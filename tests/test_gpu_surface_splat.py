"""The isotropic surface splat of the simulation's resident marker particles.

gfs_sim_add_marker_particle_points is CLScalarField::addPoints
(clscalarfield.cpp:68-122) of the marker positions that IsotropicParticleMesher
splats inside every substep (isotropicparticlemesher.cpp:309-390), taken
straight from the device-resident particle state.  It must give exactly what the
host-array entry point gives on the same positions, and agree with the oracle's
restatement of ScalarField::addPoint (scalarfield.cpp:121-166; pinned bit for bit
to the reference by tests/golden/point_splat.npz) to 1e-5 relative, with the
same set of touched nodes.
"""
import numpy as np
import pytest

from gridfluidsim3d_gb300 import CLScalarField, FluidSimulation, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("threshold", [None, 1.0])
def test_resident_splat_matches_host_splat_and_oracle(gpu_ctx, oracle_lib, threshold):
    sc = scenes.random_box(dims=(20, 16, 18), seed=6)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    sim.update(sc.dt)
    ni, nj, nk = sc.dims
    dx = sc.dx
    # the mesher's field: (n+1)^3 nodes at dx, radius 3 x the marker-particle radius
    r = (3 * dx ** 3 / 8.0 / (4 * 3.141592653)) ** (1.0 / 3.0) * 3.0
    base = np.full((nk + 1, nj + 1, ni + 1), 0.25, np.float32)   # adds into what is there
    got = base.copy()
    sim.add_marker_particle_points(r, (0.0, 0.0, 0.0), dx, got, threshold=threshold)
    pos, _, _ = sim.get_marker_particles()
    host = base.copy()
    acc = CLScalarField(gpu_ctx)
    acc.set_max_scalar_field_value_threshold(threshold)
    acc.add_points(pos, r, (0.0, 0.0, 0.0), dx, host)
    assert np.array_equal(got, host)
    want, _ = oracle_lib.splat_points(pos, None, r, (0.0, 0.0, 0.0), dx, base, threshold=threshold)
    assert np.array_equal(got != base, want != base), "touched nodes differ"
    scale = float(np.abs(want).max())
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6 * scale)
    sim.close()


def test_resident_splat_without_particles(gpu_ctx):
    sim = FluidSimulation(8, 8, 8, 0.1, max_particles=1, ctx=gpu_ctx)
    f = np.ones((9, 9, 9), np.float32)
    sim.add_marker_particle_points(0.2, (0.0, 0.0, 0.0), 0.1, f)
    assert (f == 1.0).all()
    sim.close()
