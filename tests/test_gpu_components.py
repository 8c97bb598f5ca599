"""GPU parity of the individual hot-path components against the oracle.

Every comparison runs the CUDA path through libgfs's C ABI and the oracle (the
C restatement of the reference's CPU code) on the same seeded inputs.

Tolerances (the reference's stated bars):
  * splatted face velocities: relative 1e-5, with an absolute floor of 1e-6 of
    the scene's velocity scale for values that cancel towards zero;
  * tricubic samples: relative 1e-5, absolute floor 1e-6 of the field scale;
  * advected positions: 1e-5 of a cell;
  * pressure (PLAIN, FP64): CG iteration count equal within +-1, pressure
    relative 1e-9 (only the dot-product summation order differs);
  * pressure (MIXED): FP64 max-norm residual below the reference tolerance 1e-6.
  * general point splat (addPoints / addPointValues): relative 1e-5 with an
    absolute floor of 1e-6 of the output's scale; the touched node set equal.
"""
import numpy as np
import pytest

from gridfluidsim3d_gb300 import (CLScalarField, MACVelocityField, ParticleAdvector, PressureSolver,
                                  PressureSolverParameters, PRECISION_MIXED, PRECISION_PLAIN, SWEEP_AUTO,
                                  SWEEP_BLOCK, SWEEP_CLUSTER_2X2, SWEEP_CLUSTER_4X2, SWEEP_WARP, scenes)

pytestmark = pytest.mark.gpu

SWEEP_KERNELS = {"block": SWEEP_BLOCK, "cluster4x2": SWEEP_CLUSTER_4X2, "cluster2x2": SWEEP_CLUSTER_2X2,
                 "warp": SWEEP_WARP}


@pytest.fixture(params=list(SWEEP_KERNELS))
def sweep_ctx(request, gpu_ctx):
    """The context with each wavefront kernel of the MIC(0) triangular solves in turn
    (block kernel, 4 x 2 and 2 x 2 clusters, one-warp kernel: FP32 solves only, FP64
    solves asked for it run the block kernel); every pressure test runs on each."""
    gpu_ctx.set_sweep_kernel(SWEEP_KERNELS[request.param])
    yield gpu_ctx
    gpu_ctx.set_sweep_kernel(SWEEP_AUTO)


def _fluid_state(O, sc):
    """material after classification and the MAC field before the pressure solve."""
    mat = sc.mat.copy()
    pos, vel, ids = sc.pos.copy(), sc.vel.copy(), sc.ids.copy()
    n = O.lib().gfo_update_fluid_cells(*sc.dims, sc.dx, mat, pos, vel, ids, len(pos))
    u, v, w = O.advect_velocity_field(sc.dims, sc.dx, mat, pos[:n], vel[:n])
    u, v, w = O.body_force(sc.dims, mat, np.array(sc.gravity, np.float32), sc.dt, u, v, w)
    return mat, pos[:n], vel[:n], (u, v, w)


@pytest.mark.parametrize("seed,dims", [(0, (16, 12, 14)), (5, (24, 20, 17))])
def test_velocity_splat(gpu_ctx, oracle_lib, seed, dims):
    O = oracle_lib
    sc = scenes.random_box(dims=dims, seed=seed)
    acc = CLScalarField(gpu_ctx)
    vmax = float(np.abs(sc.vel).max())
    for d in range(3):
        g_field, g_set = acc.velocity_scalar_field(d, *sc.dims, sc.dx, sc.pos, sc.vel)
        o_field, o_set = O.velocity_scalar_field(d, sc.dims, sc.dx, sc.pos, sc.vel)
        assert np.array_equal(g_set, o_set.astype(bool)), f"is-set mask differs on component {d}"
        np.testing.assert_allclose(g_field, o_field, rtol=1e-5, atol=1e-6 * vmax)


def test_splat_empty_and_single(gpu_ctx, oracle_lib):
    O = oracle_lib
    acc = CLScalarField(gpu_ctx)
    dims, dx = (8, 7, 6), 0.5
    f, s = acc.velocity_scalar_field(1, *dims, dx, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    assert not s.any() and not f.any()
    pos = np.array([[1.3, 2.2, 0.9]], np.float32)
    vel = np.array([[0.5, -2.0, 3.0]], np.float32)
    for d in range(3):
        f, s = acc.velocity_scalar_field(d, *dims, dx, pos, vel)
        of, os_ = O.velocity_scalar_field(d, dims, dx, pos, vel)
        assert np.array_equal(s, os_.astype(bool))
        np.testing.assert_allclose(f, of, rtol=1e-6, atol=1e-7)


def _point_splat_gpu(acc, c):
    f = c["field"].copy()
    w = c["weight"].copy() if "weight" in c else None
    acc.set_max_scalar_field_value_threshold(c.get("threshold"))
    if "values" in c:
        acc.add_point_values(c["points"], c["values"], c["radius"], c["offset"], c["dx"], f, w)
    else:
        if w is None:
            acc.add_points(c["points"], c["radius"], c["offset"], c["dx"], f)
        else:
            # addPoints with a weight field: v = 1 for every point
            acc.add_point_values(c["points"], np.ones(len(c["points"]), np.float32), c["radius"], c["offset"],
                                 c["dx"], f, w)
    return f, w


def test_point_splat_matches_reference_fixture(gpu_ctx):
    from test_oracle_golden import point_splat_cases
    acc = CLScalarField(gpu_ctx)
    for c in point_splat_cases():
        f, w = _point_splat_gpu(acc, c)
        ref = c["out_field"]
        scale = max(float(np.abs(ref).max()), 1e-3)
        assert np.array_equal(f != c["field"], ref != c["field"]), "touched node set differs"
        np.testing.assert_allclose(f, ref, rtol=1e-5, atol=1e-6 * scale)
        if w is not None:
            np.testing.assert_allclose(w, c["out_weight"], rtol=1e-5, atol=1e-6 * max(float(c["out_weight"].max()), 1e-3))


@pytest.mark.parametrize("seed", [0, 1])
def test_point_splat_large(gpu_ctx, oracle_lib, seed):
    O = oracle_lib
    rng = np.random.default_rng(100 + seed)
    W, H, D = 40, 33, 29
    dx = 0.1
    acc = CLScalarField(gpu_ctx)
    acc.set_max_scalar_field_value_threshold(None)
    for rmul in (1.0, 2.5):
        n = 60000
        pts = rng.uniform(-0.2, 4.2, (n, 3)).astype(np.float32)
        vals = rng.normal(size=n).astype(np.float32)
        off = np.array([0.0, 0.05, 0.05], np.float32)
        f = np.zeros((D, H, W), np.float32)
        w = np.zeros_like(f)
        acc.add_point_values(pts, vals, rmul * dx, off, dx, f, w)
        of, ow = O.splat_points(pts, vals, rmul * dx, off, dx, np.zeros_like(f), np.zeros_like(f))
        assert np.array_equal(w > 0, ow > 0)
        np.testing.assert_allclose(w, ow, rtol=1e-5, atol=1e-6 * float(ow.max()))
        np.testing.assert_allclose(f, of, rtol=1e-5, atol=1e-5 * float(np.abs(of).max()))


def test_point_splat_edge_cases(gpu_ctx):
    acc = CLScalarField(gpu_ctx)
    f = np.full((4, 5, 6), 0.25, np.float32)
    acc.add_points(np.zeros((0, 3), np.float32), 0.3, (0, 0, 0), 0.1, f)
    assert (f == 0.25).all()
    # points far outside the grid reach nothing
    acc.add_points(np.array([[50.0, 50.0, 50.0], [-9.0, 0.1, 0.1]], np.float32), 0.3, (0, 0, 0), 0.1, f)
    assert (f == 0.25).all()
    with pytest.raises(Exception):
        acc.add_points(np.zeros((3, 3), np.float32), -1.0, (0, 0, 0), 0.1, f)
    acc.disable_opencl()
    with pytest.raises(Exception):
        acc.add_points(np.zeros((1, 3), np.float32), 0.3, (0, 0, 0), 0.1, f)


def _random_mac(dims, dx, seed):
    rng = np.random.default_rng(seed)
    ni, nj, nk = dims
    return MACVelocityField(ni, nj, nk, dx,
                            rng.normal(size=(nk, nj, ni + 1)).astype(np.float32),
                            rng.normal(size=(nk, nj + 1, ni)).astype(np.float32),
                            rng.normal(size=(nk + 1, nj, ni)).astype(np.float32))


def test_tricubic_interpolate(gpu_ctx, oracle_lib):
    O = oracle_lib
    dims, dx = (20, 16, 12), 0.125
    f = _random_mac(dims, dx, 3)
    rng = np.random.default_rng(4)
    ext = np.array(dims) * dx
    pts = (rng.random((5000, 3)) * ext * 1.1 - 0.05 * ext).astype(np.float32)   # some outside the grid
    got = ParticleAdvector(gpu_ctx).tricubic_interpolate(pts, f)
    want = O.evaluate_velocity(dims, dx, f.u, f.v, f.w, pts)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6 * 4.0)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_rk_advection(gpu_ctx, oracle_lib, order):
    O = oracle_lib
    dims, dx, dt = (20, 16, 12), 0.125, 1.0 / 30.0
    f = _random_mac(dims, dx, 7)
    rng = np.random.default_rng(8)
    pts = (rng.random((4000, 3)) * np.array(dims) * dx).astype(np.float32)
    adv = ParticleAdvector(gpu_ctx)
    got = getattr(adv, f"advect_particles_rk{order}")(pts, f, dt)
    if order == 4:
        want = O.advect_rk4(dims, dx, f.u, f.v, f.w, dt, pts)
        assert np.abs(got - want).max() / dx < 1e-5
    else:
        # lower orders: same sampler, reference formulas (particleadvector.cpp:1056-1078)
        k1 = O.evaluate_velocity(dims, dx, f.u, f.v, f.w, pts)
        if order == 1:
            want = pts + np.float32(dt) * k1
        elif order == 2:
            k2 = O.evaluate_velocity(dims, dx, f.u, f.v, f.w, pts + np.float32(0.5 * dt) * k1)
            want = pts + np.float32(dt) * k2
        else:
            k2 = O.evaluate_velocity(dims, dx, f.u, f.v, f.w, pts + np.float32(0.5 * dt) * k1)
            k3 = O.evaluate_velocity(dims, dx, f.u, f.v, f.w, pts + np.float32(0.75 * dt) * k2)
            want = pts + np.float32(dt / 9.0) * (2 * k1 + 3 * k2 + 4 * k3)
        assert np.abs(got - want).max() / dx < 1e-5


@pytest.mark.parametrize("seed,dims", [(0, (16, 12, 14)), (2, (30, 22, 26))])
def test_pressure_plain_matches_oracle(sweep_ctx, oracle_lib, seed, dims):
    O = oracle_lib
    sc = scenes.random_box(dims=dims, seed=seed)
    mat, pos, vel, (u, v, w) = _fluid_state(O, sc)
    want, it_ref, res_ref = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w)
    solver = PressureSolver(sweep_ctx, precision=PRECISION_PLAIN)
    got = solver.solve(PressureSolverParameters(sc.dx, 20.0, sc.dt, mat,
                                                MACVelocityField(*sc.dims, sc.dx, u, v, w)))
    assert abs(solver.iterations - it_ref) <= 1, (solver.iterations, it_ref)
    rel = np.abs(got - want).max() / max(np.abs(want).max(), 1e-30)
    assert rel < 1e-9, rel
    assert solver.max_residual < 1e-6 or it_ref == 200


def _sparse_fluid(dims, seed):
    """Material with fluid in separate regions (a slab, a ball, a small box), so that
    most 16x16 pencil blocks of the pressure solver's layout hold no fluid."""
    ni, nj, nk = dims
    mat = scenes.solid_border(dims)
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    fluid = j < 9
    fluid |= (i - ni / 2) ** 2 + (j - 40) ** 2 + (k - 38) ** 2 < 7.5 ** 2
    fluid |= (j >= 50) & (j < 55) & (k >= 3) & (k < 9) & (i >= 4) & (i < 12)
    mat[fluid & (mat != 2)] = 1
    return mat, _random_mac(dims, 0.1, seed)


@pytest.mark.parametrize("precision", [PRECISION_PLAIN, PRECISION_MIXED])
def test_pressure_blocks_without_fluid(sweep_ctx, oracle_lib, precision):
    O = oracle_lib
    dims = (24, 60, 50)
    mat, f = _sparse_fluid(dims, 11)
    dt = 1.0 / 30.0
    want, it_ref, _ = O.pressure_solve(dims, 0.1, 20.0, dt, mat, f.u, f.v, f.w)
    solver = PressureSolver(sweep_ctx, precision=precision)
    got = solver.solve(PressureSolverParameters(0.1, 20.0, dt, mat, f))
    if precision == PRECISION_PLAIN:
        assert abs(solver.iterations - it_ref) <= 1, (solver.iterations, it_ref)
        assert np.abs(got - want).max() / np.abs(want).max() < 1e-9
    res = O.pressure_residual(dims, 0.1, 20.0, dt, mat, f.u, f.v, f.w, got)
    assert res < 1e-6 or it_ref == 200, res


def test_pressure_mixed_reaches_tolerance(sweep_ctx, oracle_lib):
    O = oracle_lib
    sc = scenes.random_box(dims=(30, 22, 26), seed=2)
    mat, pos, vel, (u, v, w) = _fluid_state(O, sc)
    want, it_ref, _ = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w, tol=1e-12, max_iters=2000)
    solver = PressureSolver(sweep_ctx, precision=PRECISION_MIXED)
    got = solver.solve(PressureSolverParameters(sc.dx, 20.0, sc.dt, mat,
                                                MACVelocityField(*sc.dims, sc.dx, u, v, w)))
    assert solver.max_residual < 1e-6
    res = O.pressure_residual(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w, got)
    assert res < 1e-6, res
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-5


def test_pressure_no_fluid_and_quiet(sweep_ctx, oracle_lib):
    dims, dx = (10, 9, 8), 0.25
    mat = scenes.solid_border(dims)
    f = MACVelocityField(*dims, dx)
    solver = PressureSolver(sweep_ctx)
    p = solver.solve(PressureSolverParameters(dx, 20.0, 1 / 30., mat, f))
    assert p.size == 0
    mat[3:6, 3:6, 3:6] = 1
    p = solver.solve(PressureSolverParameters(dx, 20.0, 1 / 30., mat, f))
    assert p.shape == (27,) and not p.any() and solver.iterations == -1
