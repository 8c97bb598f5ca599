"""The wavefront kernels of the MIC(0) triangular solves, and their bounded waits.

The triangular solves of PressureSolver::_applyPreconditioner
(pressuresolver.cpp:304-386) run as i+j+k hyperplane wavefronts over blocks of
16 x 16 pencils.  A context can run them with the block kernel (hand-overs
through L2 words) or with 4 x 2 / 2 x 2 thread-block clusters (hand-overs
inside a cluster through distributed shared memory).  The three compute the
same values in the same order, so on one system they must give bit-identical
pressures, in FP64 (PLAIN) and in FP32 (MIXED); each is also checked against
the oracle with the pressure bars (PLAIN: iterations +-1 and 1e-9 relative;
MIXED: FP64 residual below 1e-6 and 1e-5 relative to an FP64 solve to 1e-12).

The one-warp kernel (FP32 only) computes every cell with the same arithmetic
but sums the backward solve's dot product in its own order, so it is held to
the block kernel within FP32 rounding of that dot product (solves capped at 1
and 3 iterations, where a wrong preconditioner value would show at full size),
to the oracle bars, to the block kernel's iteration count +-1, and to
run-to-run bit identity; an FP64 solve asked to run it runs the block kernel.

The grid has 3 x 3 pencil blocks, so every kernel hands over across blocks, and
the clustered kernels both inside a cluster and between clusters; its 26 planes
in i give 56 wavefront steps, so the one-warp kernel's last bulk copy is partial.

The bounded waits: a test hook makes the next wavefront launches wait for an
exchange tag that no producer writes.  With a small wait limit every waiting
thread gives up at its bound, the solve fails with GFS_ERR_TIMEOUT, and the
next solve on the same context is correct again.  Nothing faults or hangs.
"""
import numpy as np
import pytest

from gridfluidsim3d_gb300 import (GFSError, MACVelocityField, PressureSolver, PressureSolverParameters,
                                  PRECISION_MIXED, PRECISION_PLAIN, SWEEP_AUTO, SWEEP_BLOCK, SWEEP_CLUSTER_2X2,
                                  SWEEP_CLUSTER_4X2, SWEEP_WARP, scenes)
from gridfluidsim3d_gb300._lib import GFS_ERR_TIMEOUT

pytestmark = pytest.mark.gpu

KERNELS = {"block": SWEEP_BLOCK, "cluster4x2": SWEEP_CLUSTER_4X2, "cluster2x2": SWEEP_CLUSTER_2X2}


def _system(O, dims=(26, 40, 44), seed=21):
    sc = scenes.random_box(dims=dims, seed=seed, fill=0.4)
    mat = sc.mat.copy()
    pos, vel, ids = sc.pos.copy(), sc.vel.copy(), sc.ids.copy()
    n = O.lib().gfo_update_fluid_cells(*sc.dims, sc.dx, mat, pos, vel, ids, len(pos))
    u, v, w = O.advect_velocity_field(sc.dims, sc.dx, mat, pos[:n], vel[:n])
    u, v, w = O.body_force(sc.dims, mat, np.array(sc.gravity, np.float32), sc.dt, u, v, w)
    return sc, mat, (u, v, w)


@pytest.fixture(scope="module")
def system(oracle_lib):
    O = oracle_lib
    sc, mat, (u, v, w) = _system(O)
    plain = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w)
    exact = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w, tol=1e-12, max_iters=4000)
    return sc, mat, (u, v, w), plain, exact


def _solve(ctx, sc, mat, uvw, precision, max_iterations=200):
    solver = PressureSolver(ctx, precision=precision, max_iterations=max_iterations)
    p = solver.solve(PressureSolverParameters(sc.dx, 20.0, sc.dt, mat, MACVelocityField(*sc.dims, sc.dx, *uvw)))
    return p, solver


@pytest.fixture
def kernel_ctx(gpu_ctx):
    yield gpu_ctx
    gpu_ctx.set_sweep_kernel(SWEEP_AUTO)
    gpu_ctx.set_wait_limit(0)
    gpu_ctx.inject_wait_timeout(0)


@pytest.mark.parametrize("precision", [PRECISION_PLAIN, PRECISION_MIXED], ids=["plain_fp64", "mixed_fp32"])
def test_kernels_match_oracle_and_each_other(kernel_ctx, oracle_lib, system, precision):
    O = oracle_lib
    sc, mat, uvw, (want, it_ref, _), (exact, _, _) = system
    results = {}
    for name, kind in KERNELS.items():
        kernel_ctx.set_sweep_kernel(kind)
        p, solver = _solve(kernel_ctx, sc, mat, uvw, precision)
        assert kernel_ctx.last_sweep_kernel() == kind, name
        results[name] = (p, solver.iterations)
        res = O.pressure_residual(sc.dims, sc.dx, 20.0, sc.dt, mat, *uvw, p)
        assert res < 1e-6, (name, res)
        if precision == PRECISION_PLAIN:
            assert abs(solver.iterations - it_ref) <= 1, (name, solver.iterations, it_ref)
            assert np.abs(p - want).max() / np.abs(want).max() < 1e-9, name
        else:
            assert np.abs(p - exact).max() / np.abs(exact).max() < 1e-5, name
    base_p, base_it = results["block"]
    for name, (p, it) in results.items():
        assert it == base_it, (name, it, base_it)
        assert np.array_equal(p, base_p), f"{name} differs from the block kernel"


def test_auto_runs_warp_for_fp32_and_block_for_fp64(kernel_ctx, system):
    sc, mat, uvw, _, _ = system
    kernel_ctx.set_sweep_kernel(SWEEP_AUTO)
    for precision, want in ((PRECISION_MIXED, SWEEP_WARP), (PRECISION_PLAIN, SWEEP_BLOCK)):
        _solve(kernel_ctx, sc, mat, uvw, precision)
        assert kernel_ctx.last_sweep_kernel() == want


def test_warp_kernel_against_block_kernel_and_oracle(kernel_ctx, oracle_lib, system):
    O = oracle_lib
    sc, mat, uvw, (want, it_ref, _), (exact, _, _) = system
    # capped solves: the preconditioner values are the block kernel's, the dot product differs in rounding
    for iters in (1, 3):
        kernel_ctx.set_sweep_kernel(SWEEP_BLOCK)
        pb, _ = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED, max_iterations=iters)
        kernel_ctx.set_sweep_kernel(SWEEP_WARP)
        pw, _ = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED, max_iterations=iters)
        assert kernel_ctx.last_sweep_kernel() == SWEEP_WARP
        assert np.abs(pb).max() > 0
        rel = np.abs(pw - pb).max() / np.abs(pb).max()
        assert rel < 1e-5, (iters, rel)
    # full solves
    kernel_ctx.set_sweep_kernel(SWEEP_BLOCK)
    pb, sb = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED)
    kernel_ctx.set_sweep_kernel(SWEEP_WARP)
    pw, sw = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED)
    pw2, sw2 = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED)
    assert np.array_equal(pw, pw2) and sw.iterations == sw2.iterations      # deterministic
    assert abs(sw.iterations - sb.iterations) <= 1, (sw.iterations, sb.iterations)
    assert O.pressure_residual(sc.dims, sc.dx, 20.0, sc.dt, mat, *uvw, pw) < 1e-6
    assert np.abs(pw - exact).max() / np.abs(exact).max() < 1e-5
    # FP64: the block kernel runs, bit for bit
    kernel_ctx.set_sweep_kernel(SWEEP_BLOCK)
    qb, tb = _solve(kernel_ctx, sc, mat, uvw, PRECISION_PLAIN)
    kernel_ctx.set_sweep_kernel(SWEEP_WARP)
    qw, tw = _solve(kernel_ctx, sc, mat, uvw, PRECISION_PLAIN)
    assert kernel_ctx.last_sweep_kernel() == SWEEP_BLOCK
    assert np.array_equal(qw, qb) and tw.iterations == tb.iterations


@pytest.mark.parametrize("dims", [(3, 40, 36), (5, 17, 33), (40, 18, 18)])
def test_warp_kernel_shapes(kernel_ctx, oracle_lib, dims):
    """The one-warp kernel on grids whose i extent is shorter than a copy group (3 and
    5 planes: 33 and 35 wavefront steps, the last copy group partial and the last
    progress check reaching past the end) or whose j / k extents leave partial pencil
    blocks: the MIXED bars against an FP64 solve to 1e-12."""
    O = oracle_lib
    sc, mat, uvw = _system(O, dims=dims, seed=4)
    exact, _, _ = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, *uvw, tol=1e-12, max_iters=4000)
    kernel_ctx.set_sweep_kernel(SWEEP_WARP)
    p, solver = _solve(kernel_ctx, sc, mat, uvw, PRECISION_MIXED)
    assert kernel_ctx.last_sweep_kernel() == SWEEP_WARP
    assert O.pressure_residual(sc.dims, sc.dx, 20.0, sc.dt, mat, *uvw, p) < 1e-6
    if np.abs(exact).max() > 0:
        assert np.abs(p - exact).max() / np.abs(exact).max() < 1e-5


def test_invalid_kernel_is_rejected(kernel_ctx):
    with pytest.raises(GFSError):
        kernel_ctx.set_sweep_kernel(7)
    with pytest.raises(GFSError):
        kernel_ctx.set_sweep_kernel(5)


@pytest.mark.parametrize("precision", [PRECISION_PLAIN, PRECISION_MIXED], ids=["plain_fp64", "mixed_fp32"])
@pytest.mark.parametrize("kernel", list(KERNELS) + ["warp"])
def test_wait_timeout_is_reported_and_the_context_recovers(kernel_ctx, oracle_lib, system, kernel, precision):
    O = oracle_lib
    sc, mat, uvw, (want, it_ref, _), (exact, _, _) = system
    kernel_ctx.set_sweep_kernel(dict(KERNELS, warp=SWEEP_WARP)[kernel])
    kernel_ctx.set_wait_limit(2000)
    # the build, forward and backward sweeps of the first iteration look for a tag nobody writes
    kernel_ctx.inject_wait_timeout(3)
    with pytest.raises(GFSError) as e:
        _solve(kernel_ctx, sc, mat, uvw, precision)
    assert e.value.code == GFS_ERR_TIMEOUT
    assert "wait" in str(e.value)
    # the next solve on the same context runs clean
    kernel_ctx.set_wait_limit(0)
    p, solver = _solve(kernel_ctx, sc, mat, uvw, precision)
    res = O.pressure_residual(sc.dims, sc.dx, 20.0, sc.dt, mat, *uvw, p)
    assert res < 1e-6
    if precision == PRECISION_PLAIN:
        assert abs(solver.iterations - it_ref) <= 1
        assert np.abs(p - want).max() / np.abs(want).max() < 1e-9
    else:
        assert np.abs(p - exact).max() / np.abs(exact).max() < 1e-5


def test_wait_timeout_inside_a_substep(kernel_ctx):
    """The same path through FluidSimulation.update, whose pressure workspace and
    exchange words persist across steps: the failed step raises, and a retry of
    the step gives the bit-identical state of a clean run."""
    from gridfluidsim3d_gb300 import FluidSimulation
    sc = scenes.random_box(dims=(22, 36, 40), seed=5)

    def make():
        sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=kernel_ctx)
        sim.precision = PRECISION_MIXED
        sim.set_material_grid(sc.mat)
        sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
        return sim

    clean = make()
    clean.update(sc.dt)
    clean.update(sc.dt)
    want = clean.get_marker_particles()
    sim = make()
    sim.update(sc.dt)
    kernel_ctx.set_wait_limit(2000)
    kernel_ctx.inject_wait_timeout(3)
    with pytest.raises(GFSError) as e:
        sim.update(sc.dt)
    assert e.value.code == GFS_ERR_TIMEOUT
    kernel_ctx.set_wait_limit(0)
    sim.update(sc.dt)
    got = sim.get_marker_particles()
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
