"""GPU parity of the whole FLIP substep against the oracle's substep.

The device-resident substep (gfs_sim_step through the C ABI) and the oracle's
restatement of FluidSimulation::_stepFluid stages 1, 5-9, 11, 12 start from the
same seeded scene.  Particles are matched by id (the device keeps them in
(cell, id) order; the reference shuffles them every substep).

Bars: identical fluid-cell classification and particle count; CG iteration
count within +-1; advected positions within 1e-5 of a cell per substep
(checked after one substep, and with a per-substep budget over three);
velocities within 1e-4 relative to the scene's velocity scale.
"""
import numpy as np
import pytest

from gridfluidsim3d_gb300 import FluidSimulation, scenes

pytestmark = pytest.mark.gpu


def _by_id(pos, vel, ids):
    o = np.argsort(ids)
    return pos[o], vel[o], ids[o]


def _run(gpu_ctx, O, sc, steps):
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    st = dict(mat=sc.mat, pos=sc.pos, vel=sc.vel, ids=sc.ids)
    out = []
    for _ in range(steps):
        gstats = sim.update(sc.dt)
        st = O.substep(sc.dims, sc.dx, sc.dt, sc.gravity, st["mat"], st["pos"], st["vel"], st["ids"])
        gpos, gvel, gids = _by_id(*sim.get_marker_particles())
        opos, ovel, oids = _by_id(st["pos"], st["vel"], st["ids"])
        out.append((gstats, st, (gpos, gvel, gids), (opos, ovel, oids), sim.get_material_grid(),
                    sim.get_velocity_field()))
    return out


@pytest.mark.parametrize("name,kw", [("random_box", dict(dims=(16, 12, 14), seed=0)),
                                     ("random_box", dict(dims=(28, 24, 20), seed=3)),
                                     ("ball_drop", dict(n=32, dx=0.25))])
def test_one_substep(gpu_ctx, oracle_lib, name, kw):
    O = oracle_lib
    sc = scenes.SCENES[name](**kw)
    (gstats, st, g, o, gmat, gfield), = _run(gpu_ctx, O, sc, 1)
    assert np.array_equal(gmat, st["mat"]), "fluid classification differs"
    assert gstats["num_fluid_cells"] == st["num_fluid_cells"]
    assert np.array_equal(g[2], o[2]), "particle sets differ"
    assert abs(gstats["cg_iterations"] - st["cg_iterations"]) <= 1
    err = np.abs(g[0] - o[0]).max() / sc.dx
    assert err < 1e-5, err
    vscale = max(float(np.abs(o[1]).max()), 1e-3)
    np.testing.assert_allclose(g[1], o[1], rtol=1e-4, atol=1e-4 * vscale)
    for a, b in ((gfield.u, st["u"]), (gfield.v, st["v"]), (gfield.w, st["w"])):
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-4 * max(float(np.abs(b).max()), 1e-3))


def test_three_substeps(gpu_ctx, oracle_lib):
    """Three substeps in a row with the single-substep bars: the device runs free
    and the oracle restarts from the device's particles before each substep."""
    O = oracle_lib
    sc = scenes.random_box(dims=(20, 18, 16), seed=11)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    for step in range(1, 4):
        pos, vel, ids = sim.get_marker_particles()
        gstats = sim.update(sc.dt)
        st = O.substep(sc.dims, sc.dx, sc.dt, sc.gravity, sc.mat, pos, vel, ids)
        g = _by_id(*sim.get_marker_particles())
        o = _by_id(st["pos"], st["vel"], st["ids"])
        assert np.array_equal(g[2], o[2]), step
        assert np.array_equal(sim.get_material_grid(), st["mat"]), step
        assert abs(gstats["cg_iterations"] - st["cg_iterations"]) <= 1, step
        err = np.abs(g[0] - o[0]).max() / sc.dx
        assert err < 1e-5, (step, err)
        vscale = max(float(np.abs(o[1]).max()), 1e-3)
        np.testing.assert_allclose(g[1], o[1], rtol=1e-4, atol=1e-4 * vscale)
    sim.close()


def test_deterministic(gpu_ctx):
    sc = scenes.random_box(dims=(20, 18, 16), seed=4)
    runs = []
    for _ in range(2):
        sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
        sim.set_material_grid(sc.mat)
        sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
        for _ in range(2):
            sim.update(sc.dt)
        runs.append(sim.get_marker_particles())
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b), "two runs of the same input differ"


def test_host_step_matches_device_step(gpu_ctx):
    sc = scenes.random_box(dims=(16, 12, 14), seed=1)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    sim.update(sc.dt)
    dpos, dvel, dids = sim.get_marker_particles()
    sim2 = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim2.set_material_grid(sc.mat)
    pos, vel, ids = sc.pos.copy(), sc.vel.copy(), sc.ids.copy()
    n, _ = sim2.update_host(sc.dt, pos, vel, ids)
    assert n == len(dids)
    assert np.array_equal(ids[:n], dids) and np.array_equal(pos[:n], dpos) and np.array_equal(vel[:n], dvel)


@pytest.mark.parametrize("layout", ["all_pinned", "mixed"])
def test_host_step_with_pinned_buffers(gpu_ctx, layout):
    """update_host with page-locked (mapped) host buffers: the pack / unpack kernels
    read and write them in place instead of a staged copy; two steps, each handing
    the previous one's output back, give the device path's particles bit for bit,
    with every buffer pinned and with pinned positions beside pageable velocities
    and ids."""
    torch = pytest.importorskip("torch")
    sc = scenes.random_box(dims=(16, 12, 14), seed=3)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    for _ in range(2):
        sim.update(sc.dt)
    dpos, dvel, dids = sim.get_marker_particles()

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
        v = t.numpy().view(a.dtype)
        v[:] = a
        return t, v

    keep = []
    tp, pos = pinned(sc.pos)
    keep.append(tp)
    if layout == "all_pinned":
        tv, vel = pinned(sc.vel)
        ti, ids = pinned(sc.ids)
        keep += [tv, ti]
    else:
        vel, ids = sc.vel.copy(), sc.ids.copy()
    sim2 = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim2.set_material_grid(sc.mat)
    n = len(pos)
    for _ in range(2):
        n, _ = sim2.update_host(sc.dt, pos[:n], vel[:n], ids[:n])
    assert n == len(dids)
    assert np.array_equal(ids[:n], dids) and np.array_equal(pos[:n], dpos) and np.array_equal(vel[:n], dvel)


def test_invalid_dt_raises(gpu_ctx):
    from gridfluidsim3d_gb300 import GFSError
    sc = scenes.random_box(dims=(10, 10, 10), seed=1)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    with pytest.raises(GFSError):
        sim.update(-1.0)


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_pressure_check_against_fp64(gpu_ctx, precision):
    """gfs_sim_pressure_check: the step's pressure against an FP64 solve of the same
    system to 1e-12 -- the per-step error of the mixed form against the FP64 oracle."""
    from gridfluidsim3d_gb300 import PRECISION_MIXED, PRECISION_PLAIN
    sc = scenes.random_box(dims=(30, 22, 26), seed=3)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.precision = PRECISION_PLAIN if precision == "plain" else PRECISION_MIXED
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    for _ in range(2):
        sim.update(sc.dt)
        chk = sim.pressure_check(sc.dt)
        assert chk["fp64_residual"] < 1e-6
        assert chk["rel_error"] < (1e-6 if precision == "plain" else 1e-5), chk
    sim.close()


@pytest.mark.parametrize("speed", [1.0, 40.0], ids=["slow", "fast"])
def test_g2p_matches_standalone_sampler(gpu_ctx, speed):
    """The substep's fused PIC/FLIP + RK4 pass and the drop-in ParticleAdvector
    (RK4) and tricubic_interpolate on the step's own fields (the PIC/FLIP update
    redone in float32 in the reference's operation order) give the same bits,
    for every particle whose RK4 end point is not in a solid cell; the fast
    scene moves particles several cells per substep."""
    from gridfluidsim3d_gb300 import ParticleAdvector
    sc = scenes.random_box(dims=(40, 24, 28), seed=6, vel_sigma=speed)
    sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
    sim.set_material_grid(sc.mat)
    sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
    sim.update(sc.dt)                                   # a substep, so the fields are not trivial
    p0, v0, i0 = _by_id(*sim.get_marker_particles())
    sim.update(sc.dt)
    p1, v1, i1 = _by_id(*sim.get_marker_particles())
    assert np.array_equal(i0, i1)
    mac, saved = sim.get_velocity_field(), sim.get_saved_velocity_field()
    adv = ParticleAdvector(gpu_ctx)
    want = adv.advect_particles_rk4(p0, mac, sc.dt)
    cell = np.floor(want.astype(np.float64) / sc.dx).astype(np.int64)
    dims = np.array(sc.dims)
    inside = np.all((cell >= 0) & (cell < dims), axis=1)
    c = np.clip(cell, 0, dims - 1)
    free = inside & (sc.mat[c[:, 2], c[:, 1], c[:, 0]] != 2)
    assert free.mean() > 0.9
    assert np.array_equal(p1[free], want[free])
    vn = adv.tricubic_interpolate(p0, mac)
    vo = adv.tricubic_interpolate(p0, saved)
    a = np.float32(0.05)
    b = np.float32(1.0) - a
    vexp = a * vn + b * ((v0 + vn) - vo)
    assert np.array_equal(v1, vexp)
    if speed > 1.0:
        disp = np.abs(want - p0).max(axis=1) / sc.dx
        assert (disp > 2.0).sum() > 100
    sim.close()


def test_context_closed_before_its_simulation():
    """A garbage collector may finalise a context before a simulation built on it:
    the C context then stays allocated until the simulation is destroyed, and the
    simulation keeps stepping (the same state as on a context that stays open)."""
    import ctypes
    from gridfluidsim3d_gb300 import Context, _lib
    sc = scenes.random_box(dims=(20, 18, 16), seed=4)
    out = []
    for early_close in (False, True):
        ctx = Context(0)
        sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=ctx)
        sim.set_material_grid(sc.mat)
        sim.set_marker_particles(sc.pos, sc.vel, sc.ids)
        sim.update(sc.dt)
        if early_close:
            _lib.lib().gfs_ctx_destroy(ctx.handle)   # as a finaliser running first would
            ctx._h = ctypes.c_void_p()
        sim.update(sc.dt)
        out.append(sim.get_marker_particles())
        sim.close()
        ctx.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_duplicate_ids_lose_no_particle(gpu_ctx):
    """Particles are ordered by (cell, id); ids a caller repeats tie-break by position in
    the scattered set, so every particle keeps a slot of its own: the same count after a
    substep as with distinct ids, finite state, and every returned id one of the input ids."""
    sc = scenes.random_box(dims=(16, 12, 14), seed=2)
    counts = []
    for dup in (False, True):
        ids = sc.ids.copy()
        if dup:
            ids[1::2] = ids[0::2][:len(ids[1::2])]   # neighbours in the input share an id
        sim = FluidSimulation(*sc.dims, sc.dx, max_particles=sc.num_particles, ctx=gpu_ctx)
        sim.set_material_grid(sc.mat)
        sim.set_marker_particles(sc.pos, sc.vel, ids)
        sim.update(sc.dt)
        pos, vel, out = sim.get_marker_particles()
        assert np.isfinite(pos).all() and np.isfinite(vel).all()
        assert np.isin(out, ids).all()
        counts.append(len(out))
        sim.close()
    assert counts[0] == counts[1] and counts[0] > 0
