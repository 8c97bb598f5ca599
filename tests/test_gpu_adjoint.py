"""GPU: the differentiable rollout's CUDA adjoint (csrc/adjoint.cu, through the
torch.autograd.Function of gridfluidsim3d_gb300.autograd) against the FP64
reference of the same rollout (oracle/diff_reference.py: its torch autograd
gradient and FP64 central finite differences, eps = 1e-4).

Tolerances: density after the rollout 1e-5 relative (5 substeps); gradients
1e-4 relative (L2 over the whole gradient against the FP64 adjoint, and
directional derivatives against FP64 central differences taken with the base
run's discrete structure held fixed -- the map the adjoint differentiates).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gridfluidsim3d_gb300 import PRECISION_PLAIN, FluidSimulation, scenes  # noqa: E402
from gridfluidsim3d_gb300.autograd import FlipRollout  # noqa: E402
from oracle import diff_reference as D  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(gpu_ctx):
    sc = scenes.diff_cube()
    dims, dx, dt = sc["dims"], sc["dx"], sc["dt"]
    model = D.Model(dims, dx, dt)
    x0 = torch.tensor(sc["pos"], dtype=torch.float64)
    rho0 = model.density(x0).detach().numpy()
    target = D.gaussian_target(dims, dx, sc["target_center"], sc["target_sigma"], rho0.sum())
    sim = FluidSimulation(*dims, dx, max_particles=len(x0), ctx=gpu_ctx)
    sim.reset_body_force()
    sim.precision = PRECISION_PLAIN
    sim.set_material_grid(sc["mat"])
    return dict(sc=sc, model=model, x0=x0, target=target, sim=sim)


def _gpu_field_gradient(cube, steps):
    sc = cube["sc"]
    roll = FlipRollout(cube["sim"], steps, sc["dt"], len(sc["pos"]))
    dev = torch.device("cuda:0")
    u = [torch.tensor(a, device=dev, requires_grad=True) for a in sc["u0"]]
    rho, _ = roll(torch.tensor(sc["pos"], device=dev), u0=u[0], v0=u[1], w0=u[2])
    loss = ((rho - torch.tensor(cube["target"], device=dev, dtype=torch.float32)) ** 2).sum()
    loss.backward()
    fwd_ms, bwd_ms, _ = roll.info()
    roll.close()
    return rho.detach().cpu().numpy(), [a.grad.double().cpu().numpy() for a in u], fwd_ms, bwd_ms


def _ref_field_gradient(cube, steps):
    u64 = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in cube["sc"]["u0"]]
    loss, _, _, rho = cube["model"].rollout(u64, cube["x0"], steps, torch.tensor(cube["target"]))
    loss.backward()
    cube["frozen"] = cube["model"].structures
    return rho.detach().numpy(), [a.grad.numpy() for a in u64], u64


def _rel_l2(a, b):
    return np.sqrt(sum(((x - y) ** 2).sum() for x, y in zip(a, b))) / np.sqrt(sum((y ** 2).sum() for y in b))


def test_field_gradient_matches_fp64_adjoint_and_fd(cube):
    steps = 5
    rho, g, fwd_ms, bwd_ms = _gpu_field_gradient(cube, steps)
    rho64, g64, u64 = _ref_field_gradient(cube, steps)
    assert np.abs(rho - rho64).max() / np.abs(rho64).max() < 1e-5
    assert _rel_l2(g, g64) < 1e-4
    # directional derivatives against FP64 central differences of the reference
    rng = np.random.default_rng(3)
    eps = 1e-4
    model, x0, target = cube["model"], cube["x0"], torch.tensor(cube["target"])
    for _ in range(2):
        dirs = [rng.normal(size=a.shape) for a in g64]
        with torch.no_grad():
            lp = model.rollout([a + eps * torch.tensor(d) for a, d in zip(u64, dirs)], x0, steps, target,
                               cube["frozen"])[0]
            lm = model.rollout([a - eps * torch.tensor(d) for a, d in zip(u64, dirs)], x0, steps, target,
                               cube["frozen"])[0]
        fd = float((lp - lm) / (2 * eps))
        dg = float(sum((a * d).sum() for a, d in zip(g, dirs)))
        assert abs(dg - fd) <= 1e-4 * abs(fd), (dg, fd)
    assert bwd_ms <= 3.0 * fwd_ms + 5.0, (fwd_ms, bwd_ms)


def test_field_gradient_20_substeps(cube):
    """The small differentiable-control configuration: 32^3, 12^3 cube, 20 substeps."""
    rho, g, fwd_ms, bwd_ms = _gpu_field_gradient(cube, 20)
    rho64, g64, _ = _ref_field_gradient(cube, 20)
    assert np.abs(rho - rho64).max() / np.abs(rho64).max() < 1e-3
    assert _rel_l2(g, g64) < 1e-4
    assert bwd_ms <= 3.0 * fwd_ms, (fwd_ms, bwd_ms)


def test_gradients_bitwise_reproducible(cube):
    """The G2P adjoint scatters in fixed point (integer sums), and the centroid
    sums in a fixed tree: two runs of the same rollout give the same bits."""
    sc = cube["sc"]
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    v0 = rng.uniform(-1.0, 1.0, size=sc["pos"].shape).astype(np.float32)
    runs = []
    for _ in range(2):
        _, g, _, _ = _gpu_field_gradient(cube, 6)
        roll = FlipRollout(cube["sim"], 4, sc["dt"], len(sc["pos"]))
        vg = torch.tensor(v0, device=dev, requires_grad=True)
        _, cen = roll(torch.tensor(sc["pos"], device=dev), velocities=vg)
        (cen.double() ** 2).sum().backward()
        roll.close()
        runs.append((g, cen.detach().cpu().numpy(), vg.grad.cpu().numpy()))
    (g0, c0, v0g), (g1, c1, v1g) = runs
    for a, b in zip(g0, g1):
        assert np.array_equal(a, b), "field gradients differ between runs"
    assert np.array_equal(c0, c1) and np.array_equal(v0g, v1g)
    assert any(np.abs(a).max() > 0 for a in g0)


def test_velocity_parameters_and_centroid_loss(cube):
    """Per-particle initial velocities as parameters, loss on the centroid trajectory."""
    sc = cube["sc"]
    steps = 4
    rng = np.random.default_rng(9)
    v0 = rng.uniform(-1.0, 1.0, size=sc["pos"].shape).astype(np.float32)
    goal = (rng.normal(size=(steps + 1, 3)) * 0.05 + sc["pos"].mean(0)).astype(np.float64)
    dev = torch.device("cuda:0")
    roll = FlipRollout(cube["sim"], steps, sc["dt"], len(sc["pos"]))
    vg = torch.tensor(v0, device=dev, requires_grad=True)
    _, cen = roll(torch.tensor(sc["pos"], device=dev), velocities=vg)
    loss = ((cen.double() - torch.tensor(goal, device=dev)) ** 2).sum()
    loss.backward()
    roll.close()
    v64 = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    _, cents, _, _ = cube["model"].run(cube["x0"], v64, steps)
    loss64 = ((cents - torch.tensor(goal)) ** 2).sum()
    loss64.backward()
    assert np.abs(cen.detach().cpu().numpy() - cents.detach().numpy()).max() < 1e-5
    assert _rel_l2([vg.grad.double().cpu().numpy()], [v64.grad.numpy()]) < 1e-4


def test_adam_reduces_the_loss(cube):
    """The autograd integration: a few Adam steps on the parameter field lower the loss."""
    sc = cube["sc"]
    dev = torch.device("cuda:0")
    roll = FlipRollout(cube["sim"], 3, sc["dt"], len(sc["pos"]))
    u = [torch.tensor(a, device=dev, requires_grad=True) for a in sc["u0"]]
    opt = torch.optim.Adam(u, lr=0.05)
    xs = torch.tensor(sc["pos"], device=dev)
    tgt = torch.tensor(cube["target"], device=dev, dtype=torch.float32)
    losses = []
    for _ in range(4):
        opt.zero_grad()
        rho, _ = roll(xs, u0=u[0], v0=u[1], w0=u[2])
        loss = ((rho - tgt) ** 2).sum()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    roll.close()
    assert losses[-1] < losses[0], losses


def test_gravity_without_wall_contact(gpu_ctx):
    """Body force on the fluid-bordering faces: the cube falling under gravity
    (0, -25, 0) for 4 substeps, clear of the walls, against the FP64 reference."""
    sc = scenes.diff_cube()
    dims, dx, dt = sc["dims"], sc["dx"], sc["dt"]
    model = D.Model(dims, dx, dt, gravity=(0.0, -25.0, 0.0))
    x0 = torch.tensor(sc["pos"], dtype=torch.float64)
    rho0 = model.density(x0).detach().numpy()
    target = D.gaussian_target(dims, dx, sc["target_center"], sc["target_sigma"], rho0.sum())
    sim = FluidSimulation(*dims, dx, max_particles=len(x0), ctx=gpu_ctx)
    sim.reset_body_force()
    sim.add_body_force(0.0, -25.0, 0.0)
    sim.precision = PRECISION_PLAIN
    sim.set_material_grid(sc["mat"])
    cube = dict(sc=sc, model=model, x0=x0, target=target, sim=sim)
    rho, g, _, _ = _gpu_field_gradient(cube, 4)
    rho64, g64, _ = _ref_field_gradient(cube, 4)
    assert np.abs(rho - rho64).max() / np.abs(rho64).max() < 1e-5
    assert _rel_l2(g, g64) < 1e-4
    sim.close()
