"""The FP64 reference of the differentiable rollout (oracle/diff_reference.py)
against FP64 central finite differences of itself, so that it can serve as the
checker of the CUDA adjoint.  The differences are taken with the discrete
structure of the base run held fixed (the map the adjoint differentiates), so
that a perturbation cannot flip a cell's classification or a face's set mask.
CPU only."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import diff_reference as D  # noqa: E402
from gridfluidsim3d_gb300 import scenes  # noqa: E402


def _setup(steps):
    sc = scenes.diff_cube(n=24, cube=8, ppc=4, seed=5)
    dims, dx, dt = sc["dims"], sc["dx"], sc["dt"]
    m = D.Model(dims, dx, dt)
    x0 = torch.tensor(sc["pos"], dtype=torch.float64)
    rho0 = m.density(x0).detach().numpy()
    target = torch.tensor(D.gaussian_target(dims, dx, (dims[0] / 2 + 4, dims[1] / 2, dims[2] / 2), 3.0, rho0.sum()))
    return sc, m, x0, target


def test_field_gradient_matches_central_differences():
    sc, m, x0, target = _setup(2)
    u0 = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in sc["u0"]]
    loss = m.rollout(u0, x0, 2, target)[0]
    loss.backward()
    frozen = m.structures
    rng = np.random.default_rng(1)
    for _ in range(2):
        dirs = [torch.tensor(rng.normal(size=a.shape)) for a in sc["u0"]]
        eps = 1e-4   # the FD step of the gradient check
        with torch.no_grad():
            lp = m.rollout([a + eps * d for a, d in zip(u0, dirs)], x0, 2, target, frozen)[0]
            lm = m.rollout([a - eps * d for a, d in zip(u0, dirs)], x0, 2, target, frozen)[0]
        fd = float((lp - lm) / (2 * eps))
        ad = float(sum((a.grad * d).sum() for a, d in zip(u0, dirs)))
        assert abs(fd - ad) <= 1e-4 * abs(fd), (fd, ad)


def test_velocity_gradient_of_centroid_loss_matches_central_differences():
    sc, m, x0, target = _setup(2)
    rng = np.random.default_rng(2)
    v0 = torch.tensor(rng.uniform(-1, 1, x0.shape), requires_grad=True)
    goal = torch.tensor(rng.normal(size=(3, 3)) * 0.05) + x0.mean(0)
    _, cents, _, _ = m.run(x0, v0, 2)
    frozen = m.structures
    loss = ((cents - goal) ** 2).sum()
    loss.backward()
    d = torch.tensor(rng.normal(size=x0.shape))
    eps = 1e-4
    with torch.no_grad():
        lp = ((m.run(x0, v0 + eps * d, 2, frozen)[1] - goal) ** 2).sum()
        lm = ((m.run(x0, v0 - eps * d, 2, frozen)[1] - goal) ** 2).sum()
    fd = float((lp - lm) / (2 * eps))
    ad = float((v0.grad * d).sum())
    assert abs(fd - ad) <= 1e-4 * abs(fd), (fd, ad)
