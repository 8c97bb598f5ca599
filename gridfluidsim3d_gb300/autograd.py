"""torch.autograd over the differentiable FLIP rollout (gfs_diff_* in include/gfs.h).

    sim = FluidSimulation(ni, nj, nk, dx, max_particles)   # grid, material, parameters
    sim.set_material_grid(mat)
    roll = FlipRollout(sim, nsteps=20, dt=1/30, num_particles=len(x0))
    density, centroids = roll(x0_cuda, u0=u0, v0=v0, w0=w0)   # CUDA float32 face fields, requires_grad
    loss = ((density - target) ** 2).sum()
    loss.backward()                          # u0.grad etc. from the hand-written CUDA adjoint

    density, centroids = roll(x0_cuda, velocities=v_particles)   # per-particle parameters instead

The forward runs the device-resident substep `nsteps` times from particles at
`x0` whose velocities are given or sampled from (u0, v0, w0), keeping every
substep's particle state in HBM; its outputs are the final cell density and
the centroid trajectory ((nsteps + 1) x 3).  Backward replays each substep's
grids from its checkpoint and runs the adjoint kernels (adjoint.cu), including
a second MIC(0)-PCG solve per substep for the pressure adjoint.  The starting
positions are inputs, not parameters.  There is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .core import FluidSimulation


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


class FlipRollout:
    """A differentiable rollout bound to one simulation (grid, material, parameters)."""

    def __init__(self, sim: FluidSimulation, nsteps: int, dt: float, num_particles: int):
        self.sim = sim
        self.nsteps, self.dt, self.n = int(nsteps), float(dt), int(num_particles)
        h = ctypes.c_void_p()
        _lib.lib().gfs_diff_create(sim._h, self.nsteps, self.n, self.dt, ctypes.byref(h))
        self._h = h
        sim._dependents.add(self)   # closed before the simulation it runs on

    def __call__(self, positions: torch.Tensor, u0=None, v0=None, w0=None, velocities=None):
        if velocities is None and (u0 is None or v0 is None or w0 is None):
            raise _lib.GFSError(_lib.GFS_ERR_INVALID, "FlipRollout", "give velocities or u0, v0 and w0")
        return _RolloutFn.apply(self, positions, velocities, u0, v0, w0)

    def info(self):
        """(forward ms, backward ms, device bytes of the rollout) of the last calls."""
        f, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        _lib.lib().gfs_diff_info(self._h, ctypes.byref(f), ctypes.byref(b), ctypes.byref(n))
        return f.value, b.value, n.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gfs_diff_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check(t: torch.Tensor, shape, name):
    if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and tuple(t.shape) == tuple(shape)):
        raise _lib.GFSError(_lib.GFS_ERR_INVALID, "FlipRollout",
                            f"{name} must be a contiguous CUDA float32 tensor of shape {tuple(shape)}")


def _opt(t):
    return _ptr(t) if t is not None else None


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, roll: FlipRollout, positions, velocities, u0, v0, w0):
        s = roll.sim
        ni, nj, nk = s.isize, s.jsize, s.ksize
        _check(positions, (roll.n, 3), "positions")
        sampled = velocities is None
        if sampled:
            _check(u0, (nk, nj, ni + 1), "u0")
            _check(v0, (nk, nj + 1, ni), "v0")
            _check(w0, (nk + 1, nj, ni), "w0")
        else:
            _check(velocities, (roll.n, 3), "velocities")
        dev = positions.device
        density = torch.empty((nk, nj, ni), device=dev, dtype=torch.float32)
        centroids = torch.empty((roll.nsteps + 1, 3), device=dev, dtype=torch.float32)
        torch.cuda.synchronize(dev)   # inputs written on torch's stream; the library uses its own
        if sampled:
            _lib.lib().gfs_diff_forward(roll._h, _ptr(positions), None, _ptr(u0), _ptr(v0), _ptr(w0), _ptr(density),
                                        _ptr(centroids))
        else:
            _lib.lib().gfs_diff_forward(roll._h, _ptr(positions), _ptr(velocities), None, None, None, _ptr(density),
                                        _ptr(centroids))
        ctx.roll = roll
        ctx.sampled = sampled
        ctx.shapes = (u0.shape, v0.shape, w0.shape) if sampled else None
        return density, centroids

    @staticmethod
    def backward(ctx, grad_density, grad_centroids):
        roll = ctx.roll
        gd = grad_density.contiguous().to(torch.float32) if grad_density is not None else None
        gc = grad_centroids.contiguous().to(torch.float32) if grad_centroids is not None else None
        dev = (gd if gd is not None else gc).device
        gu = gv = gw = gvel = None
        if ctx.sampled:
            gu, gv, gw = (torch.empty(sh, device=dev, dtype=torch.float32) for sh in ctx.shapes)
        else:
            gvel = torch.empty((roll.n, 3), device=dev, dtype=torch.float32)
        torch.cuda.synchronize(dev)
        _lib.lib().gfs_diff_backward(roll._h, _opt(gd), _opt(gc), _opt(gu), _opt(gv), _opt(gw), _opt(gvel), None)
        return None, None, gvel, gu, gv, gw
