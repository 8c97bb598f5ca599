"""Seeded synthetic scenes for the FLIP substep (host side, numpy).

The reference seeds particles on a jittered 2x2x2 sub-lattice
(fluidsimulation.cpp:1219-1247) with the global rand(); these scenes instead
place `ppc` particles uniformly at random inside every fluid cell from a fixed
numpy seed, so that the oracle and the CUDA path see bit-identical inputs.

Arrays use the reference's flat layout (index i + ni*(j + nj*k)); numpy shapes
are (nk, nj, ni).  Material: 0 air, 1 fluid, 2 solid; the domain border is
solid, as FluidSimulation::_initializeSolidCells makes it
(fluidsimulation.cpp:1191-1213).  Fluid cells are not marked here: the first
substep's classification (the reference's _updateFluidCells) marks them from
the particles.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

AIR, FLUID, SOLID = 0, 1, 2


@dataclass
class Scene:
    name: str
    dims: tuple            # (ni, nj, nk)
    dx: float
    mat: np.ndarray        # uint8 (nk, nj, ni)
    pos: np.ndarray        # float32 (N, 3)
    vel: np.ndarray        # float32 (N, 3)
    ids: np.ndarray        # uint32 (N,)
    gravity: tuple = (0.0, -25.0, 0.0)
    dt: float = 1.0 / 30.0
    meta: dict = field(default_factory=dict)

    @property
    def num_particles(self) -> int:
        return int(self.pos.shape[0])


def solid_border(dims) -> np.ndarray:
    ni, nj, nk = dims
    mat = np.zeros((nk, nj, ni), np.uint8)
    mat[0, :, :] = SOLID
    mat[-1, :, :] = SOLID
    mat[:, 0, :] = SOLID
    mat[:, -1, :] = SOLID
    mat[:, :, 0] = SOLID
    mat[:, :, -1] = SOLID
    return mat


def cell_centers(dims, dx):
    ni, nj, nk = dims
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    return (i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dx


def seed_particles(fluid: np.ndarray, dx: float, ppc: int, rng: np.random.Generator):
    """`ppc` particles per True cell of `fluid` ((nk, nj, ni) bool), uniform in-cell.

    Offsets are drawn in [0.0005, 0.9995) of a cell so that float32 rounding of
    (cell + offset) * dx can never land on the next cell's boundary.
    """
    kk, jj, ii = np.nonzero(fluid)
    nc = ii.shape[0]
    base = np.stack([ii, jj, kk], axis=1).astype(np.float64)
    base = np.repeat(base, ppc, axis=0)
    off = rng.random((nc * ppc, 3)) * 0.999 + 0.0005
    pos = ((base + off) * dx).astype(np.float32)
    return pos


def _finish(name, dims, dx, mat, pos, vel, seed, **meta):
    ids = np.arange(pos.shape[0], dtype=np.uint32)
    return Scene(name=name, dims=tuple(dims), dx=float(dx), mat=mat, pos=np.ascontiguousarray(pos),
                 vel=np.ascontiguousarray(vel), ids=ids, meta=dict(seed=seed, **meta))


def ball_drop(n: int = 64, dx: float = 0.125, seed: int = 1, ppc: int = 8) -> Scene:
    """Hello-world ball drop: sphere r=1.6 centred at (4,4,4) in a solid box."""
    dims = (n, n, n)
    mat = solid_border(dims)
    cx, cy, cz = cell_centers(dims, dx)
    c = np.array([4.0, 4.0, 4.0]) * (n * dx / 8.0)
    r = 1.6 * (n * dx / 8.0)
    fluid = ((cx - c[0]) ** 2 + (cy - c[1]) ** 2 + (cz - c[2]) ** 2 < r * r) & (mat != SOLID)
    rng = np.random.default_rng(seed)
    pos = seed_particles(fluid, dx, ppc, rng)
    vel = np.zeros_like(pos)
    return _finish("ball_drop", dims, dx, mat, pos, vel, seed, frames=30)


def dam_break(n: int = 128, dx: float = 0.0625, seed: int = 2, ppc: int = 8) -> Scene:
    """Dam break: fluid box x in [0, 0.35L], y in [0, 0.6L], full z."""
    dims = (n, n, n)
    L = n * dx
    mat = solid_border(dims)
    cx, cy, cz = cell_centers(dims, dx)
    fluid = (cx < 0.35 * L) & (cy < 0.6 * L) & (mat != SOLID)
    rng = np.random.default_rng(seed)
    pos = seed_particles(fluid, dx, ppc, rng)
    vel = np.zeros_like(pos)
    return _finish("dam_break", dims, dx, mat, pos, vel, seed, substeps=60)


def slab_spheres(n: int = 256, dx: float = 1.0 / 32.0, seed: int = 3, ppc: int = 8,
                 num_spheres: int = 20, vel_sigma: float = 0.5) -> Scene:
    """Throughput scene: slab y < 0.3L plus 20 spheres of radius U(4,12) cells
    centred uniformly in the band y in [0.3L, 0.9L]; velocities N(0, 0.5^2)."""
    dims = (n, n, n)
    L = n * dx
    mat = solid_border(dims)
    rng = np.random.default_rng(seed)
    cx, cy, cz = cell_centers(dims, dx)
    fluid = cy < 0.3 * L
    scale = n / 256.0
    for _ in range(num_spheres):
        r = rng.uniform(4.0, 12.0) * scale * dx
        c = np.array([rng.uniform(0.1 * L, 0.9 * L), rng.uniform(0.3 * L, 0.9 * L),
                      rng.uniform(0.1 * L, 0.9 * L)])
        fluid |= (cx - c[0]) ** 2 + (cy - c[1]) ** 2 + (cz - c[2]) ** 2 < r * r
    fluid &= mat != SOLID
    pos = seed_particles(fluid, dx, ppc, rng)
    vel = rng.normal(0.0, vel_sigma, size=pos.shape).astype(np.float32)
    return _finish("slab_spheres", dims, dx, mat, pos, vel, seed, substeps=100)


def random_box(dims=(16, 12, 14), dx: float = 0.1, seed: int = 0, ppc: int = 8,
               fill: float = 0.45, vel_sigma: float = 1.0, solid_blocks: int = 2) -> Scene:
    """Small irregular scene for parity tests: a random blob of fluid with
    random velocities and a few interior solid blocks."""
    ni, nj, nk = dims
    rng = np.random.default_rng(seed)
    mat = solid_border(dims)
    for _ in range(solid_blocks):
        a = rng.integers(2, [max(3, ni - 4), max(3, nj - 4), max(3, nk - 4)])
        mat[a[2]:a[2] + 2, a[1]:a[1] + 2, a[0]:a[0] + 2] = SOLID
    cx, cy, cz = cell_centers(dims, dx)
    c = np.array([ni, nj * 0.6, nk]) * dx * 0.5
    rad = fill * min(ni, nj, nk) * dx
    noise = rng.random(mat.shape) * 0.3 * rad
    fluid = ((cx - c[0]) ** 2 + (cy - c[1]) ** 2 + (cz - c[2]) ** 2 < (rad + noise) ** 2)
    fluid |= cy < 0.25 * nj * dx
    fluid &= mat != SOLID
    pos = seed_particles(fluid, dx, ppc, rng)
    vel = rng.normal(0.0, vel_sigma, size=pos.shape).astype(np.float32)
    return _finish("random_box", dims, dx, mat, pos, vel, seed)


def diff_cube(n: int = 32, dx: float = 0.25, cube: int = 12, ppc: int = 8, seed: int = 4):
    """Differentiable-control scene (small): an n^3 grid with solid walls, a cube of
    `cube`^3 fluid cells at the centre with `ppc` particles per cell uniform in each
    cell, a parameter MAC field U(-1, 1), and a target cell density: a Gaussian
    blob of sigma 3 cells, 6 cells in +x from the cube centre, with the total of
    the initial density (computed by the caller's density operator)."""
    dims = (n, n, n)
    rng = np.random.default_rng(seed)
    mat = solid_border(dims)
    lo = (n - cube) // 2
    fluid = np.zeros(dims[::-1], bool)
    fluid[lo:lo + cube, lo:lo + cube, lo:lo + cube] = True
    pos = seed_particles(fluid, dx, ppc, rng)
    u0 = [rng.uniform(-1.0, 1.0, size=shape).astype(np.float32)
          for shape in ((n, n, n + 1), (n, n + 1, n), (n + 1, n, n))]
    center = (n / 2 + 6.0, n / 2, n / 2)
    return dict(dims=dims, dx=dx, dt=1.0 / 30.0, steps=20, mat=mat, pos=pos, u0=u0, target_center=center,
                target_sigma=3.0)


SCENES = {"ball_drop": ball_drop, "dam_break": dam_break, "slab_spheres": slab_spheres,
          "random_box": random_box}
