"""Write the substep fixtures of tests/golden/ with the reference's own code.

The reference's simulator library is built on the CPU with oracle/reftree.py:
fluidsimulation.cpp, the reference's own PressureSolver and everything else
compiled unchanged, with only the two OpenCL classes replaced by CPU backends
that run the reference's OpenCL-disabled arithmetic (oracle/refcpu/).  The probe
oracle/ref_substep_probe.cpp then runs one substep of FluidSimulation stage by
stage and writes the state after each stage.

Scenes (each written as a savestate with the oracle's writer, which the
reference reads with FluidSimulationSaveState::loadState):

* ``substep_pool`` -- 18 x 16 x 14 cells, dx 0.1, solid border and two interior
  solid blocks, a random blob of fluid over a pool, 8 particles per fluid cell
  uniform in-cell, velocities N(0, 1), gravity (0, -25, 0), dt 1/30: splat,
  saved-field extrapolation, body force, pressure, apply-pressure next to
  solids, PIC/FLIP and RK4 with solid collisions.
* ``substep_sparse`` -- 14 x 12 x 12 cells, dx 0.1, one particle in 70% of the
  cells of a blob and a pool, half of them at rest: many faces bordering fluid
  get no splat weight and take the 26-neighbour fill, and set faces holding
  exactly 0 separate the U fill (nonzero neighbours) from the V / W fills (set
  neighbours).
* ``substep_crowd`` -- 12 x 10 x 10 cells, dx 0.2, a resting pool three cells
  deep with 8 particles per cell, and three pool cells crowded with 137, 101 and
  100 particles; zero velocity, gravity (0, -25, 0), dt 1/30: the per-cell cap of
  _removeMarkerParticles (100 per cell).

Stored per scene (npz): the input (material, positions, velocities, dims, dx,
dt, gravity), the classification, the three face grids after stages 5, 6, 8 and
9 and the saved field, the float pressure grid, the particle velocities after
the PIC/FLIP update, the positions after advection (input order: no removal
pass), and the per-cell particle counts after the reference's removal pass.

Needs the reference's src/ ($GFS_REFERENCE_SRC or the recorded oracle build) and
g++; the fixtures are committed.

    python tests/golden/make_substep_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import reference_src, reftree  # noqa: E402
from oracle import savestate as S  # noqa: E402
from gridfluidsim3d_gb300 import scenes  # noqa: E402

SRC = reference_src()   # $GFS_REFERENCE_SRC, or the directory the last oracle build recorded
DT = 1.0 / 30.0
GRAVITY = (0.0, -25.0, 0.0)
MAX_PER_CELL = 100
SHUFFLE_SEED = 1


def pool_scene():
    sc = scenes.random_box(dims=(18, 16, 14), dx=0.1, seed=7, fill=0.4, vel_sigma=1.0, solid_blocks=2)
    return dict(name="substep_pool", dims=sc.dims, dx=sc.dx, mat=sc.mat, pos=sc.pos, vel=sc.vel)


def crowd_scene(seed=9):
    dims, dx = (12, 10, 10), 0.2
    rng = np.random.default_rng(seed)
    mat = scenes.solid_border(dims)
    fluid = np.zeros(mat.shape, bool)
    fluid[1:-1, 1:4, 1:-1] = True
    pos = scenes.seed_particles(fluid, dx, 8, rng)
    extra = []
    for (i, j, k), n in (((4, 2, 5), 129), ((7, 1, 3), 93), ((2, 3, 7), 92)):
        off = rng.random((n, 3)) * 0.999 + 0.0005
        extra.append(((np.array([i, j, k]) + off) * dx).astype(np.float32))
    pos = np.concatenate([pos] + extra).astype(np.float32)
    vel = np.zeros_like(pos)
    return dict(name="substep_crowd", dims=dims, dx=dx, mat=mat, pos=pos, vel=vel)


def sparse_scene(seed=13):
    """Few particles per fluid cell, so that many faces bordering fluid get no
    splat weight and take the 26-neighbour fill; half the particles are at rest,
    so that set faces with the value 0 exist, which the U fill skips and the V / W
    fills count (fluidsimulation.cpp:2630 vs :2675, :2720)."""
    dims, dx = (14, 12, 12), 0.1
    rng = np.random.default_rng(seed)
    mat = scenes.solid_border(dims)
    mat[5:7, 2:4, 6:8] = scenes.SOLID
    k, j, i = np.meshgrid(np.arange(dims[2]), np.arange(dims[1]), np.arange(dims[0]), indexing="ij")
    blob = ((i - 7) ** 2 + (j - 5) ** 2 + (k - 6) ** 2 < 16) | (j <= 2)
    fluid = blob & (mat != scenes.SOLID) & (rng.random(mat.shape) < 0.7)
    pos = scenes.seed_particles(fluid, dx, 1, rng)
    vel = rng.normal(0.0, 1.0, pos.shape).astype(np.float32)
    vel[rng.random(len(pos)) < 0.5] = 0.0
    return dict(name="substep_sparse", dims=dims, dx=dx, mat=mat, pos=pos, vel=vel)


def _read(d, name, dtype, shape):
    a = np.fromfile(os.path.join(d, name), dtype=dtype)
    return a.reshape(shape)


def run(scene, tree, exe, tmp):
    dims, dx = scene["dims"], scene["dx"]
    ni, nj, nk = dims
    fin = os.path.join(tmp, scene["name"] + ".state")
    S.write_state(fin, dims, dx, 0, scene["pos"], scene["vel"], scene["mat"])
    out = os.path.join(tmp, scene["name"])
    os.makedirs(out, exist_ok=True)
    r = subprocess.run([exe, fin, out, repr(DT), *map(repr, GRAVITY), str(MAX_PER_CELL), str(SHUFFLE_SEED)],
                       capture_output=True, text=True, timeout=600, cwd=tmp)
    if r.returncode != 0:
        raise RuntimeError(f"probe failed ({r.returncode}): {r.stderr[-2000:]}")
    line = [l for l in r.stdout.splitlines() if l.startswith("PROBE ")][-1]
    nfluid, n_adv, n_cap = map(int, line.split()[1:])
    shapes = {"u": (nk, nj, ni + 1), "v": (nk, nj + 1, ni), "w": (nk + 1, nj, ni)}
    res = dict(dims=np.array(dims), dx=np.float64(dx), dt=np.float64(DT), gravity=np.array(GRAVITY, np.float32),
               max_per_cell=np.int32(MAX_PER_CELL), mat_in=scene["mat"], pos_in=scene["pos"], vel_in=scene["vel"],
               num_fluid_cells=np.int64(nfluid))
    res["mat1"] = _read(out, "mat1.u8", np.uint8, (nk, nj, ni))
    p1 = _read(out, "p1.f32", np.float32, (-1, 6))
    # _updateFluidCells keeps the input order; record which input particles it kept
    assert len(p1) == n_adv
    for tag in ("advected", "saved", "body", "applied", "extrap"):
        for c in "uvw":
            res[f"{tag}_{c}"] = _read(out, f"{tag}.{c}", np.float32, shapes[c])
    res["pressure"] = _read(out, "pressure.f32", np.float32, (nk, nj, ni))
    p11 = _read(out, "p11.f32", np.float32, (-1, 6))
    p12 = _read(out, "p12.f32", np.float32, (-1, 6))
    cap = _read(out, "p12cap.f32", np.float32, (-1, 6))
    assert len(cap) == n_cap
    res["pos1"] = p1[:, :3].copy()
    res["vel11"] = p11[:, 3:].copy()
    res["pos12"] = p12[:, :3].copy()
    cells = np.floor(cap[:, :3].astype(np.float64) / dx).astype(np.int64)
    counts = np.zeros((nk, nj, ni), np.int32)
    np.add.at(counts, (cells[:, 2], cells[:, 1], cells[:, 0]), 1)
    res["cap_counts"] = counts
    print(f"{scene['name']}: {len(scene['pos'])} particles in, {n_adv} after stage 1, {n_cap} after the cap, "
          f"{nfluid} fluid cells, max|p| {np.abs(res['pressure']).max():.4g}")
    return res


def main():
    if SRC is None:
        sys.exit("the reference's src/ directory is unknown: set GFS_REFERENCE_SRC")
    with tempfile.TemporaryDirectory() as tmp:
        tree = os.path.join(tmp, "tree")
        reftree.build_cpu_tree(SRC, tree)
        exe = reftree.build_probe(tree, os.path.join(ROOT, "oracle", "ref_substep_probe.cpp"),
                                  os.path.join(tmp, "probe"))
        for scene in (pool_scene(), sparse_scene(), crowd_scene()):
            res = run(scene, tree, exe, tmp)
            np.savez_compressed(os.path.join(HERE, scene["name"] + ".npz"), **res)


if __name__ == "__main__":
    main()
