"""Host-side logic on the CPU: seeded scenes, the oracle's substep invariants,
and the bench's CPU-baseline estimate on a tiny scene."""
import numpy as np

import oracle as O
from gridfluidsim3d_gb300 import scenes


def test_scenes_are_seeded_and_in_cell():
    a = scenes.random_box(dims=(12, 10, 11), seed=7)
    b = scenes.random_box(dims=(12, 10, 11), seed=7)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)
    cells = np.floor(a.pos / np.float32(a.dx)).astype(int)
    assert (cells >= 1).all() and (cells < np.array(a.dims) - 1).all()
    c = np.floor(scenes.ball_drop(n=32, dx=0.25).pos / 0.25).astype(int)
    _, counts = np.unique(c, axis=0, return_counts=True)
    assert (counts == 8).all()


def test_scene_sizes():
    d = scenes.dam_break(n=32, dx=0.25)
    assert d.num_particles > 0 and d.dims == (32, 32, 32)
    s = scenes.slab_spheres(n=32, dx=0.25, seed=3)
    assert abs(float(s.vel.std()) - 0.5) < 0.05


def test_oracle_substep_invariants(oracle_lib):
    sc = scenes.random_box(dims=(14, 12, 13), seed=2)
    st = O.substep(sc.dims, sc.dx, sc.dt, sc.gravity, sc.mat, sc.pos, sc.vel, sc.ids)
    # no cell is over the cap, so every particle survives; ids are a permutation
    assert len(st["ids"]) == sc.num_particles
    assert np.array_equal(np.sort(st["ids"]), sc.ids)
    # the fluid cells are the cells that held particles at the start of the substep
    cells = np.floor(sc.pos / np.float32(sc.dx)).astype(int)
    occ = np.zeros(sc.mat.shape, bool)
    occ[cells[:, 2], cells[:, 1], cells[:, 0]] = True
    assert np.array_equal(st["mat"] == 1, occ)
    assert st["cg_iterations"] >= 0 and st["cg_max_resid"] < 1e-6
    # particles never end in solid cells
    c2 = np.floor(st["pos"] / np.float32(sc.dx)).astype(int)
    assert (sc.mat[c2[:, 2], c2[:, 1], c2[:, 0]] != 2).all()


def test_particle_cap_keeps_smallest_ids(oracle_lib):
    dims, dx = (6, 6, 6), 1.0
    pos = np.full((150, 3), 2.5, np.float32) + np.linspace(0, 0.4, 150, dtype=np.float32)[:, None]
    vel = np.zeros_like(pos)
    ids = np.arange(150, dtype=np.uint32)[::-1].copy()
    n = O.lib().gfo_cap_particles_per_cell(*dims, dx, 100, pos, vel, ids, len(pos))
    assert n == 100 and set(ids[:n].tolist()) == set(range(100))


def test_bench_cpu_estimate_small(oracle_lib):
    import bench
    sc = scenes.random_box(dims=(14, 12, 13), seed=3)
    total, parts, wall, ns, n = bench.cpu_estimate(sc, iters=10, sample_particles=500)
    assert total > 0 and ns == 500 and n == sc.num_particles
    assert set(parts) >= {"splat_particles", "pressure", "g2p_rk4", "extrapolate"}
