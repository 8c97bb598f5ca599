"""The oracle against the reference's own CPU code, live (oracle/_ref, compiled from
the reference sources by oracle/Makefile).  Only where the reference tree is
present; the committed golden fixtures cover the same ground elsewhere.
Comparisons are bit-exact.
"""
import numpy as np
import pytest

import oracle as O
from gridfluidsim3d_gb300 import scenes

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference tree not present")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_splat(oracle_lib, seed):
    sc = scenes.random_box(dims=(11 + seed, 9 + 2 * seed, 10), seed=seed)
    for c in range(3):
        f, m = O.velocity_scalar_field(c, sc.dims, sc.dx, sc.pos, sc.vel)
        rf, rw = O.ref_velocity_scalar_field(c, sc.dims, sc.dx, sc.pos, sc.vel)
        assert np.array_equal(f, rf) and np.array_equal(m.astype(bool), rw > 1e-9)


@pytest.mark.parametrize("seed", [7, 8, 9])
def test_point_splat(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    W, H, D = (int(x) for x in rng.integers(5, 12, 3))
    dx = float(rng.uniform(0.05, 1.0))
    for rmul in (0.6, 1.0, 1.7, 3.1):
        n = int(rng.integers(0, 500))
        pts = rng.uniform(-3 * dx, (max(W, H, D) + 3) * dx, (n, 3)).astype(np.float32)
        vals = rng.normal(size=n).astype(np.float32) if rmul != 1.0 else None
        off = rng.uniform(-dx, dx, 3).astype(np.float32)
        field = rng.uniform(0, 2, (D, H, W)).astype(np.float32)
        weight = np.zeros_like(field) if rmul > 1.0 else None
        a = O.splat_points(pts, vals, rmul * dx, off, dx, field, weight)
        b = O.ref_add_point_values(pts, vals, rmul * dx, off, dx, field, weight)
        assert np.array_equal(a[0], b[0])
        if weight is not None:
            assert np.array_equal(a[1], b[1])


@pytest.mark.parametrize("seed", [4, 5])
def test_pressure_and_extrapolate(oracle_lib, seed):
    sc = scenes.random_box(dims=(12, 10 + seed, 13), seed=seed, solid_blocks=3)
    mat = sc.mat.copy()
    pos, vel, ids = sc.pos.copy(), sc.vel.copy(), sc.ids.copy()
    n = O.lib().gfo_update_fluid_cells(*sc.dims, sc.dx, mat, pos, vel, ids, len(pos))
    u, v, w = O.advect_velocity_field(sc.dims, sc.dx, mat, pos[:n], vel[:n])
    p, it, _ = O.pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w)
    rp, rit = O.ref_pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w)
    assert it == rit and np.array_equal(p, rp)
    e = O.extrapolate(sc.dims, mat, 7, u, v, w)
    re = O.ref_extrapolate(sc.dims, sc.dx, mat, 7, u, v, w)
    assert all(np.array_equal(a, b) for a, b in zip(e, re))


def test_rk4_is_reference_formula(oracle_lib):
    """ParticleAdvector::_RK4 (particleadvector.cpp:1045-1054) over the reference's sampler."""
    rng = np.random.default_rng(9)
    dims, dx, dt = (10, 9, 8), 0.2, 1.0 / 30.0
    u = rng.normal(size=(8, 9, 11)).astype(np.float32)
    v = rng.normal(size=(8, 10, 10)).astype(np.float32)
    w = rng.normal(size=(9, 9, 10)).astype(np.float32)
    p0 = (rng.random((500, 3)) * np.array(dims) * dx).astype(np.float32)
    ev = lambda p: O.ref_evaluate_velocity(dims, dx, u, v, w, p)  # noqa: E731
    k1 = ev(p0)
    k2 = ev(p0 + np.float32(0.5 * dt) * k1)
    k3 = ev(p0 + np.float32(0.5 * dt) * k2)
    k4 = ev(p0 + np.float32(dt) * k3)
    want = p0 + np.float32(dt / np.float32(6.0)) * (((k1 + np.float32(2) * k2) + np.float32(2) * k3) + k4)
    got = O.advect_rk4(dims, dx, u, v, w, dt, p0)
    assert np.array_equal(got, want)


def test_ray_aabb(oracle_lib):
    rng = np.random.default_rng(3)
    for _ in range(300):
        p0 = (rng.random(3) * 3).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        d /= np.float32(np.linalg.norm(d))
        if rng.random() < 0.2:
            d[rng.integers(3)] = 0.0
        bpos = (rng.random(3) * 3).astype(np.float32)
        out_r = np.zeros(3, np.float32)
        hit_r = O.ref().gfsref_ray_aabb(p0, d, bpos, 0.5, 0.5, 0.5, out_r)
        bmin = bpos
        bmax = (bpos + np.float32(0.5)).astype(np.float32)
        out_o = np.zeros(3, np.float32)
        hit_o = O.lib().gfo_ray_aabb(p0, d, bmin, bmax, out_o)
        assert hit_o == hit_r
        if hit_o:
            assert np.array_equal(out_o, out_r)
