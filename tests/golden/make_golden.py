"""Write the golden fixtures of tests/golden/ from the reference's own CPU code.

Runs in a container that has the reference tree: oracle/Makefile's `ref` target
compiles the reference's CL-free sources (where they lie) with oracle/ref_shim.cpp
into oracle/_ref/libgfsref.so, and this script calls the reference's
ScalarField / PressureSolver / MACVelocityField / Collision through it on small
seeded inputs, saving inputs and outputs as .npz.  The fixtures are committed;
the tests compare the oracle (and, on a GPU, the CUDA path) against them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from gridfluidsim3d_gb300 import scenes  # noqa: E402


def fluid_state(sc):
    mat = sc.mat.copy()
    pos, vel, ids = sc.pos.copy(), sc.vel.copy(), sc.ids.copy()
    n = O.lib().gfo_update_fluid_cells(*sc.dims, sc.dx, mat, pos, vel, ids, len(pos))
    return mat, pos[:n], vel[:n], ids[:n]


def point_splat_cases():
    """Seeded inputs of the general point-splat fixture."""
    rng = np.random.default_rng(51)
    cases = []
    for t, (rmul, with_vals, with_w, thr) in enumerate([(1.0, True, True, False), (1.5, True, False, False),
                                                         (2.3, False, True, False), (0.7, False, False, False),
                                                         (1.2, True, True, True), (1.0, False, True, True)]):
        W, H, D = (int(x) for x in rng.integers(6, 13, 3))
        dx = float(rng.uniform(0.1, 0.5))
        n = int(rng.integers(200, 600))
        pts = rng.uniform(-2 * dx, (max(W, H, D) + 2) * dx, (n, 3)).astype(np.float32)
        field = np.zeros((D, H, W), np.float32)
        if thr:
            field = rng.uniform(0, 1, (D, H, W)).astype(np.float32)
            field[rng.random((D, H, W)) < 0.4] = 100.0
        cases.append(dict(points=pts, values=rng.normal(size=n).astype(np.float32) if with_vals else None,
                          radius=rmul * dx, offset=rng.uniform(-dx, dx, 3).astype(np.float32), dx=dx,
                          field=field, weight=np.zeros_like(field) if with_w else None,
                          threshold=50.0 if thr else None))
    return cases


def main():
    O.build(ref=True)
    out = {}
    # 1. velocity splat (ScalarField::addPointValue + applyWeightField), all three components
    for tag, kw in (("a", dict(dims=(14, 11, 12), seed=21)), ("b", dict(dims=(9, 16, 10), seed=22, fill=0.6))):
        sc = scenes.random_box(**kw)
        d = dict(dims=np.array(sc.dims), dx=sc.dx, pos=sc.pos, vel=sc.vel)
        for c in range(3):
            f, w = O.ref_velocity_scalar_field(c, sc.dims, sc.dx, sc.pos, sc.vel)
            d[f"field{c}"] = f
            d[f"weight{c}"] = w
        np.savez_compressed(os.path.join(HERE, f"splat_{tag}.npz"), **d)
    # 2. pressure (PressureSolver::solve) on the advected, body-forced field
    for tag, kw in (("a", dict(dims=(14, 11, 12), seed=31)), ("b", dict(dims=(18, 14, 16), seed=32, solid_blocks=4))):
        sc = scenes.random_box(**kw)
        mat, pos, vel, ids = fluid_state(sc)
        u, v, w = O.advect_velocity_field(sc.dims, sc.dx, mat, pos, vel)
        u, v, w = O.body_force(sc.dims, mat, np.array(sc.gravity, np.float32), sc.dt, u, v, w)
        p, iters = O.ref_pressure_solve(sc.dims, sc.dx, 20.0, sc.dt, mat, u, v, w)
        np.savez_compressed(os.path.join(HERE, f"pressure_{tag}.npz"), dims=np.array(sc.dims), dx=sc.dx, dt=sc.dt,
                            mat=mat, u=u, v=v, w=w, pressure=p, iterations=iters)
    # 3. extrapolation (MACVelocityField::extrapolateVelocityField) and tricubic sampling
    sc = scenes.random_box(dims=(13, 12, 15), seed=41)
    mat, pos, vel, ids = fluid_state(sc)
    u, v, w = O.advect_velocity_field(sc.dims, sc.dx, mat, pos, vel)
    eu, ev, ew = O.ref_extrapolate(sc.dims, sc.dx, mat, 7, u, v, w)
    rng = np.random.default_rng(42)
    ext = np.array(sc.dims) * sc.dx
    pts = (rng.random((3000, 3)) * ext * 1.1 - 0.05 * ext).astype(np.float32)
    samples = O.ref_evaluate_velocity(sc.dims, sc.dx, eu, ev, ew, pts)
    np.savez_compressed(os.path.join(HERE, "extrapolate_sample.npz"), dims=np.array(sc.dims), dx=sc.dx, mat=mat,
                        u=u, v=v, w=w, eu=eu, ev=ev, ew=ew, points=pts, samples=samples)
    # 4. collision primitives (Collision::getLineSegmentVoxelIntersection, rayIntersectsAABB)
    dims = (12, 12, 12)
    mat = scenes.solid_border(dims)
    mat[5:7, 4:8, 6:9] = 2
    dx = 0.25
    p0 = (rng.random((400, 3)) * 2.0 + 0.3).astype(np.float32)
    p1 = (p0 + rng.normal(0, 0.6, size=p0.shape)).astype(np.float32)
    hit = np.zeros(len(p0), np.int32)
    vox = np.zeros((len(p0), 3), np.int32)
    for q in range(len(p0)):
        v3 = np.zeros(3, np.int32)
        hit[q] = O.ref().gfsref_segment_voxel(p0[q], p1[q], dx, *dims, np.ascontiguousarray(mat), v3)
        vox[q] = v3
    np.savez_compressed(os.path.join(HERE, "collision.npz"), dims=np.array(dims), dx=dx, mat=mat, p0=p0, p1=p1,
                        hit=hit, voxel=vox)
    # 5. general point splat (ScalarField::addPoint / addPointValue, the CLScalarField
    #    addPoints / addPointValues semantics): radii, offsets, no values, no weight
    #    field, points outside the grid, and a max-value threshold over a preset field
    d = {}
    for t, case in enumerate(point_splat_cases()):
        f, w = O.ref_add_point_values(case["points"], case.get("values"), case["radius"], case["offset"],
                                      case["dx"], case["field"], case.get("weight"), case.get("threshold"))
        for key, val in case.items():
            if val is not None:
                d[f"{t}_{key}"] = np.asarray(val)
        d[f"{t}_out_field"] = f
        if w is not None:
            d[f"{t}_out_weight"] = w
    np.savez_compressed(os.path.join(HERE, "point_splat.npz"), ncases=len(point_splat_cases()), **d)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
