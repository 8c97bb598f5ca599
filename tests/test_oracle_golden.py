"""Pins the oracle (oracle/gfs_oracle.c, the C restatement of the reference's CPU
path) to golden vectors written from the reference's own compiled code
(tests/golden/make_golden.py).  Every comparison is bit-exact: the restatement
keeps the reference's float/double casts and operation order.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


@pytest.mark.parametrize("name", ["splat_a.npz", "splat_b.npz"])
def test_splat_matches_reference(oracle_lib, name):
    O = oracle_lib
    d = _load(name)
    dims = tuple(int(x) for x in d["dims"])
    for c in range(3):
        field, mask = O.velocity_scalar_field(c, dims, float(d["dx"]), d["pos"], d["vel"])
        assert np.array_equal(field, d[f"field{c}"])
        assert np.array_equal(mask.astype(bool), d[f"weight{c}"] > 1e-9)


@pytest.mark.parametrize("name", ["pressure_a.npz", "pressure_b.npz"])
def test_pressure_matches_reference(oracle_lib, name):
    O = oracle_lib
    d = _load(name)
    dims = tuple(int(x) for x in d["dims"])
    p, iters, res = O.pressure_solve(dims, float(d["dx"]), 20.0, float(d["dt"]), d["mat"], d["u"], d["v"], d["w"])
    assert iters == int(d["iterations"])
    assert np.array_equal(p, d["pressure"])
    assert res < 1e-6


def test_extrapolate_and_sample_match_reference(oracle_lib):
    O = oracle_lib
    d = _load("extrapolate_sample.npz")
    dims = tuple(int(x) for x in d["dims"])
    eu, ev, ew = O.extrapolate(dims, d["mat"], 7, d["u"], d["v"], d["w"])
    assert np.array_equal(eu, d["eu"]) and np.array_equal(ev, d["ev"]) and np.array_equal(ew, d["ew"])
    s = O.evaluate_velocity(dims, float(d["dx"]), d["eu"], d["ev"], d["ew"], d["points"])
    assert np.array_equal(s, d["samples"])


def test_segment_voxel_matches_reference(oracle_lib):
    O = oracle_lib
    d = _load("collision.npz")
    dims = tuple(int(x) for x in d["dims"])
    mat = np.ascontiguousarray(d["mat"])
    for q in range(len(d["p0"])):
        v = np.zeros(3, np.int32)
        hit = O.lib().gfo_segment_voxel(d["p0"][q], d["p1"][q], float(d["dx"]), *dims, mat, v)
        assert hit == d["hit"][q]
        if hit:
            assert np.array_equal(v, d["voxel"][q])


def point_splat_cases():
    """The general point-splat fixture: inputs and the reference's outputs per case."""
    d = _load("point_splat.npz")
    cases = []
    for t in range(int(d["ncases"])):
        c = {k[len(f"{t}_"):]: d[k] for k in d.files if k.startswith(f"{t}_")}
        for k in ("radius", "dx", "threshold"):
            if k in c:
                c[k] = float(c[k])
        cases.append(c)
    return cases


def test_point_splat_matches_reference(oracle_lib):
    O = oracle_lib
    for c in point_splat_cases():
        f, w = O.splat_points(c["points"], c.get("values"), c["radius"], c["offset"], c["dx"], c["field"],
                              c.get("weight"), c.get("threshold"))
        assert np.array_equal(f, c["out_field"])
        if "out_weight" in c:
            assert np.array_equal(w, c["out_weight"])
