"""The host half of the fluid-source stage (csrc/sources.cu source_geometry: the
overlapping-cell bounds, the AABB fitted to the grid, its index bounds and
offset) against the oracle's restatement of Grid3d::getGridIndexBounds and
fitAABBtoGrid (grid3d.h:350-371, 426-439, 485-502), which the reference's own
results pin (tests/test_fluidsource.py).  The function is called in libgfs.so
through its C++ symbol; no GPU is involved.

Cases: every source of the committed fixtures, and seeded random spheres and
cuboids across the grid's faces (negative positions, boxes past the far
corner, radii of zero and below).
"""
import ctypes
import json
import os
import random
import shutil

import numpy as np
import pytest

from gridfluidsim3d_gb300 import _lib
from oracle import fluidsource as F

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIMS = (16, 14, 12)
DX = 0.25


class SrcGeom(ctypes.Structure):
    # the layout of struct SrcGeom in csrc/sources.cu
    _fields_ = [("sphere", ctypes.c_int), ("c", ctypes.c_float * 3), ("rsq", ctypes.c_double),
                ("g1", ctypes.c_int * 3), ("n1", ctypes.c_int * 3), ("f1", ctypes.c_int * 3),
                ("nf", ctypes.c_int * 3), ("fp", ctypes.c_float * 3), ("fw", ctypes.c_double * 3),
                ("off", ctypes.c_float * 3), ("vel", ctypes.c_float * 3)]


@pytest.fixture(scope="module")
def geometry():
    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no CUDA toolkit")
    from gridfluidsim3d_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    fn = getattr(lib, "_ZN3gfs15source_geometryERK16gfs_fluid_sourcediii")
    fn.argtypes = [ctypes.POINTER(_lib.FluidSourceC), ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    fn.restype = SrcGeom

    def call(src, dx, dims):
        c = _lib.FluidSourceC()
        c.shape = 0 if src["shape"] == "sphere" else 1
        c.outflow, c.active = int(src.get("outflow", False)), 1
        c.position = (ctypes.c_float * 3)(*src["position"])
        c.radius = float(src.get("radius", 0.0))
        c.size = (ctypes.c_double * 3)(*src.get("size", (0.0, 0.0, 0.0)))
        c.velocity = (ctypes.c_float * 3)(*src["velocity"])
        return fn(ctypes.byref(c), dx, *dims)
    return call


def oracle_geometry(src, dx, dims):
    f32 = np.float32
    if src["shape"] == "sphere":
        r = max(float(src["radius"]), 0.0)
        lo, hi = F.bounds_sphere([f32(x) for x in src["position"]], r, dx, dims)
    else:
        lo, hi = F.bounds_box([f32(x) for x in src["position"]], src["size"], dx, dims)
    bp, bw = F.aabb(src)
    fp, fw = F.fit_box(bp, bw, dx, dims)
    f1, f2 = F.bounds_box(fp, fw, dx, dims)
    return {
        "g1": lo, "n1": [max(hi[a] - lo[a] + 1, 0) for a in range(3)],
        "f1": f1, "nf": [max(f2[a] - f1[a] + 1, 0) for a in range(3)],
        "fp": [float(x) for x in fp], "fw": [float(x) for x in fw],
        "off": [float(F.index_to_pos(f1[a], dx)) for a in range(3)],
    }


def check(geometry, src, dx=DX, dims=DIMS):
    got = geometry(src, dx, dims)
    want = oracle_geometry(src, dx, dims)
    n1 = list(got.n1)
    assert n1 == want["n1"], (src, n1, want["n1"])
    if all(n1):                       # an empty box's first index is not used
        assert list(got.g1) == want["g1"], src
    assert list(got.nf) == want["nf"], src
    if all(want["nf"]):
        assert list(got.f1) == want["f1"], src
        assert [float(x) for x in got.off] == want["off"], src
    assert [float(x) for x in got.fp] == want["fp"], src
    assert list(got.fw) == want["fw"], src
    assert got.sphere == (src["shape"] == "sphere")


def fixture_sources():
    out = []
    for name in ("fluidsource_sources.json", "fluidsource_edge_sources.json"):
        out += json.load(open(os.path.join(G, name)))
    return out


def test_fixture_sources(geometry):
    for src in fixture_sources():
        check(geometry, src)


def test_random_sources_across_the_faces(geometry):
    rnd = random.Random(7)
    ext = [DIMS[a] * DX for a in range(3)]
    for _ in range(400):
        pos = [rnd.uniform(-1.0, ext[a] + 1.0) for a in range(3)]
        vel = [rnd.uniform(-1, 1) for _ in range(3)]
        if rnd.random() < 0.5:
            src = {"shape": "sphere", "position": pos, "radius": rnd.choice([0.0, -0.5, rnd.uniform(0, 1.5)]),
                   "velocity": vel}
        else:
            src = {"shape": "cuboid", "position": pos, "size": [rnd.uniform(0, 2.0) for _ in range(3)],
                   "velocity": vel}
        check(geometry, src)
