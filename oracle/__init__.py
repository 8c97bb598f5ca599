"""ctypes front-end of the oracle (test infrastructure only).

Two libraries live here:

* ``_build/libgfsoracle.so`` -- the C restatement in ``gfs_oracle.c`` of the
  reference's per-substep FLIP core (the checker for the CUDA path);
* ``_ref/libgfsref.so`` -- the reference's own CPU sources compiled where they
  lie, behind ``ref_shim.cpp`` (only where the reference tree exists; used to
  pin the restatement and to write the golden fixtures).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product path never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgfsoracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libgfsref.so")
# The reference's src/ directory is found through $GFS_REFERENCE_SRC, or the
# directory the last build(ref_src=...) recorded in the git-ignored _ref/.
REF_ENV = "GFS_REFERENCE_SRC"
REF_RECORD = os.path.join(HERE, "_ref", "reference_src.txt")

AIR, FLUID, SOLID = 0, 1, 2


def reference_src() -> str | None:
    """The reference's src/ directory, or None where it is not available."""
    p = os.environ.get(REF_ENV, "")
    if not p and os.path.exists(REF_RECORD):
        p = open(REF_RECORD).read().strip()
    return p if p and os.path.isfile(os.path.join(p, "pressuresolver.cpp")) else None

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i = ctypes.c_int
_i64 = ctypes.c_int64
_d = ctypes.c_double


class SubstepStats(ctypes.Structure):
    _fields_ = [("num_fluid_cells", ctypes.c_int64), ("num_particles", ctypes.c_int64),
                ("cg_iterations", ctypes.c_int), ("cg_max_resid", ctypes.c_double)]


def build(ref: bool | None = None, ref_src: str | None = None) -> None:
    """Compile the restatement and, when the reference's src/ is known (ref_src,
    recorded for later runs, or reference_src()), the shim over its sources."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref_src and os.path.isfile(os.path.join(ref_src, "pressuresolver.cpp")):
        os.makedirs(os.path.dirname(REF_RECORD), exist_ok=True)
        with open(REF_RECORD, "w") as f:
            f.write(os.path.abspath(ref_src) + "\n")
    src = reference_src()
    if ref is None:
        ref = src is not None
    if ref:
        if src is None:
            raise RuntimeError(f"the reference's src/ directory is unknown: set {REF_ENV}")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={src}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.gfo_splat_add.argtypes = [_f32p, _f32p, _i64, _d, _f32p, _d, _i, _i, _i, _f32p, _f32p]
        L.gfo_splat_points.argtypes = [_f32p, ctypes.c_void_p, _i64, _d, _f32p, _d, _i, _i, _i, _f32p,
                                       ctypes.c_void_p, _i, _d]
        L.gfo_apply_weight.argtypes = [_i64, _f32p, _f32p]
        L.gfo_velocity_scalar_field.argtypes = [_i, _i, _i, _i, _d, _f32p, _f32p, _i64, _f32p, _u8p]
        L.gfo_advect_velocity_field.argtypes = [_i, _i, _i, _d, _u8p, _f32p, _f32p, _i64, _f32p, _f32p, _f32p]
        L.gfo_velocity_from_splat.argtypes = [_i, _i, _i, _i, _u8p, _f32p, _f32p, _f32p]
        L.gfo_extrapolate.argtypes = [_i, _i, _i, _u8p, _i, _f32p, _f32p, _f32p]
        L.gfo_body_force.argtypes = [_i, _i, _i, _u8p, _f32p, _d, _f32p, _f32p, _f32p]
        L.gfo_pressure_solve.argtypes = [_i, _i, _i, _d, _d, _d, _u8p, _f32p, _f32p, _f32p, _d, _i,
                                         _f64p, ctypes.POINTER(_i), ctypes.POINTER(_d)]
        L.gfo_pressure_solve.restype = _i64
        L.gfo_pressure_residual.argtypes = [_i, _i, _i, _d, _d, _d, _u8p, _f32p, _f32p, _f32p, _f64p]
        L.gfo_pressure_residual.restype = _d
        L.gfo_pressure_to_grid.argtypes = [_i, _i, _i, _u8p, _f64p, _f32p]
        L.gfo_apply_pressure.argtypes = [_i, _i, _i, _d, _d, _d, _u8p, _f32p, _f32p, _f32p, _f32p]
        L.gfo_evaluate_velocity.argtypes = [_i, _i, _i, _d, _f32p, _f32p, _f32p, _f32p, _i64, _f32p]
        L.gfo_flip_update.argtypes = [_i, _i, _i, _d, _d, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                      _f32p, _i64, _f32p]
        L.gfo_advect_rk4.argtypes = [_i, _i, _i, _d, _f32p, _f32p, _f32p, _d, _f32p, _i64, _f32p]
        L.gfo_resolve_collisions.argtypes = [_i, _i, _i, _d, _u8p, _f32p, _i64, _f32p]
        L.gfo_segment_voxel.argtypes = [_f32p, _f32p, _d, _i, _i, _i, _u8p, _i32p]
        L.gfo_segment_voxel.restype = _i
        L.gfo_ray_aabb.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p]
        L.gfo_ray_aabb.restype = _i
        L.gfo_update_fluid_cells.argtypes = [_i, _i, _i, _d, _u8p, _f32p, _f32p, _u32p, _i64]
        L.gfo_update_fluid_cells.restype = _i64
        L.gfo_cap_particles_per_cell.argtypes = [_i, _i, _i, _d, _i, _f32p, _f32p, _u32p, _i64]
        L.gfo_cap_particles_per_cell.restype = _i64
        L.gfo_substep.argtypes = [_i, _i, _i, _d, _d, _f32p, _d, _d, _i, _i, _u8p, _f32p, _f32p,
                                  _u32p, _i64, _f32p, _f32p, _f32p, _f32p, ctypes.POINTER(SubstepStats)]
        L.gfo_substep.restype = _i64
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH) or reference_src() is not None


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            build(ref=True)
        L = ctypes.CDLL(REF_PATH)
        L.gfsref_add_point_values.argtypes = [_f32p, ctypes.c_void_p, _i64, _d, _f32p, _d, _i, _i, _i, _f32p,
                                              ctypes.c_void_p, _i, _d]
        L.gfsref_velocity_scalar_field.argtypes = [_i, _i, _i, _i, _d, _f32p, _f32p, _i64, _f32p, _f32p]
        L.gfsref_pressure_solve.argtypes = [_i, _i, _i, _d, _d, _d, _u8p, _f32p, _f32p, _f32p, _f64p]
        L.gfsref_pressure_solve.restype = _i
        L.gfsref_evaluate_velocity.argtypes = [_i, _i, _i, _d, _f32p, _f32p, _f32p, _f32p, _i64, _f32p]
        L.gfsref_extrapolate.argtypes = [_i, _i, _i, _d, _u8p, _i, _f32p, _f32p, _f32p]
        L.gfsref_segment_voxel.argtypes = [_f32p, _f32p, _d, _i, _i, _i, _u8p, _i32p]
        L.gfsref_segment_voxel.restype = _i
        L.gfsref_ray_aabb.argtypes = [_f32p, _f32p, _f32p, _d, _d, _d, _f32p]
        L.gfsref_ray_aabb.restype = _i
        _ref = L
    return _ref


# ----------------------------------------------------------------- helpers

def face_shape(dir_: int, ni: int, nj: int, nk: int):
    """numpy shape (k, j, i) of the face grid of component dir_."""
    return (nk + (dir_ == 2), nj + (dir_ == 1), ni + (dir_ == 0))


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def velocity_scalar_field(dir_, dims, dx, pos, vel):
    ni, nj, nk = dims
    field = np.zeros(face_shape(dir_, ni, nj, nk), np.float32)
    mask = np.zeros(field.shape, np.uint8)
    lib().gfo_velocity_scalar_field(dir_, ni, nj, nk, dx, _c(pos, np.float32), _c(vel, np.float32),
                                    len(pos), field, mask)
    return field, mask


def advect_velocity_field(dims, dx, mat, pos, vel):
    ni, nj, nk = dims
    u = np.zeros(face_shape(0, *dims), np.float32)
    v = np.zeros(face_shape(1, *dims), np.float32)
    w = np.zeros(face_shape(2, *dims), np.float32)
    lib().gfo_advect_velocity_field(ni, nj, nk, dx, _c(mat, np.uint8), _c(pos, np.float32),
                                    _c(vel, np.float32), len(pos), u, v, w)
    return u, v, w


def extrapolate(dims, mat, layers, u, v, w):
    u, v, w = (np.array(a, np.float32, copy=True) for a in (u, v, w))
    lib().gfo_extrapolate(*dims, _c(mat, np.uint8), layers, u, v, w)
    return u, v, w


def body_force(dims, mat, g, dt, u, v, w):
    u, v, w = (np.array(a, np.float32, copy=True) for a in (u, v, w))
    lib().gfo_body_force(*dims, _c(mat, np.uint8), _c(g, np.float32), dt, u, v, w)
    return u, v, w


def pressure_solve(dims, dx, density, dt, mat, u, v, w, tol=1e-6, max_iters=200):
    mat = _c(mat, np.uint8)
    F = int((mat == FLUID).sum())
    p = np.zeros(max(F, 1), np.float64)
    it = _i(0)
    res = _d(0.0)
    lib().gfo_pressure_solve(*dims, dx, density, dt, mat, _c(u, np.float32), _c(v, np.float32),
                             _c(w, np.float32), tol, max_iters, p, ctypes.byref(it), ctypes.byref(res))
    return p[:F], it.value, res.value


def pressure_residual(dims, dx, density, dt, mat, u, v, w, p):
    """max|b - A p| with the reference's b and stencil."""
    return lib().gfo_pressure_residual(*dims, dx, density, dt, _c(mat, np.uint8), _c(u, np.float32),
                                       _c(v, np.float32), _c(w, np.float32),
                                       _c(p if len(p) else np.zeros(1), np.float64))


def pressure_to_grid(dims, mat, p):
    g = np.zeros(mat.shape, np.float32)
    lib().gfo_pressure_to_grid(*dims, _c(mat, np.uint8), _c(p if len(p) else np.zeros(1), np.float64), g)
    return g


def apply_pressure(dims, dx, density, dt, mat, pgrid, u, v, w):
    u, v, w = (np.array(a, np.float32, copy=True) for a in (u, v, w))
    lib().gfo_apply_pressure(*dims, dx, density, dt, _c(mat, np.uint8), _c(pgrid, np.float32), u, v, w)
    return u, v, w


def evaluate_velocity(dims, dx, u, v, w, pos):
    out = np.zeros((len(pos), 3), np.float32)
    lib().gfo_evaluate_velocity(*dims, dx, _c(u, np.float32), _c(v, np.float32), _c(w, np.float32),
                                _c(pos, np.float32), len(pos), out)
    return out


def flip_update(dims, dx, ratio_pic, new, old, pos, vel):
    vel = np.array(vel, np.float32, copy=True)
    lib().gfo_flip_update(*dims, dx, ratio_pic, *(_c(a, np.float32) for a in new),
                          *(_c(a, np.float32) for a in old), _c(pos, np.float32), len(pos), vel)
    return vel


def advect_rk4(dims, dx, u, v, w, dt, pos):
    out = np.zeros((len(pos), 3), np.float32)
    lib().gfo_advect_rk4(*dims, dx, _c(u, np.float32), _c(v, np.float32), _c(w, np.float32), dt,
                         _c(pos, np.float32), len(pos), out)
    return out


def resolve_collisions(dims, dx, mat, p0, p1):
    p1 = np.array(p1, np.float32, copy=True)
    lib().gfo_resolve_collisions(*dims, dx, _c(mat, np.uint8), _c(p0, np.float32), len(p0), p1)
    return p1


def substep(dims, dx, dt, g, mat, pos, vel, ids, density=20.0, ratio_pic=float(np.float32(0.05)),
            num_layers=7, max_per_cell=100):
    """One full substep of the restatement; returns a dict of the new state."""
    ni, nj, nk = dims
    mat = np.array(mat, np.uint8, copy=True)
    pos = np.array(pos, np.float32, copy=True)
    vel = np.array(vel, np.float32, copy=True)
    ids = np.array(ids, np.uint32, copy=True)
    u = np.zeros(face_shape(0, *dims), np.float32)
    v = np.zeros(face_shape(1, *dims), np.float32)
    w = np.zeros(face_shape(2, *dims), np.float32)
    pg = np.zeros(mat.shape, np.float32)
    st = SubstepStats()
    n = lib().gfo_substep(ni, nj, nk, dx, dt, _c(g, np.float32), density, ratio_pic, num_layers,
                          max_per_cell, mat, pos, vel, ids, len(pos), u, v, w, pg, ctypes.byref(st))
    return dict(mat=mat, pos=pos[:n], vel=vel[:n], ids=ids[:n], u=u, v=v, w=w, pressure=pg,
                num_fluid_cells=st.num_fluid_cells, cg_iterations=st.cg_iterations,
                cg_max_resid=st.cg_max_resid)


def _splat_args(points, values, offset, field, weight):
    pts = _c(points, np.float32).reshape(-1, 3)
    vals = None if values is None else _c(values, np.float32)
    off = _c(offset, np.float32)
    f = _c(field, np.float32).copy()
    w = None if weight is None else _c(weight, np.float32).copy()
    D, H, W = f.shape
    vp = None if vals is None else vals.ctypes.data_as(ctypes.c_void_p)
    wp = None if w is None else w.ctypes.data_as(ctypes.c_void_p)
    return pts, vals, off, f, w, (W, H, D), vp, wp


def splat_points(points, values, radius, offset, dx, field, weight=None, threshold=None):
    """CLScalarField::addPointValues (values given) / addPoints (values None) into
    copies of field / weight; returns (field, weight)."""
    pts, vals, off, f, w, (W, H, D), vp, wp = _splat_args(points, values, offset, field, weight)
    lib().gfo_splat_points(pts, vp, len(pts), float(radius), off, float(dx), W, H, D, f, wp,
                           int(threshold is not None), float(threshold or 0.0))
    return f, w


# ------------------------------------------------- reference shim wrappers

def ref_add_point_values(points, values, radius, offset, dx, field, weight=None, threshold=None):
    """The reference's ScalarField::addPoint / addPointValue on copies of field / weight."""
    pts, vals, off, f, w, (W, H, D), vp, wp = _splat_args(points, values, offset, field, weight)
    ref().gfsref_add_point_values(pts, vp, len(pts), float(radius), off, float(dx), W, H, D, f, wp,
                                  int(threshold is not None), float(threshold or 0.0))
    return f, w


def ref_velocity_scalar_field(dir_, dims, dx, pos, vel):
    ni, nj, nk = dims
    field = np.zeros(face_shape(dir_, ni, nj, nk), np.float32)
    weight = np.zeros(field.shape, np.float32)
    ref().gfsref_velocity_scalar_field(dir_, ni, nj, nk, dx, _c(pos, np.float32), _c(vel, np.float32),
                                       len(pos), field, weight)
    return field, weight


def ref_pressure_solve(dims, dx, density, dt, mat, u, v, w):
    mat = _c(mat, np.uint8)
    F = int((mat == FLUID).sum())
    p = np.zeros(max(F, 1), np.float64)
    it = ref().gfsref_pressure_solve(*dims, dx, density, dt, mat, _c(u, np.float32), _c(v, np.float32),
                                     _c(w, np.float32), p)
    return p[:F], it


def ref_evaluate_velocity(dims, dx, u, v, w, pos):
    out = np.zeros((len(pos), 3), np.float32)
    ref().gfsref_evaluate_velocity(*dims, dx, _c(u, np.float32), _c(v, np.float32), _c(w, np.float32),
                                   _c(pos, np.float32), len(pos), out)
    return out


def ref_extrapolate(dims, dx, mat, layers, u, v, w):
    u, v, w = (np.array(a, np.float32, copy=True) for a in (u, v, w))
    ref().gfsref_extrapolate(*dims, dx, _c(mat, np.uint8), layers, u, v, w)
    return u, v, w
