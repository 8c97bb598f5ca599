"""Host-side mirror of the reference's interfaces for the FLIP substep path.

The classes keep the names and argument meaning of the reference's C++ /
pyfluid API and forward to libgfs's C ABI:

* ``CLScalarField``     -- CLScalarField (clscalarfield.h:67-125): point splats
* ``ParticleAdvector``  -- ParticleAdvector (particleadvector.h:62-110):
                           tricubic interpolation and RK1..RK4 advection
* ``PressureSolver``    -- PressureSolver::solve (pressuresolver.h:113-117) with
                           ``PressureSolverParameters`` (:38-47)
* ``MACVelocityField``  -- the three face grids (macvelocityfield.h)
* ``FluidSimulation``   -- the device-resident substep behind a subset of
                           pyfluid's FluidSimulation (pyfluid/fluidsimulation.py):
                           ``update(dt)`` runs one substep of the full frame dt,
                           as the reference does (its CFL limit never binds,
                           fluidsimulation.cpp:3392-3451).

Arrays are numpy, laid out like the reference's Array3d (index i + W*(j + H*k),
numpy shape (k, j, i)).  Errors raise GFSError (a RuntimeError), as pyfluid
raises RuntimeError from its bindings.
"""
from __future__ import annotations

import atexit
import ctypes
import os
import weakref

import numpy as np

from . import _lib, config
from ._lib import GFSError, PRECISION_MIXED, PRECISION_PLAIN, SimParams, StepStats

AIR, FLUID, SOLID = 0, 1, 2


def _arr(a, dtype, shape=None, name="array"):
    a = np.asarray(a)
    if a.dtype != dtype or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=dtype)
    if shape is not None and a.size != int(np.prod(shape)):
        raise GFSError(_lib.GFS_ERR_INVALID, name, f"expected {int(np.prod(shape))} elements, got {a.size}")
    return a


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def face_shape(d, isize, jsize, ksize):
    return (ksize + (d == 2), jsize + (d == 1), isize + (d == 0))


class GridIndex:
    """A cell index (i, j, k), as pyfluid's GridIndex (pyfluid/gridindex.py):
    attributes i, j, k, indexable and iterable in that order."""

    __slots__ = ("i", "j", "k")

    def __init__(self, i=0, j=0, k=0):
        if isinstance(i, GridIndex):
            i, j, k = i.i, i.j, i.k
        self.i, self.j, self.k = int(i), int(j), int(k)

    def __getitem__(self, a):
        if not isinstance(a, int):
            raise TypeError("index must be an integer")
        if not 0 <= a <= 2:
            raise IndexError("index must be in [0, 2]")
        return (self.i, self.j, self.k)[a]

    def __setitem__(self, a, value):
        if not isinstance(a, int):
            raise TypeError("index must be an integer")
        if not 0 <= a <= 2:
            raise IndexError("index must be in [0, 2]")
        setattr(self, "ijk"[a], int(value))

    def __iter__(self):
        return iter((self.i, self.j, self.k))

    def __eq__(self, other):
        return isinstance(other, GridIndex) and tuple(self) == tuple(other)

    def __hash__(self):
        return hash((self.i, self.j, self.k))

    def __repr__(self):
        return f"GridIndex({self.i}, {self.j}, {self.k})"


# Live contexts, closed at interpreter exit (each closes what was built on it first).
_CONTEXTS = weakref.WeakSet()


@atexit.register
def _close_all():
    for c in list(_CONTEXTS):
        try:
            c.close()
        except Exception:
            pass


class Context:
    """One CUDA device and stream (replaces the reference's OpenCL set-up).

    A context outlives everything built on it: close() first closes the
    simulations (and their rollouts) that use it, and every live context is
    closed at interpreter exit in that order."""

    _default = None

    def __init__(self, device: int = 0):
        L = _lib.lib()
        h = ctypes.c_void_p()
        L.gfs_ctx_create(device, ctypes.byref(h))
        self._h = h
        self.device = device
        self._dependents = weakref.WeakSet()
        _CONTEXTS.add(self)

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        _lib.lib().gfs_ctx_stream(self._h, ctypes.byref(s))
        return s.value or 0

    def synchronize(self):
        _lib.lib().gfs_ctx_synchronize(self._h)

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        _lib.lib().gfs_ctx_device_name(self._h, buf, 256)
        return buf.value.decode()

    def launch_count(self) -> int:
        c = ctypes.c_int64()
        _lib.lib().gfs_ctx_launch_count(self._h, ctypes.byref(c))
        return c.value

    # -- wavefront kernels of the MIC(0) triangular solves (gfs_ctx_set_sweep_kernel) --
    def set_sweep_kernel(self, kind: int):
        """SWEEP_AUTO (default), SWEEP_BLOCK, SWEEP_CLUSTER_4X2, SWEEP_CLUSTER_2X2 or SWEEP_WARP (FP32 solves)."""
        _lib.lib().gfs_ctx_set_sweep_kernel(self._h, int(kind))

    def last_sweep_kernel(self) -> int:
        k = ctypes.c_int()
        _lib.lib().gfs_ctx_last_sweep_kernel(self._h, ctypes.byref(k))
        return k.value

    def set_wait_limit(self, polls: int = 0):
        """Bound of every wavefront wait in polls (0: the library default)."""
        _lib.lib().gfs_ctx_set_wait_limit(self._h, int(polls))

    def inject_wait_timeout(self, sweeps: int = 1):
        """Make the next `sweeps` wavefront launches wait for a tag nobody writes
        (test hook of the GFS_ERR_TIMEOUT path; every wait ends at its bound)."""
        _lib.lib().gfs_ctx_inject_wait_timeout(self._h, int(sweeps))

    def close(self):
        for d in list(getattr(self, "_dependents", ())):
            d.close()
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().gfs_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MACVelocityField:
    """U (ni+1, nj, nk), V (ni, nj+1, nk), W (ni, nj, nk+1) float grids."""

    def __init__(self, isize, jsize, ksize, dx, u=None, v=None, w=None):
        self.isize, self.jsize, self.ksize, self.dx = int(isize), int(jsize), int(ksize), float(dx)
        dims = (self.isize, self.jsize, self.ksize)
        self.u = _arr(u, np.float32, face_shape(0, *dims), "U").reshape(face_shape(0, *dims)) if u is not None \
            else np.zeros(face_shape(0, *dims), np.float32)
        self.v = _arr(v, np.float32, face_shape(1, *dims), "V").reshape(face_shape(1, *dims)) if v is not None \
            else np.zeros(face_shape(1, *dims), np.float32)
        self.w = _arr(w, np.float32, face_shape(2, *dims), "W").reshape(face_shape(2, *dims)) if w is not None \
            else np.zeros(face_shape(2, *dims), np.float32)

    def get_grid_dimensions(self):
        return self.isize, self.jsize, self.ksize

    def get_grid_cell_size(self):
        return self.dx


class CLScalarField:
    """Splat accelerator (CLScalarField, clscalarfield.h:67-125), CUDA backed.

    Methods keep the reference's names in snake case.  The device/work-load
    toggles of the reference's OpenCL path are kept for source compatibility;
    disable_opencl() leaves no backend (there is no CPU path here), so compute
    calls then raise instead of silently running something else."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        self._initialized = False
        self._enabled = True
        self._thr = None
        self._workload = 10000

    def initialize(self) -> bool:
        self._initialized = True
        return True

    # -- CLScalarField::setMaxScalarFieldValueThreshold & co (clscalarfield.cpp:303-318)
    def set_max_scalar_field_value_threshold(self, val: float | None = None):
        self._thr = None if val is None else float(np.float32(val))

    def is_max_scalar_field_value_threshold_set(self) -> bool:
        return self._thr is not None

    def get_max_scalar_field_value_threshold(self) -> float:
        return 0.0 if self._thr is None else self._thr

    # -- device toggles (clscalarfield.cpp:320-517)
    def enable_opencl(self):
        self._enabled = True

    def disable_opencl(self):
        self._enabled = False

    def is_opencl_enabled(self) -> bool:
        return self._enabled

    def is_using_gpu(self) -> bool:
        return self._enabled

    def is_using_cpu(self) -> bool:
        return False

    def get_device_info(self) -> str:
        return self.ctx.device_name()

    def get_kernel_work_load_size(self) -> int:
        return self._workload

    def set_kernel_work_load_size(self, n: int):
        self._workload = int(n)

    def _check(self, func):
        if not self._enabled:
            raise GFSError(_lib.GFS_ERR_STATE, func, "accelerator disabled (disable_opencl); no CPU path is provided")

    def _splat(self, func, points, values, radius, offset, dx, field, weight):
        self._check(func)
        pts = _arr(points, np.float32).reshape(-1, 3)
        vals = None
        if values is not None:
            vals = _arr(values, np.float32)
            if len(vals) != len(pts):
                raise GFSError(_lib.GFS_ERR_INVALID, func, "points and values differ in length")
        for name, a in (("field", field), ("weightfield", weight)):
            if a is not None and (a.dtype != np.float32 or not a.flags.c_contiguous or a.ndim != 3):
                raise GFSError(_lib.GFS_ERR_INVALID, func, f"{name} must be a contiguous 3-D float32 array")
        if weight is not None and weight.shape != field.shape:
            raise GFSError(_lib.GFS_ERR_INVALID, func, "scalarfield and weightfield differ in shape")
        D, H, W = field.shape
        off = _arr(offset, np.float32)
        thr = self._thr
        _lib.lib().gfs_scalar_field_add_point_values(
            self.ctx.handle, _p(pts), _p(vals) if vals is not None else None, len(pts), float(radius), _p(off),
            float(dx), W, H, D, _p(field), _p(weight) if weight is not None else None, int(thr is not None),
            float(thr or 0.0))

    def add_points(self, points, radius, offset, dx, field):
        """CLScalarField::addPoints (clscalarfield.cpp:68-122): field += w for every
        node within `radius` of point - offset.  `field` is updated in place."""
        self._splat("add_points", points, None, radius, offset, dx, field, None)

    def add_point_values(self, points, values, radius, offset, dx, scalarfield, weightfield=None):
        """CLScalarField::addPointValues (clscalarfield.cpp:144-267): scalarfield +=
        w*v (and weightfield += w) for every node within `radius` of point - offset.
        The arrays are updated in place."""
        self._splat("add_point_values", points, values, radius, offset, dx, scalarfield, weightfield)

    def velocity_scalar_field(self, dir_, isize, jsize, ksize, dx, positions, velocities):
        """FluidSimulation::_computeVelocityScalarField for one MAC component:
        returns (field, is_set)."""
        pos = _arr(positions, np.float32).reshape(-1, 3)
        vel = _arr(velocities, np.float32).reshape(-1, 3)
        shape = face_shape(dir_, isize, jsize, ksize)
        field = np.zeros(shape, np.float32)
        is_set = np.zeros(shape, np.uint8)
        _lib.lib().gfs_velocity_scalar_field(self.ctx.handle, dir_, isize, jsize, ksize, float(dx), _p(pos), _p(vel),
                                             len(pos), _p(field), _p(is_set))
        return field, is_set.astype(bool)


class ParticleAdvector:
    """G2P sampling and RK advection (ParticleAdvector, particleadvector.h:62-110)."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or Context.default()

    def initialize(self) -> bool:
        return True

    def _field(self, vfield: MACVelocityField):
        return (vfield.isize, vfield.jsize, vfield.ksize, vfield.dx, _arr(vfield.u, np.float32),
                _arr(vfield.v, np.float32), _arr(vfield.w, np.float32))

    def tricubic_interpolate(self, particles, vfield: MACVelocityField):
        pts = _arr(particles, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        ni, nj, nk, dx, u, v, w = self._field(vfield)
        _lib.lib().gfs_tricubic_interpolate(self.ctx.handle, ni, nj, nk, dx, _p(u), _p(v), _p(w), _p(pts), len(pts),
                                            _p(out))
        return out

    def _advect(self, order, particles, vfield, dt):
        pts = _arr(particles, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        ni, nj, nk, dx, u, v, w = self._field(vfield)
        _lib.lib().gfs_advect_particles(self.ctx.handle, order, ni, nj, nk, dx, _p(u), _p(v), _p(w), float(dt),
                                        _p(pts), len(pts), _p(out))
        return out

    def advect_particles_rk4(self, particles, vfield, dt):
        return self._advect(4, particles, vfield, dt)

    def advect_particles_rk3(self, particles, vfield, dt):
        return self._advect(3, particles, vfield, dt)

    def advect_particles_rk2(self, particles, vfield, dt):
        return self._advect(2, particles, vfield, dt)

    def advect_particles_rk1(self, particles, vfield, dt):
        return self._advect(1, particles, vfield, dt)


class PressureSolverParameters:
    """PressureSolverParameters (pressuresolver.h:38-47).  The fluid cells are the
    material grid's fluid cells in lexicographic order."""

    def __init__(self, cellwidth, density, delta_time, material_grid, velocity_field: MACVelocityField):
        self.cellwidth = float(cellwidth)
        self.density = float(density)
        self.delta_time = float(delta_time)
        self.material_grid = material_grid
        self.velocity_field = velocity_field


class PressureSolver:
    """MICCG(0) pressure solve (PressureSolver::solve, pressuresolver.cpp:116)."""

    def __init__(self, ctx: Context | None = None, precision: int = PRECISION_PLAIN, tol: float = 1e-6,
                 max_iterations: int = 200):
        self.ctx = ctx or Context.default()
        self.precision = precision
        self.tol = tol
        self.max_iterations = max_iterations
        self.iterations = None
        self.max_residual = None

    def solve(self, params: PressureSolverParameters):
        vf = params.velocity_field
        mat = _arr(params.material_grid, np.uint8)
        F = ctypes.c_int64(0)
        L = _lib.lib()
        ni, nj, nk = vf.isize, vf.jsize, vf.ksize
        L.gfs_pressure_solve(self.ctx.handle, ni, nj, nk, params.cellwidth, params.density, params.delta_time,
                             _p(mat), None, None, None, self.precision, self.tol, self.max_iterations, None,
                             ctypes.byref(F), None, None)
        out = np.zeros(max(F.value, 1), np.float64)
        it = ctypes.c_int(0)
        res = ctypes.c_double(0.0)
        u, v, w = (_arr(a, np.float32) for a in (vf.u, vf.v, vf.w))
        L.gfs_pressure_solve(self.ctx.handle, ni, nj, nk, params.cellwidth, params.density, params.delta_time,
                             _p(mat), _p(u), _p(v), _p(w), self.precision, self.tol, self.max_iterations, _p(out),
                             ctypes.byref(F), ctypes.byref(it), ctypes.byref(res))
        self.iterations = it.value
        self.max_residual = res.value
        return out[:F.value]


class FluidSimulation:
    """Device-resident FLIP simulation behind a subset of pyfluid's FluidSimulation.

    ``update(dt)`` runs one substep of length dt (stages 1, 5-9, 11, 12 of
    FluidSimulation::_stepFluid), with the queued fluid cells and the fluid
    sources at its start; meshing, level set, diffuse particles and autosave are
    not part of this core.
    """

    def __init__(self, isize, jsize, ksize, dx, max_particles=None, ctx: Context | None = None):
        """max_particles: the device capacity; None reserves 8 per cell, the most
        initialize() can seed."""
        self.ctx = ctx or Context.default()
        self.isize, self.jsize, self.ksize, self.dx = int(isize), int(jsize), int(ksize), float(dx)
        if max_particles is None:
            max_particles = 8 * self.isize * self.jsize * self.ksize
        h = ctypes.c_void_p()
        _lib.lib().gfs_sim_create(self.ctx.handle, self.isize, self.jsize, self.ksize, self.dx, int(max_particles),
                                  ctypes.byref(h))
        self._h = h
        self._dependents = weakref.WeakSet()   # rollouts built on this simulation
        if getattr(self.ctx, "_dependents", None) is not None:
            self.ctx._dependents.add(self)
        self._params = SimParams()
        _lib.lib().gfs_sim_default_params(ctypes.byref(self._params))
        self.last_stats = None
        self.current_frame = 0
        self._autosave = False
        self._fluid_points = []     # FluidSimulation::_fluidPoints (fluidsimulation.h:1112)
        self._fluid_cuboids = []    # FluidSimulation::_fluidCuboids
        self._initialized = False

    # -- scene set-up (fluidsimulation.cpp:48-55, 703-765, 845-885; pyfluid/fluidsimulation.py:89-101,
    #    609-671) --
    def add_implicit_fluid_point(self, x, y=None, z=None, radius=None):
        """addImplicitFluidPoint(x, y, z, r) or (p, r): a sphere of fluid seeded by initialize()."""
        if radius is None and z is None:
            (x, y, z), radius = x, y
        if not radius >= 0.0:
            raise GFSError(_lib.GFS_ERR_INVALID, "add_implicit_fluid_point", "radius must be >= 0")
        if self._initialized:
            raise GFSError(_lib.GFS_ERR_STATE, "add_implicit_fluid_point", "the simulation is already initialized")
        self._fluid_points.append((float(x), float(y), float(z), float(radius)))

    def add_fluid_cuboid(self, *args):
        """addFluidCuboid: an AABB (position, width, height, depth attributes, as
        pyfluid's AABB), (x, y, z, w, h, d), (p, w, h, d) or two opposite corners."""
        if len(args) == 1:
            b = args[0]
            p, w, h, d = b.position, b.width, b.height, b.depth
        elif len(args) == 2:
            p1, p2 = (tuple(float(c) for c in a) for a in args)
            p = tuple(min(a, b) for a, b in zip(p1, p2))
            w, h, d = (abs(b - a) for a, b in zip(p1, p2))
        elif len(args) == 4:
            p, w, h, d = args
        elif len(args) == 6:
            p, (w, h, d) = args[:3], args[3:]
        else:
            raise TypeError("add_fluid_cuboid takes an AABB, two corners, (p, w, h, d) or (x, y, z, w, h, d)")
        if not (w >= 0 and h >= 0 and d >= 0):
            raise GFSError(_lib.GFS_ERR_INVALID, "add_fluid_cuboid", "dimensions must be >= 0")
        if self._initialized:
            raise GFSError(_lib.GFS_ERR_STATE, "add_fluid_cuboid", "the simulation is already initialized")
        self._fluid_cuboids.append(tuple(float(c) for c in p) + (float(w), float(h), float(d)))

    def add_solid_cells(self, cell_list):
        """addSolidCells: cells (GridIndex objects or (i, j, k) rows) become solid."""
        c = self._cells(cell_list)
        _lib.lib().gfs_sim_add_solid_cells(self._h, _p(c), len(c))

    def remove_solid_cells(self, cell_list):
        """removeSolidCells: solid cells of the list become air."""
        c = self._cells(cell_list)
        _lib.lib().gfs_sim_remove_solid_cells(self._h, _p(c), len(c))

    def initialize(self):
        """FluidSimulation::initialize: solid border, then the fluid seeded from the
        implicit points and cuboids (8 particles per full cell on the 2x2x2
        sub-lattice, sub-cell particles at the surface), with the jitter of
        set_marker_particle_jitter (factor 0.1 by default)."""
        if self._initialized:
            return
        pts = np.ascontiguousarray(np.array(self._fluid_points, np.float64).reshape(-1, 4))
        cub = np.ascontiguousarray(np.array(self._fluid_cuboids, np.float64).reshape(-1, 6))
        n = ctypes.c_int64(0)
        _lib.lib().gfs_sim_initialize(self._h, _p(pts), len(pts), _p(cub), len(cub), ctypes.byref(n))
        self._initialized = True

    def is_initialized(self) -> bool:
        return self._initialized

    # -- parameters (fluidsimulation.h:146-446 setters) --
    def _push(self):
        _lib.lib().gfs_sim_set_params(self._h, ctypes.byref(self._params))

    @property
    def density(self):
        return self._params.density

    @density.setter
    def density(self, value):
        if not value > 0:
            raise GFSError(_lib.GFS_ERR_INVALID, "density", "must be > 0")
        self._params.density = float(value)
        self._push()

    @property
    def precision(self):
        return self._params.precision

    @precision.setter
    def precision(self, value):
        self._params.precision = int(value)
        self._push()

    @property
    def pressure_tolerance(self):
        return self._params.tol

    @pressure_tolerance.setter
    def pressure_tolerance(self, value):
        self._params.tol = float(value)
        self._push()

    @property
    def max_cg_iterations(self):
        return self._params.max_cg_iterations

    @max_cg_iterations.setter
    def max_cg_iterations(self, value):
        self._params.max_cg_iterations = int(value)
        self._push()

    def add_body_force(self, fx, fy=None, fz=None):
        if fy is None:
            fx, fy, fz = fx
        g = self._params.gravity
        self._params.gravity = (ctypes.c_float * 3)(g[0] + fx, g[1] + fy, g[2] + fz)
        self._push()

    def reset_body_force(self):
        self._params.gravity = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
        self._push()

    # -- state --
    def set_material_grid(self, mat):
        mat = _arr(mat, np.uint8, (self.ksize, self.jsize, self.isize), "material")
        _lib.lib().gfs_sim_set_material(self._h, _p(mat))

    def get_material_grid(self):
        out = np.zeros((self.ksize, self.jsize, self.isize), np.uint8)
        _lib.lib().gfs_sim_get_material(self._h, _p(out))
        return out

    def set_marker_particles(self, positions, velocities=None, ids=None):
        pos = _arr(positions, np.float32).reshape(-1, 3)
        vel = _arr(velocities, np.float32).reshape(-1, 3) if velocities is not None else None
        idv = _arr(ids, np.uint32) if ids is not None else None
        _lib.lib().gfs_sim_set_particles(self._h, _p(pos), _p(vel), _p(idv), len(pos))

    def get_num_marker_particles(self) -> int:
        n = ctypes.c_int64(0)
        _lib.lib().gfs_sim_num_particles(self._h, ctypes.byref(n))
        return n.value

    def get_marker_particles(self):
        """(positions, velocities, ids) in the device's (cell, id) order."""
        n = self.get_num_marker_particles()
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        ids = np.zeros(n, np.uint32)
        nn = ctypes.c_int64(0)
        if n:
            _lib.lib().gfs_sim_get_particles(self._h, _p(pos), _p(vel), _p(ids), ctypes.byref(nn))
        return pos, vel, ids

    def get_marker_particle_positions(self):
        return self.get_marker_particles()[0]

    def get_marker_particle_velocities(self):
        return self.get_marker_particles()[1]

    def get_velocity_field(self) -> MACVelocityField:
        f = MACVelocityField(self.isize, self.jsize, self.ksize, self.dx)
        _lib.lib().gfs_sim_get_velocity_field(self._h, _p(f.u), _p(f.v), _p(f.w))
        return f

    def get_pressure_grid(self):
        out = np.zeros((self.ksize, self.jsize, self.isize), np.float32)
        _lib.lib().gfs_sim_get_pressure_grid(self._h, _p(out))
        return out

    def add_marker_particle_points(self, radius, offset, dx, field, threshold=None):
        """CLScalarField::addPoints of the simulation's device-resident marker
        particles (the scalar field IsotropicParticleMesher builds every substep):
        field (3-D float32, shape (D, H, W)) += the splat of every particle.  The
        positions never leave the device."""
        if field.dtype != np.float32 or not field.flags.c_contiguous or field.ndim != 3:
            raise GFSError(_lib.GFS_ERR_INVALID, "add_marker_particle_points",
                           "field must be a contiguous 3-D float32 array")
        D, H, W = field.shape
        off = _arr(offset, np.float32)
        _lib.lib().gfs_sim_add_marker_particle_points(self._h, float(radius), _p(off), float(dx), W, H, D, _p(field),
                                                      int(threshold is not None), float(threshold or 0.0))

    def get_saved_velocity_field(self) -> MACVelocityField:
        """The last step's saved field (after _advectVelocityField, extrapolated),
        which the PIC/FLIP update reads as the old velocities."""
        f = MACVelocityField(self.isize, self.jsize, self.ksize, self.dx)
        _lib.lib().gfs_sim_get_saved_velocity_field(self._h, _p(f.u), _p(f.v), _p(f.w))
        return f

    def step_stages(self, dt, last_stage) -> dict:
        """The substep of update(dt) up to the end of stage `last_stage` of
        FluidSimulation::_stepFluid (STAGE_UPDATE_FLUID_CELLS, STAGE_BODY_FORCES,
        STAGE_PRESSURE, STAGE_APPLY_PRESSURE, STAGE_EXTRAPOLATE or STAGE_ALL).
        Before STAGE_ALL the particles are not advanced and the frame counter
        does not move."""
        st = StepStats()
        _lib.lib().gfs_sim_step_stages(self._h, float(dt), int(last_stage), ctypes.byref(st))
        self.last_stats = st.as_dict()
        return self.last_stats

    # -- fluid sources (fluidsimulation.cpp:767-810; pyfluid/fluidsimulation.py:626-648) --
    def _push_sources(self):
        srcs = getattr(self, "_sources", [])
        arr = (_lib.FluidSourceC * max(len(srcs), 1))()
        for q, s in enumerate(srcs):
            arr[q] = s._c()
        _lib.lib().gfs_sim_set_fluid_sources(self._h, arr, len(srcs))

    def add_spherical_fluid_source(self, source):
        if not isinstance(source, SphericalFluidSource):
            raise TypeError("source must be a SphericalFluidSource")
        self._sources = getattr(self, "_sources", []) + [source]
        self._push_sources()

    def add_cuboid_fluid_source(self, source):
        if not isinstance(source, CuboidFluidSource):
            raise TypeError("source must be a CuboidFluidSource")
        self._sources = getattr(self, "_sources", []) + [source]
        self._push_sources()

    def remove_fluid_source(self, source):
        self._sources = [s for s in getattr(self, "_sources", []) if s is not source]
        self._push_sources()

    def remove_fluid_sources(self):
        self._sources = []
        self._push_sources()

    def set_marker_particle_jitter(self, factor, seed=0):
        """Jitter of source-added particles: 0.25 * factor * dx per component."""
        _lib.lib().gfs_sim_set_marker_particle_jitter(self._h, float(factor), int(seed))

    def update_fluid_sources(self):
        """Apply the queued fluid cells and the fluid sources once (re-reading
        the sources' parameters); returns (added, removed).  update() applies
        them at every step."""
        self._push_sources()
        a, r = ctypes.c_int64(), ctypes.c_int64()
        _lib.lib().gfs_sim_update_fluid_sources(self._h, ctypes.byref(a), ctypes.byref(r))
        return a.value, r.value

    # -- fluid-cell queues (fluidsimulation.cpp:887-940; pyfluid/fluidsimulation.py:673-700) --
    @staticmethod
    def _cells(cell_list):
        """cell_list: objects with .i/.j/.k (pyfluid's GridIndex) or (i, j, k) rows."""
        if len(cell_list) and hasattr(cell_list[0], "i"):
            cell_list = [(c.i, c.j, c.k) for c in cell_list]
        return np.ascontiguousarray(np.asarray(cell_list, np.int32).reshape(-1, 3))

    def add_fluid_cells(self, cell_list, vx=0.0, vy=0.0, vz=0.0):
        """Queue cells to become fluid at the next update, 8 particles each with
        velocity (vx, vy, vz); only cells that are air now are queued."""
        c = self._cells(cell_list)
        v = (ctypes.c_float * 3)(vx, vy, vz)
        _lib.lib().gfs_sim_add_fluid_cells(self._h, _p(c), len(c), v)

    def remove_fluid_cells(self, cell_list):
        """Queue cells whose marker particles the next update removes."""
        c = self._cells(cell_list)
        _lib.lib().gfs_sim_remove_fluid_cells(self._h, _p(c), len(c))

    # -- savestates (FluidSimulationSaveState file format) --
    def save_state(self, filename, current_frame=None):
        """FluidSimulation.save_state (pyfluid/fluidsimulation.py:109-113): the
        marker particles and solid cells in the reference's savestate format."""
        frame = self.current_frame if current_frame is None else int(current_frame)
        _lib.lib().gfs_sim_save_state(self._h, os.fsencode(filename), frame)

    def load_state(self, filename) -> int:
        """Replace the material grid and particles by a savestate's (grid must
        match); returns and adopts the file's current frame."""
        frame = ctypes.c_int(0)
        _lib.lib().gfs_sim_load_state(self._h, os.fsencode(filename), ctypes.byref(frame))
        self.current_frame = frame.value
        return frame.value

    @classmethod
    def from_save_state(cls, savestate, max_particles=None, ctx: Context | None = None):
        """FluidSimulation.from_save_state (pyfluid/fluidsimulation.py:67-75): a
        simulation with the savestate's grid, solid cells, particles and frame.
        `savestate` is a FluidSimulationSaveState or a file name."""
        st = savestate if isinstance(savestate, FluidSimulationSaveState) else FluidSimulationSaveState()
        if st is not savestate:
            st.load_state(savestate)
        i, j, k = st.get_grid_dimensions()
        cap = max(int(max_particles or 0), st.get_num_marker_particles(), 1)
        sim = cls(i, j, k, st.get_cell_size(), cap, ctx=ctx)
        sim.load_state(st.filename)
        return sim

    # -- autosave (fluidsimulation.cpp:566-582, 3412-3415; pyfluid/fluidsimulation.py:496-509) --
    @property
    def enable_autosave(self) -> bool:
        """When set, update() first writes the state to
        `config.get_savestates_directory()/autosave.state`, as the reference's
        update does at the start of every frame.  Off by default: the reference
        enables it by default, but at 40M particles every save writes 1.1 GB."""
        return self._autosave

    @enable_autosave.setter
    def enable_autosave(self, value):
        self._autosave = bool(value)

    def autosave_path(self) -> str:
        return os.path.join(config.get_savestates_directory(), "autosave.state")

    # -- stepping --
    def update(self, dt) -> dict:
        """One substep of length dt (FluidSimulation::update, fluidsimulation.cpp:3417-3455)."""
        if dt < 0.0:
            raise GFSError(_lib.GFS_ERR_INVALID, "update", f"delta time must be >= 0 (got {dt})")
        if self._autosave:                 # _autosave, before the frame's substeps (:3433-3435)
            os.makedirs(config.get_savestates_directory(), exist_ok=True)
            self.save_state(self.autosave_path())
        if getattr(self, "_sources", None):
            self._push_sources()          # sources are mutable objects, as in pyfluid
        st = StepStats()
        _lib.lib().gfs_sim_step(self._h, float(dt), ctypes.byref(st))
        self.last_stats = st.as_dict()
        self.current_frame += 1
        return self.last_stats

    def pressure_check(self, dt, rel_tol=1e-12) -> dict:
        """Error of the last step's pressure against an FP64 solve of the same system
        to rel_tol: {"fp64_residual": max|b - A p|, "rel_error": max|p - p_ref| / max|p_ref|}."""
        r, e, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _lib.lib().gfs_sim_pressure_check(self._h, float(dt), float(rel_tol), ctypes.byref(r), ctypes.byref(e),
                                          ctypes.byref(it))
        return {"fp64_residual": r.value, "rel_error": e.value, "ref_iterations": it.value}

    def update_host(self, dt, positions, velocities, ids):
        """The same substep on host-resident particle arrays (copied in and out):
        arrays are updated in place; returns (count, stats)."""
        n = ctypes.c_int64(len(positions))
        st = StepStats()
        _lib.lib().gfs_sim_step_host(self._h, float(dt), _p(positions), _p(velocities), _p(ids), ctypes.byref(n),
                                     ctypes.byref(st))
        self.last_stats = st.as_dict()
        return n.value, self.last_stats

    def close(self):
        for d in list(getattr(self, "_dependents", ())):
            d.close()
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().gfs_sim_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FluidSimulationSaveState:
    """The header of a savestate file, as pyfluid's FluidSimulationSaveState
    (pyfluid/fluidsimulationsavestate.py:18-207) reports it after load_state."""

    def __init__(self):
        self.filename = None
        self._h = None

    def load_state(self, filename) -> bool:
        i, j, k, fr, br = (ctypes.c_int() for _ in range(5))
        dx = ctypes.c_double()
        nm, nd, ns = (ctypes.c_int64() for _ in range(3))
        _lib.lib().gfs_savestate_read_header(os.fsencode(filename), ctypes.byref(i), ctypes.byref(j), ctypes.byref(k),
                                             ctypes.byref(dx), ctypes.byref(fr), ctypes.byref(nm), ctypes.byref(nd),
                                             ctypes.byref(ns), ctypes.byref(br))
        self.filename = filename
        self._h = dict(dims=(i.value, j.value, k.value), dx=dx.value, frame=fr.value, marker=nm.value,
                       diffuse=nd.value, solid=ns.value, brick=bool(br.value))
        return True

    def close_state(self):
        self.filename = None
        self._h = None

    def is_load_state_initialized(self) -> bool:
        return self._h is not None

    def _hdr(self):
        if self._h is None:
            raise GFSError(_lib.GFS_ERR_STATE, "FluidSimulationSaveState", "no state is loaded")
        return self._h

    def get_grid_dimensions(self):
        return self._hdr()["dims"]

    def get_cell_size(self):
        return self._hdr()["dx"]

    def get_current_frame(self):
        return self._hdr()["frame"]

    def get_num_marker_particles(self):
        return self._hdr()["marker"]

    def get_num_diffuse_particles(self):
        return self._hdr()["diffuse"]

    def get_num_solid_cells(self):
        return self._hdr()["solid"]

    def is_fluid_brick_grid_enabled(self):
        return self._hdr()["brick"]


class FluidSource:
    """FluidSource (fluidsource.h; pyfluid/fluidsource.py:10-123): position,
    velocity, inflow/outflow and active state of a source."""

    def __init__(self, position=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0)):
        self.position = tuple(float(x) for x in position)
        self.velocity = tuple(float(x) for x in velocity)
        self.is_inflow = True
        self.is_active = True

    @property
    def is_outflow(self):
        return not self.is_inflow

    @is_outflow.setter
    def is_outflow(self, value):
        self.is_inflow = not bool(value)

    def _c(self):
        c = _lib.FluidSourceC()
        c.outflow = 0 if self.is_inflow else 1
        c.active = 1 if self.is_active else 0
        c.position = (ctypes.c_float * 3)(*self.position)
        c.velocity = (ctypes.c_float * 3)(*self.velocity)
        return c


class SphericalFluidSource(FluidSource):
    """SphericalFluidSource(position, radius) (sphericalfluidsource.cpp:25-29)."""

    def __init__(self, position=(0.0, 0.0, 0.0), radius=0.0, velocity=(0.0, 0.0, 0.0)):
        super().__init__(position, velocity)
        self.radius = float(radius)

    def _c(self):
        c = super()._c()
        c.shape = 0
        c.radius = self.radius
        return c


class CuboidFluidSource(FluidSource):
    """CuboidFluidSource(position, width, height, depth) (cuboidfluidsource.cpp:25-41):
    the box [position, position + (width, height, depth))."""

    def __init__(self, position=(0.0, 0.0, 0.0), width=0.0, height=0.0, depth=0.0, velocity=(0.0, 0.0, 0.0)):
        super().__init__(position, velocity)
        self.width, self.height, self.depth = float(width), float(height), float(depth)

    def _c(self):
        c = super()._c()
        c.shape = 1
        c.size = (ctypes.c_double * 3)(self.width, self.height, self.depth)
        return c
