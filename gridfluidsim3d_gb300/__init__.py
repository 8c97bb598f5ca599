"""gridfluidsim3d_gb300 -- GB300-native (sm_103a) per-substep FLIP core of
GridFluidSim3D: P2G velocity splat, MICCG(0) pressure projection, PIC/FLIP G2P
with RK4 advection, behind the reference's interfaces.

The compute path is libgfs.so (CUDA kernels + C ABI, include/gfs.h).  This
package is its host-side mirror; importing it needs no GPU, calling into it
does, and there is no CPU fallback.
"""
from ._lib import GFSError, PRECISION_MIXED, PRECISION_PLAIN  # noqa: F401
from ._lib import (SWEEP_AUTO, SWEEP_BLOCK, SWEEP_CLUSTER_2X2, SWEEP_CLUSTER_4X2, SWEEP_WARP,  # noqa: F401
                   STAGE_ALL, STAGE_APPLY_PRESSURE, STAGE_BODY_FORCES, STAGE_EXTRAPOLATE, STAGE_PRESSURE,
                   STAGE_UPDATE_FLUID_CELLS)
from . import config  # noqa: F401
from .core import (AIR, FLUID, SOLID, CLScalarField, Context, CuboidFluidSource, FluidSimulation,  # noqa: F401
                   GridIndex,
                   FluidSimulationSaveState, FluidSource, MACVelocityField, SphericalFluidSource, ParticleAdvector, PressureSolver,
                   PressureSolverParameters, face_shape)

__all__ = ["GFSError", "PRECISION_PLAIN", "PRECISION_MIXED", "AIR", "FLUID", "SOLID", "Context",
           "CLScalarField", "ParticleAdvector", "PressureSolver", "PressureSolverParameters",
           "MACVelocityField", "FluidSimulation", "FluidSimulationSaveState", "FluidSource", "SphericalFluidSource", "CuboidFluidSource",
           "GridIndex", "face_shape", "config"]
