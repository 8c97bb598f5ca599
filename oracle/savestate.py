"""NumPy restatement of GridFluidSim3D's FluidSimulationSaveState file format
(test infrastructure only: the checker for gfs_sim_save_state /
gfs_sim_load_state; the product path never imports it).

Layout, native (little-endian) byte order, no padding between fields:

    int32 isize, jsize, ksize; float64 dx; int32 current frame;     (fluidsimulationsavestate.cpp:47-55)
    int32 marker count n; int32 diffuse count m; int32 solid count s; (:58-67)
    bool brick grid flag (1 byte)                                     (:70-71)
    float32[n][3] marker positions; float32[n][3] marker velocities   (:74-77, _writeBinaryVector3f :623-626)
    float32[m][3] diffuse positions; float32[m][3] diffuse velocities;
    float32[m] diffuse lifetimes; char[m] diffuse types               (:80-89)
    int32[s][3] solid cell indices, i fastest                         (:92, :543-573, :638-642)
    brick grid data when the flag is set                              (:94-96)

The reader mirrors FluidSimulationSaveState::loadState's offsets (:101-150).
"""
from __future__ import annotations

import numpy as np

HEADER = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("dx", "<f8"), ("frame", "<i4"),
                   ("n_marker", "<i4"), ("n_diffuse", "<i4"), ("n_solid", "<i4"), ("brick", "u1")])
assert HEADER.itemsize == 37

SOLID = 2


def solid_cells(material: np.ndarray) -> np.ndarray:
    """Solid cells of a (k, j, i)-shaped material array as [i, j, k] rows, i fastest
    (FluidSimulationSaveState::_writeBinarySolidCellIndices, :543-573)."""
    k, j, i = np.nonzero(material == SOLID)          # C order: k slowest, i fastest
    return np.stack([i, j, k], axis=1).astype("<i4")


def write_state(path, dims, dx, frame, positions, velocities, material, diffuse=None) -> None:
    """FluidSimulationSaveState::saveState (:31-99).  dims = (isize, jsize, ksize);
    material is indexed [k, j, i]; diffuse = (positions, velocities, lifetimes, types)."""
    pos = np.ascontiguousarray(positions, dtype="<f4").reshape(-1, 3)
    vel = np.ascontiguousarray(velocities, dtype="<f4").reshape(-1, 3)
    assert pos.shape == vel.shape
    if diffuse is None:
        dpos = dvel = np.zeros((0, 3), "<f4")
        life = np.zeros(0, "<f4")
        types = np.zeros(0, "i1")
    else:
        dpos, dvel, life, types = (np.ascontiguousarray(a) for a in diffuse)
    solid = solid_cells(material)
    h = np.zeros((), HEADER)
    h["i"], h["j"], h["k"] = dims
    h["dx"] = dx
    h["frame"] = frame
    h["n_marker"] = len(pos)
    h["n_diffuse"] = len(dpos)
    h["n_solid"] = len(solid)
    h["brick"] = 0
    with open(path, "wb") as f:
        f.write(h.tobytes())
        for a in (pos, vel, dpos.astype("<f4"), dvel.astype("<f4"), life.astype("<f4"), types.astype("i1"), solid):
            f.write(a.tobytes())


def read_state(path) -> dict:
    """The header and arrays at the offsets FluidSimulationSaveState::loadState
    computes (:101-150)."""
    raw = np.fromfile(path, dtype=np.uint8)
    h = np.frombuffer(raw[:HEADER.itemsize].tobytes(), HEADER)[0]
    n, m, s = int(h["n_marker"]), int(h["n_diffuse"]), int(h["n_solid"])
    off = HEADER.itemsize

    def take(count, dtype, shape):
        nonlocal off
        nbytes = count * np.dtype(dtype).itemsize
        a = np.frombuffer(raw[off:off + nbytes].tobytes(), dtype).reshape(shape)
        off += nbytes
        return a

    out = {"dims": (int(h["i"]), int(h["j"]), int(h["k"])), "dx": float(h["dx"]), "frame": int(h["frame"]),
           "brick": bool(h["brick"])}
    out["positions"] = take(3 * n, "<f4", (n, 3))
    out["velocities"] = take(3 * n, "<f4", (n, 3))
    out["diffuse_positions"] = take(3 * m, "<f4", (m, 3))
    out["diffuse_velocities"] = take(3 * m, "<f4", (m, 3))
    out["diffuse_lifetimes"] = take(m, "<f4", (m,))
    out["diffuse_types"] = take(m, "i1", (m,))
    out["solid_cells"] = take(3 * s, "<i4", (s, 3))
    out["trailing_bytes"] = len(raw) - off
    return out


def material_from_solid(dims, solid: np.ndarray) -> np.ndarray:
    """All-air material grid [k, j, i] with the listed solid cells
    (FluidSimulation::_initializeSolidCellsFromSaveState, fluidsimulation.cpp:1613-1636)."""
    ni, nj, nk = dims
    mat = np.zeros((nk, nj, ni), np.uint8)
    if len(solid):
        mat[solid[:, 2], solid[:, 1], solid[:, 0]] = SOLID
    return mat
