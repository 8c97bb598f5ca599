"""NumPy restatement of FluidSimulation::_updateFluidSources
(fluidsimulation.cpp:1717-1879) and of the fluid-cell queues
(addFluidCells / removeFluidCells, :887-940, 1881-1930) for small grids (test infrastructure only: the
checker for gfs_sim_update_fluid_sources and the source stage of gfs_sim_step;
the product path never imports it).

The reference draws the jitter of new particles from rand(); like the CUDA path
this restatement uses the counter-based hash jitter(seed, particle id, axis),
and with a jitter factor of 0 both reproduce the reference's positions exactly
(pinned by tests/golden/fluidsource_ref.state, written by the reference).

Float / double steps follow the reference's types: vmath::vec3 is float32,
radii, extents and dx are float64 (grid3d.h, aabb.cpp, sphericalfluidsource.cpp).
"""
from __future__ import annotations

import math

import numpy as np

AIR, FLUID, SOLID = 0, 1, 2
f32 = np.float32

M64 = (1 << 64) - 1


def jitter_component(seed: int, pid: int, axis: int, j: float) -> np.float32:
    """splitmix64 of the counter (seed, id, axis) -> uniform in [-j, j], as float32."""
    z = (seed + 0x9E3779B97F4A7C15 * (pid * 3 + axis + 1)) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    z ^= z >> 31
    u = (z >> 11) * (1.0 / 9007199254740992.0)
    return f32(-j + 2.0 * j * u)


def pos_to_index(p, dx):                     # Grid3d::positionToGridIndex (grid3d.h:58-63)
    inv = 1.0 / dx
    return tuple(int(math.floor(float(c) * inv)) for c in p)


def index_to_pos(i, dx):                     # GridIndexToPosition: (float)i*dx -> float
    return f32(float(f32(i)) * dx)


def cell_center(i, dx):                      # GridIndexToCellCenter (grid3d.h:103-106)
    return f32(float(f32(i)) * dx + 0.5 * dx)


def bounds_sphere(p, r, dx, dims):           # getGridIndexBounds(vec3 p, double r, ...) (:350-371)
    c = pos_to_index(p, dx)
    t = [f32(p[a] - index_to_pos(c[a], dx)) for a in range(3)]
    inv = 1.0 / dx
    lo = [max(c[a] - int(max(0.0, math.ceil((r - float(t[a])) * inv))), 0) for a in range(3)]
    hi = [min(c[a] + int(max(0.0, math.ceil((r - dx + float(t[a])) * inv))), dims[a] - 1) for a in range(3)]
    return lo, hi


def bounds_box(bp, bw, dx, dims):            # getGridIndexBounds(AABB, ...)
    q = [f32(bp[a] + f32(bw[a])) for a in range(3)]
    g1 = pos_to_index(bp, dx)
    g2 = pos_to_index(q, dx)
    return [max(g1[a], 0) for a in range(3)], [min(g2[a], dims[a] - 1) for a in range(3)]


def fit_box(bp, bw, dx, dims):               # fitAABBtoGrid + AABB(vec3, vec3) (aabb.cpp:33-45)
    pmin = [f32(x) for x in bp]
    pmax = [f32(bp[a] + f32(bw[a])) for a in range(3)]
    gmin, gmax = pos_to_index(pmin, dx), pos_to_index(pmax, dx)
    inr = lambda g: all(0 <= g[a] < dims[a] for a in range(3))
    if not inr(gmin):
        pmin = [f32(0.0)] * 3
    if not inr(gmax):
        pmax = [f32(f32(index_to_pos(gmax[a], dx) + f32(dx)) - f32(10e-9)) for a in range(3)]
    mn = [min(float(pmin[a]), float(pmax[a])) for a in range(3)]
    mx = [max(float(pmin[a]), float(pmax[a])) for a in range(3)]
    return [f32(x) for x in mn], [mx[a] - mn[a] for a in range(3)]


def overlapping(src, dx, dims):
    """Overlapping cells, k, j, i loops (i fastest) (Spherical/CuboidFluidSource::_getOverlappingCells)."""
    if src["shape"] == "sphere":
        r = max(float(src["radius"]), 0.0)
        c = [f32(x) for x in src["position"]]
        lo, hi = bounds_sphere(c, r, dx, dims)
        out = []
        for k in range(lo[2], hi[2] + 1):
            for j in range(lo[1], hi[1] + 1):
                for i in range(lo[0], hi[0] + 1):
                    v = [f32(cell_center(g, dx) - c[a]) for a, g in enumerate((i, j, k))]
                    d2 = f32(f32(f32(v[0] * v[0]) + f32(v[1] * v[1])) + f32(v[2] * v[2]))
                    if float(d2) < r * r:
                        out.append((i, j, k))
        return out
    lo, hi = bounds_box([f32(x) for x in src["position"]], src["size"], dx, dims)
    return [(i, j, k) for k in range(lo[2], hi[2] + 1) for j in range(lo[1], hi[1] + 1)
            for i in range(lo[0], hi[0] + 1)]


def aabb(src):
    if src["shape"] == "sphere":              # SphericalFluidSource::getAABB (:48-52)
        r = max(float(src["radius"]), 0.0)
        return [f32(f32(x) - f32(r)) for x in src["position"]], [2.0 * r] * 3
    return [f32(x) for x in src["position"]], [float(x) for x in src["size"]]


ORDER8 = [(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)]


def cell_particles(g, dx, nid, seed, jit):
    """_addMarkerParticlesToCell (fluidsimulation.cpp:1223-1246): 8 positions at
    the 2x2x2 sub-cell centres (double offsets from the float centre, stored as
    float) plus jitter, for ids nid .. nid + 7."""
    q = 0.25 * dx
    cc = [cell_center(x, dx) for x in g]
    out = []
    for n, sgn in enumerate(ORDER8):
        out.append(tuple(f32(f32(float(cc[a]) + sgn[a] * q) + jitter_component(seed, nid + n, a, jit))
                         for a in range(3)))
    return out


def add_fluid_cells_filter(dims, mat, cells):
    """FluidSimulation::addFluidCells (fluidsimulation.cpp:887-909): an index out
    of range raises (nothing is queued); the cells that are air now are kept."""
    for g in cells:
        if not all(0 <= g[a] < dims[a] for a in range(3)):
            raise IndexError(f"fluid cell index out of range: {tuple(g)}")
    return [tuple(int(x) for x in g) for g in cells if mat[g[2], g[1], g[0]] == AIR]


def update_fluid_cell_queues(dims, dx, mat, pos, vel, ids, added, removed, jitter_factor=0.1, seed=0,
                             next_id=None):
    """_updateAddedFluidCellQueue then _updateRemovedFluidCellQueue
    (fluidsimulation.cpp:1881-1930) on (mat [k, j, i], pos, vel, ids).
    added: [(cells, velocity)] groups as queued (already filtered by
    add_fluid_cells_filter); removed: cells.  Returns (mat, pos, vel, ids, next_id)."""
    mat = mat.copy()
    P = [tuple(p) for p in np.asarray(pos, np.float32)]
    V = [tuple(v) for v in np.asarray(vel, np.float32)]
    I = [int(i) for i in ids]
    nid = (max(I) + 1 if I else 0) if next_id is None else int(next_id)
    jit = 0.25 * jitter_factor * dx
    for cells, velo in added:
        velo = tuple(f32(x) for x in velo)
        for g in cells:                          # _addNewFluidCells (:1749-1759)
            if mat[g[2], g[1], g[0]] != AIR:
                continue
            P.extend(cell_particles(g, dx, nid, seed, jit))
            V.extend([velo] * 8)
            I.extend(range(nid, nid + 8))
            nid += 8
            mat[g[2], g[1], g[0]] = FLUID
    rm = {tuple(int(x) for x in g) for g in removed}
    keep = np.array([pos_to_index(p, dx) not in rm for p in P], bool) if P else np.zeros(0, bool)
    pos = np.array(P, np.float32).reshape(-1, 3)[keep]
    vel = np.array(V, np.float32).reshape(-1, 3)[keep]
    ids = np.array(I, np.uint32)[keep]
    return mat, pos, vel, ids, nid


def update_fluid_sources(dims, dx, mat, pos, vel, ids, sources, jitter_factor=0.1, seed=0, next_id=None):
    """_updateFluidSources on (mat [k, j, i], pos, vel, ids); returns the new
    (mat, pos, vel, ids): particles appended in the reference's creation order
    with ids from next_id (default max id + 1), outflow cells' particles removed."""
    mat = mat.copy()
    P = [tuple(p) for p in np.asarray(pos, np.float32)]
    V = [tuple(v) for v in np.asarray(vel, np.float32)]
    I = [int(i) for i in ids]
    nid = (max(I) + 1 if I else 0) if next_id is None else int(next_id)
    jit = 0.25 * jitter_factor * dx
    for src in sources:
        if not src.get("active", True) or src.get("outflow", False):
            continue
        velo = tuple(f32(x) for x in src["velocity"])
        cells = overlapping(src, dx, dims)
        # 1. air cells get 8 particles (_addNewFluidCells, _addMarkerParticlesToCell)
        kind = {}
        for g in cells:
            m = mat[g[2], g[1], g[0]]
            kind[g] = 1 if m == AIR else (2 if m == FLUID else 0)
        for g in cells:
            if kind[g] != 1:
                continue
            mat[g[2], g[1], g[0]] = FLUID
            P.extend(cell_particles(g, dx, nid, seed, jit))
            V.extend([velo] * 8)
            I.extend(range(nid, nid + 8))
            nid += 8
        # 2. empty sub-cells of fluid-or-air overlapping cells (_getNewFluidParticles)
        bp, bw = aabb(src)
        fp, fw = fit_box(bp, bw, dx, dims)
        f1, f2 = bounds_box(fp, fw, dx, dims)
        nf = [max(f2[a] - f1[a] + 1, 0) for a in range(3)]
        sub = np.zeros((2 * nf[2], 2 * nf[1], 2 * nf[0]), bool)
        for g in cells:
            if kind[g] == 0:
                continue
            l = [g[a] - f1[a] for a in range(3)]
            if all(0 <= l[a] < nf[a] for a in range(3)):
                sub[2 * l[2]:2 * l[2] + 2, 2 * l[1]:2 * l[1] + 2, 2 * l[0]:2 * l[0] + 2] = True
        off = [index_to_pos(f1[a], dx) for a in range(3)]
        for p in P:
            if all(float(p[a]) >= float(fp[a]) and float(p[a]) < float(fp[a]) + fw[a] for a in range(3)):
                s = pos_to_index([f32(p[a] - off[a]) for a in range(3)], 0.5 * dx)
                if all(0 <= s[a] < 2 * nf[a] for a in range(3)):
                    sub[s[2], s[1], s[0]] = False
        for k, j, i in zip(*np.nonzero(sub)):      # C order: i fastest
            p = [f32(f32(cell_center(int(x), 0.5 * dx) + off[a]) + jitter_component(seed, nid, a, jit))
                 for a, x in enumerate((i, j, k))]
            P.append(tuple(p))
            V.append(velo)
            I.append(nid)
            nid += 1
            g = pos_to_index(p, dx)
            if all(0 <= g[a] < dims[a] for a in range(3)):
                mat[g[2], g[1], g[0]] = FLUID
    # outflow: particles in the overlapping fluid cells are removed
    remove = np.zeros_like(mat, bool)
    for src in sources:
        if not src.get("active", True) or not src.get("outflow", False):
            continue
        for g in overlapping(src, dx, dims):
            if mat[g[2], g[1], g[0]] == FLUID:
                remove[g[2], g[1], g[0]] = True
    keep = []
    for n, p in enumerate(P):
        g = pos_to_index(p, dx)
        inside = all(0 <= g[a] < dims[a] for a in range(3))
        keep.append(not (inside and remove[g[2], g[1], g[0]]))
    keep = np.array(keep, bool) if keep else np.zeros(0, bool)
    pos = np.array(P, np.float32).reshape(-1, 3)[keep]
    vel = np.array(V, np.float32).reshape(-1, 3)[keep]
    ids = np.array(I, np.uint32)[keep]
    return mat, pos, vel, ids, nid
