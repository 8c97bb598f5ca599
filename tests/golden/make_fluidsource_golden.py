"""Write the fluid-source fixtures of tests/golden/ with the reference's own code.

1. `fluidsource_in.state`: a seeded 16 x 14 x 12 state, dx 0.25 (solid border, a
   pool of fluid in the bottom four cell layers, 8 particles per pool cell),
   written with the oracle's savestate writer.
2. `fluidsource_sources.json`: the sources -- an inflow sphere across the pool's
   surface, an inflow cuboid in the air, an inflow sphere against the solid
   wall, an outflow sphere inside the pool and an inactive inflow sphere.
3. `fluidsource_ref.state`: the reference's result.  Its simulator library is
   built with the drop-in classes (asserts compiled out by NFLUIDSIMDEBUG, no GPU
   needed); a probe loads the input with FluidSimulation(FluidSimulationSaveState&),
   registers the sources with addSphericalFluidSource / addCuboidFluidSource,
   sets the marker-particle jitter factor to 0 (rand() jitter is not
   reproducible; with 0 the new positions are deterministic), runs the
   reference's _updateFluidSources and saves the state with
   FluidSimulation::saveState.  The probe reaches the two private members by
   defining private/protected as public in its own translation unit, after the
   standard headers; the library is compiled unchanged.

4. `fluidcells_ref.state` and `fluidcells_queues.json`: the same input with
   the same sources, plus two addFluidCells groups (one with a velocity, one
   through the overload without; duplicates, fluid and solid cells among them)
   and one removeFluidCells list (pool cells, a cell inside the inflow sphere,
   an added cell), after the reference's whole _updateFluidCells (solid
   removal, the added queue, the removed queue, the sources, classification),
   jitter factor 0, saved with FluidSimulation::saveState.

5. `fluidsource_edge_ref.state` and `fluidsource_edge_sources.json`: the same input
   with sources across the grid's faces (see EDGE_SOURCES), after the reference's
   _updateFluidSources, jitter factor 0.

Needs the reference's source tree and g++; the fixtures are committed.

    python tests/golden/make_fluidsource_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import reference_src  # noqa: E402
from oracle import savestate as S  # noqa: E402

SRC = reference_src()   # $GFS_REFERENCE_SRC, or the directory the last oracle build recorded
DIMS = (16, 14, 12)
DX = 0.25

SOURCES = [
    {"shape": "sphere", "position": [2.0, 1.2, 1.5], "radius": 0.6, "velocity": [1.0, 0.0, 0.0]},
    {"shape": "cuboid", "position": [2.6, 2.2, 0.8], "size": [0.7, 0.5, 0.9], "velocity": [0.0, -1.0, 0.5]},
    {"shape": "sphere", "position": [0.4, 2.0, 2.0], "radius": 0.5, "velocity": [0.0, 0.0, -0.75]},
    {"shape": "sphere", "position": [3.0, 0.6, 2.2], "radius": 0.45, "velocity": [0.0, 0.0, 0.0], "outflow": True},
    {"shape": "sphere", "position": [1.5, 2.5, 1.5], "radius": 0.5, "velocity": [0.0, 0.0, 0.0], "active": False},
]


# Sources across the grid's faces, for the clamping branches of fitAABBtoGrid and
# getGridIndexBounds (grid3d.h:350-371, 426-439, 485-502): a sphere past the far
# corner, a cuboid starting below zero (fitAABBtoGrid then moves the whole minimum
# corner to the origin), a cuboid past the far faces, spheres of radius 0 and -1,
# and an outflow cuboid over the pool's edge.  Written to fluidsource_edge_*.
EDGE_SOURCES = [
    {"shape": "sphere", "position": [3.9, 3.4, 2.9], "radius": 0.5, "velocity": [0.0, -1.0, 0.0]},
    {"shape": "cuboid", "position": [-0.3, 1.8, -0.2], "size": [0.9, 0.6, 0.8], "velocity": [0.5, 0.0, 0.25]},
    {"shape": "cuboid", "position": [3.2, 2.6, 2.2], "size": [1.5, 1.5, 1.5], "velocity": [-0.5, 0.0, 0.0]},
    {"shape": "sphere", "position": [2.0, 2.0, 1.5], "radius": 0.0, "velocity": [1.0, 1.0, 1.0]},
    {"shape": "sphere", "position": [1.0, 2.5, 1.0], "radius": -1.0, "velocity": [1.0, 1.0, 1.0]},
    {"shape": "cuboid", "position": [0.1, 0.2, 0.1], "size": [1.0, 0.9, 2.9], "velocity": [0.0, 0.0, 0.0],
     "outflow": True},
]

# addFluidCells groups (cells, velocity or None for the overload without one) and
# the removeFluidCells list; (i, j, k) in the 16 x 14 x 12 grid above
ADD_GROUPS = [
    ([[3, 6, 4], [4, 6, 4], [5, 7, 5], [2, 2, 2], [3, 6, 4], [10, 9, 4]], [0.5, -0.25, 0.0]),
    ([[4, 6, 4], [8, 9, 6], [9, 9, 6], [0, 5, 5]], None),
]
REMOVED = [[6, 3, 6], [7, 3, 6], [5, 7, 5], [8, 4, 6], [1, 1, 1]]


def scene(seed=17):
    rng = np.random.default_rng(seed)
    ni, nj, nk = DIMS
    mat = np.zeros((nk, nj, ni), np.uint8)
    mat[0, :, :] = mat[-1, :, :] = mat[:, 0, :] = mat[:, -1, :] = mat[:, :, 0] = mat[:, :, -1] = S.SOLID
    cells = np.argwhere(mat == 0)                      # rows (k, j, i)
    cells = cells[cells[:, 1] <= 4]
    cells = np.repeat(cells, 8, axis=0)
    pos = ((cells[:, ::-1] + rng.random((len(cells), 3))) * DX).astype(np.float32)
    vel = rng.normal(0.0, 0.3, pos.shape).astype(np.float32)
    return mat, pos, vel


def _probe_source(q, s):
    p = "vmath::vec3((float){!r}, (float){!r}, (float){!r})".format(*map(float, s["position"]))
    v = "vmath::vec3((float){!r}, (float){!r}, (float){!r})".format(*map(float, s["velocity"]))
    if s["shape"] == "sphere":
        line = f"    SphericalFluidSource *s{q} = new SphericalFluidSource({p}, {s['radius']!r}, {v});\n"
        add = f"    sim.addSphericalFluidSource(s{q});\n"
    else:
        w, h, d = s["size"]
        line = f"    CuboidFluidSource *s{q} = new CuboidFluidSource({p}, {w!r}, {h!r}, {d!r}, {v});\n"
        add = f"    sim.addCuboidFluidSource(s{q});\n"
    if s.get("outflow"):
        line += f"    s{q}->setAsOutflow();\n"
    if s.get("active") is False:
        line += f"    s{q}->deactivate();\n"
    return line + add


def _probe_cells(name, cells):
    out = f"    std::vector<GridIndex> {name};\n"
    for c in cells:
        out += f"    {name}.push_back(GridIndex({c[0]}, {c[1]}, {c[2]}));\n"
    return out


def _probe_queues():
    body = ""
    for q, (cells, v) in enumerate(ADD_GROUPS):
        body += _probe_cells(f"add{q}", cells)
        if v is None:
            body += f"    sim.addFluidCells(add{q});\n"
        else:
            body += "    sim.addFluidCells(add{}, vmath::vec3((float){!r}, (float){!r}, (float){!r}));\n".format(
                q, *map(float, v))
    body += _probe_cells("rem", REMOVED)
    body += "    sim.removeFluidCells(rem);\n"
    return body


def probe_source(queues=False, sources=SOURCES):
    body = "".join(_probe_source(q, s) for q, s in enumerate(sources))
    if queues:
        body += _probe_queues()
    update = "sim._updateFluidCells();" if queues else "sim._updateFluidSources();"
    return r'''
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <limits>
#include <queue>
#include <sstream>
#include <string>
#include <vector>
#define private public
#define protected public
#include "fluidsimulation.h"
#include "fluidsimulationsavestate.h"
#include "sphericalfluidsource.h"
#include "cuboidfluidsource.h"

int main(int argc, char **argv) {
    FluidSimulationSaveState state;
    if (!state.loadState(argv[1])) return 2;
    FluidSimulation sim(state);
    state.closeState();
    sim._markerParticleJitterFactor = 0.0;
''' + body + r'''
    int before = sim.getNumMarkerParticles();
    ''' + update + r'''
    sim.saveState(argv[2]);
    std::printf("%d %d\n", before, sim.getNumMarkerParticles());
    return 0;
}
'''


def main():
    if SRC is None:
        sys.exit("the reference's src/ directory is unknown: set GFS_REFERENCE_SRC")
    from gridfluidsim3d_gb300 import build
    from gridfluidsim3d_gb300.dropin import build_reference_tree
    mat, pos, vel = scene()
    fin = os.path.join(HERE, "fluidsource_in.state")
    fref = os.path.join(HERE, "fluidsource_ref.state")
    S.write_state(fin, DIMS, DX, 0, pos, vel, mat)
    with open(os.path.join(HERE, "fluidsource_sources.json"), "w") as f:
        json.dump(SOURCES, f, indent=1)
    with open(os.path.join(HERE, "fluidcells_queues.json"), "w") as f:
        json.dump({"added": [{"cells": c, "velocity": v} for c, v in ADD_GROUPS], "removed": REMOVED}, f, indent=1)
    with open(os.path.join(HERE, "fluidsource_edge_sources.json"), "w") as f:
        json.dump(EDGE_SOURCES, f, indent=1)
    build.build()
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "tree")
        build_reference_tree(SRC, out, opt="-O0")
        lib_dir = os.path.dirname(build.LIB)
        runs = ((False, SOURCES, fref), (True, SOURCES, os.path.join(HERE, "fluidcells_ref.state")),
                (False, EDGE_SOURCES, os.path.join(HERE, "fluidsource_edge_ref.state")))
        for queues, sources, dst in runs:
            probe = os.path.join(tmp, "probe.cpp")
            with open(probe, "w") as f:
                f.write(probe_source(queues, sources))
            exe = os.path.join(tmp, "probe")
            subprocess.run(["g++", "-std=c++11", "-O0", "-w", "-DNFLUIDSIMDEBUG", "-include", "limits", "-I" + out,
                            "-I" + os.path.join(ROOT, "include"), probe, "-o", exe, "-L" + out, "-lfluidsim_gfs",
                            "-Wl,-rpath," + out, "-L" + lib_dir, "-lgfs", "-Wl,-rpath," + lib_dir], check=True)
            r = subprocess.run([exe, fin, dst], capture_output=True, text=True, timeout=300, cwd=tmp)
            if r.returncode != 0:
                raise RuntimeError(f"probe failed ({r.returncode}): {r.stderr[-2000:]}")
            print(os.path.basename(dst), "reference particles before / after:", r.stdout.strip())


if __name__ == "__main__":
    main()
