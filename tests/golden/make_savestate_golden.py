"""Write the savestate fixtures of tests/golden/ with the reference's own code.

1. `savestate_in.state`: a seeded small state, 12 x 10 x 9 cells, dx 0.25 (solid
   border, a few interior solid cells, 300 marker particles, frame 7), written by
   the oracle's restatement of the format (oracle/savestate.py).
2. `savestate_ref.state`: what the reference makes of it.  The reference's
   simulator library is built with the drop-in classes (its asserts compiled out
   by its own NFLUIDSIMDEBUG switch, so no GPU is needed), and a probe program
   loads the file with FluidSimulationSaveState::loadState, constructs
   FluidSimulation(FluidSimulationSaveState&) from it and writes it back with
   FluidSimulation::saveState -- all reference code.

Needs the reference's source tree and g++; the fixtures are committed.

    python tests/golden/make_savestate_golden.py
"""
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
DIMS = (12, 10, 9)
DX = 0.25
FRAME = 7

PROBE = r'''
#include <cstdio>
#include "fluidsimulation.h"
#include "fluidsimulationsavestate.h"

int main(int argc, char **argv) {
    FluidSimulationSaveState state;
    if (!state.loadState(argv[1])) return 2;
    FluidSimulation sim(state);
    state.closeState();
    sim.saveState(argv[2]);
    std::printf("%d %d\n", sim.getNumMarkerParticles(), sim.getCurrentFrame());
    return 0;
}
'''


def scene(seed=91):
    rng = np.random.default_rng(seed)
    ni, nj, nk = DIMS
    mat = np.zeros((nk, nj, ni), np.uint8)
    mat[0, :, :] = mat[-1, :, :] = mat[:, 0, :] = mat[:, -1, :] = mat[:, :, 0] = mat[:, :, -1] = S.SOLID
    for (i, j, k) in [(4, 3, 2), (5, 3, 2), (7, 6, 5), (3, 7, 6)]:
        mat[k, j, i] = S.SOLID
    free = np.argwhere(mat == 0)                     # rows (k, j, i)
    cells = free[rng.integers(0, len(free), 300)]
    jitter = rng.random((300, 3))
    pos = ((cells[:, ::-1] + jitter) * DX).astype(np.float32)
    vel = rng.normal(0.0, 0.5, (300, 3)).astype(np.float32)
    return mat, pos, vel


def main():
    if SRC is None:
        sys.exit("the reference's src/ directory is unknown: set GFS_REFERENCE_SRC")
    from gridfluidsim3d_gb300 import build
    from gridfluidsim3d_gb300.dropin import build_reference_tree
    mat, pos, vel = scene()
    fin = os.path.join(HERE, "savestate_in.state")
    fref = os.path.join(HERE, "savestate_ref.state")
    S.write_state(fin, DIMS, DX, FRAME, pos, vel, mat)
    build.build()
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "tree")
        build_reference_tree(SRC, out, opt="-O0")
        probe = os.path.join(tmp, "probe.cpp")
        with open(probe, "w") as f:
            f.write(PROBE)
        exe = os.path.join(tmp, "probe")
        lib_dir = os.path.dirname(build.LIB)
        subprocess.run(["g++", "-std=c++11", "-O0", "-w", "-DNFLUIDSIMDEBUG", "-include", "limits", "-I" + out,
                        "-I" + os.path.join(ROOT, "include"), probe, "-o", exe, "-L" + out, "-lfluidsim_gfs",
                        "-Wl,-rpath," + out, "-L" + lib_dir, "-lgfs", "-Wl,-rpath," + lib_dir], check=True)
        r = subprocess.run([exe, fin, fref], capture_output=True, text=True, timeout=300, cwd=tmp)
        if r.returncode != 0:
            raise RuntimeError(f"probe failed ({r.returncode}): {r.stderr[-2000:]}")
        print("reference re-save:", r.stdout.strip())
    same = open(fin, "rb").read() == open(fref, "rb").read()
    print("byte-identical:", same)


if __name__ == "__main__":
    main()
