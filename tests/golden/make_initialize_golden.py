"""Write the seeding fixtures of tests/golden/ with the reference's own code.

The reference's FluidSimulation::initialize (fluidsimulation.cpp:48-55,
1383-1434) seeds each scene below; its simulator library is built on the CPU with
oracle/reftree.py (fluidsimulation.cpp compiled unchanged, CPU backends of the
OpenCL classes) and driven by oracle/ref_initialize_probe.cpp with the
marker-particle jitter factor 0 (the reference's jitter is rand()).

* ``initialize_ball`` -- the hello-world ball of the 64^3 ball drop on a 32^3 grid
  of the same 8 m box (dx 0.25): one implicit fluid point of radius 1.6 at
  (4, 4, 4).
* ``initialize_mixed`` -- 24 x 20 x 18 cells, dx 0.1: two implicit points (one
  overlapping a cuboid, one cut by the domain border), a fluid cuboid on the
  floor, and solid cells added inside the fluid and inside the cuboid.

Stored per scene (npz): the grid, the scene's points / cuboids / solid cells, the
material grid the probe was given (air; the solid cells are added by the probe)
and the reference's particle positions in creation order and material grid.

    python tests/golden/make_initialize_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import reference_src, reftree  # noqa: E402

SRC = reference_src()   # $GFS_REFERENCE_SRC, or the directory the last oracle build recorded

SCENES = {
    "initialize_ball": dict(grid=(32, 32, 32, 0.25), points=[(4.0, 4.0, 4.0, 1.6)], cuboids=[], solids=[]),
    "initialize_mixed": dict(grid=(24, 20, 18, 0.1),
                             points=[(0.9, 1.1, 0.8, 0.45), (2.2, 0.6, 1.5, 0.5)],
                             cuboids=[(0.35, 0.1, 0.25, 1.3, 0.42, 1.1)],
                             solids=[(8, 2, 6), (8, 3, 6), (9, 11, 8), (3, 1, 4)]),
}


def main():
    if SRC is None:
        sys.exit("the reference's src/ directory is unknown: set GFS_REFERENCE_SRC")
    with tempfile.TemporaryDirectory() as tmp:
        tree = os.path.join(tmp, "tree")
        reftree.build_cpu_tree(SRC, tree)
        exe = reftree.build_probe(tree, os.path.join(ROOT, "oracle", "ref_initialize_probe.cpp"),
                                  os.path.join(tmp, "probe"))
        for name, sc in SCENES.items():
            ni, nj, nk, dx = sc["grid"]
            txt = os.path.join(tmp, name + ".txt")
            with open(txt, "w") as f:
                f.write(f"grid {ni} {nj} {nk} {dx!r}\n")
                for p in sc["points"]:
                    f.write("point " + " ".join(repr(float(x)) for x in p) + "\n")
                for c in sc["cuboids"]:
                    f.write("cuboid " + " ".join(repr(float(x)) for x in c) + "\n")
                for s in sc["solids"]:
                    f.write("solid " + " ".join(str(int(x)) for x in s) + "\n")
            out = os.path.join(tmp, name)
            os.makedirs(out)
            r = subprocess.run([exe, txt, out], capture_output=True, text=True, timeout=300, cwd=tmp)
            if r.returncode != 0:
                raise RuntimeError(f"probe failed ({r.returncode}): {r.stderr[-2000:]}")
            n = int([l for l in r.stdout.splitlines() if l.startswith("PROBE ")][-1].split()[1])
            pos = np.fromfile(os.path.join(out, "particles.f32"), np.float32).reshape(-1, 3)
            mat = np.fromfile(os.path.join(out, "mat.u8"), np.uint8).reshape(nk, nj, ni)
            assert len(pos) == n
            np.savez_compressed(os.path.join(HERE, name + ".npz"), grid=np.array([ni, nj, nk]), dx=np.float64(dx),
                                points=np.array(sc["points"], np.float64).reshape(-1, 4),
                                cuboids=np.array(sc["cuboids"], np.float64).reshape(-1, 6),
                                solids=np.array(sc["solids"], np.int32).reshape(-1, 3), positions=pos, material=mat)
            print(f"{name}: {n} particles, {int((mat == 1).sum())} fluid cells")


if __name__ == "__main__":
    main()
