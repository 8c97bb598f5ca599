import argparse

from . import build_reference_tree

ap = argparse.ArgumentParser(description="Build GridFluidSim3D with the libgfs drop-in classes")
ap.add_argument("--src", required=True, help="the reference's src/ directory")
ap.add_argument("--out", required=True, help="build directory (symlink tree + objects)")
ap.add_argument("--main", action="store_true", help="also build the reference's example program")
a = ap.parse_args()
print(build_reference_tree(a.src, a.out, main=a.main))
