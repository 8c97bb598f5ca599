"""The C++ drop-in classes (gridfluidsim3d_gb300/dropin/) against the reference
tree: GridFluidSim3D's simulator library -- fluidsimulation.cpp, the meshers,
diffuse particles and the C bindings, unchanged -- compiles against the drop-in
PressureSolver / ParticleAdvector / CLScalarField headers and links with
libgfs.so with no undefined symbol; a probe program then exercises the classes'
host-side behaviour.  Needs the reference's source tree (skipped elsewhere).
"""
import os
import shutil
import subprocess

import pytest

from oracle import reference_src

SRC = reference_src()   # $GFS_REFERENCE_SRC, or the directory the last oracle build recorded

pytestmark = pytest.mark.skipif(SRC is None or not shutil.which("g++"),
                                reason="reference tree or g++ not present")

PROBE = r'''
#include <cstdio>
#include "clscalarfield.h"
#include "particleadvector.h"
#include "pressuresolver.h"
#include "fluidsimulation.h"

int main() {
    ParticleAdvector advector;
    CLScalarField splatter;
    bool a = advector.initialize();
    bool c = splatter.initialize();
    splatter.setMaxScalarFieldValueThreshold(2.5f);
    VectorXd v(4, -1.5);
    v[2] = 3.0;
    VectorXd w(v);
    PressureSolver solver;
    solver.setPrecision(1);
    // an empty fluid set is solved without touching the device
    GridIndexVector cells(4, 4, 4);
    FluidMaterialGrid mat(4, 4, 4);
    MACVelocityField field(4, 4, 4, 0.25);
    VectorXd p(0);
    PressureSolverParameters prm;
    prm.cellwidth = 0.25; prm.density = 20.0; prm.deltaTime = 1.0 / 30.0;
    prm.fluidCells = &cells; prm.materialGrid = &mat; prm.velocityField = &field; prm.logfile = nullptr;
    solver.solve(prm, p);
    std::printf("init %d %d\n", (int)a, (int)c);
    std::printf("threshold %d %.2f\n", (int)splatter.isMaxScalarFieldValueThresholdSet(),
                splatter.getMaxScalarFieldValueThreshold());
    std::printf("vector %.1f %.2f %d\n", w.absMaxCoeff(), v.dot(w), (int)p.size());
    std::printf("gpu %d %d\n", (int)advector.isUsingGPU(), (int)advector.isUsingCPU());
    return 0;
}
'''


def test_reference_tree_builds_with_dropins(tmp_path):
    from gridfluidsim3d_gb300 import build
    from gridfluidsim3d_gb300.dropin import build_reference_tree
    build.build()
    out = str(tmp_path / "tree")
    built = build_reference_tree(SRC, out, main=True, opt="-O0")
    assert os.path.exists(built["library"]) and os.path.exists(built["program"])
    names = {os.path.basename(o) for o in built["objects"]}
    for unit in ("fluidsimulation.o", "pressuresolver.o", "particleadvector.o", "clscalarfield.o",
                 "isotropicparticlemesher.o", "diffuseparticlesimulation.o", "c_bindings_fluidsimulation_c.o"):
        assert unit in names, unit
    # the replaced files in the tree are this repository's, the rest the reference's
    assert os.path.realpath(os.path.join(out, "pressuresolver.h")).endswith("dropin/pressuresolver.h")
    assert os.path.realpath(os.path.join(out, "fluidsimulation.cpp")) == os.path.join(SRC, "fluidsimulation.cpp")

    probe = tmp_path / "probe.cpp"
    probe.write_text(PROBE)
    exe = str(tmp_path / "probe")
    lib_dir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++11", "-O0", "-w", "-include", "limits", "-I" + out,
                    "-I" + os.path.join(build.ROOT, "include"), str(probe), "-o", exe, "-L" + out,
                    "-lfluidsim_gfs", "-Wl,-rpath," + out, "-L" + lib_dir, "-lgfs", "-Wl,-rpath," + lib_dir],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    import torch
    gpu = int(torch.cuda.is_available())
    assert lines["init"] == f"{gpu} {gpu}"
    assert lines["threshold"] == "1 2.50"
    assert lines["vector"] == "3.0 15.75 0"
    assert lines["gpu"] == f"{gpu} 0"
