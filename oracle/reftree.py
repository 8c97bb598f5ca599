"""The reference's whole simulator on the CPU (test infrastructure only).

`build_cpu_tree(src, out)` assembles, in `out`, a tree of symlinks to the
reference's `src/` directory (left untouched) in which only the two OpenCL
classes are replaced: `clscalarfield.h` / `particleadvector.h` by the drop-in
headers of this repository (gridfluidsim3d_gb300/dropin/), and their `.cpp`
files by the CPU backends in oracle/refcpu/, which run the reference's own
OpenCL-disabled arithmetic (ScalarField splat, MACVelocityField sampler, the
_RK1.._RK4 formulas).  Everything else -- fluidsimulation.cpp, the reference's
own PressureSolver, the data structures, the meshers and the savestate code --
is the reference's source, compiled unchanged with g++ into
`out/libfluidsim_refcpu.so`.  No GPU and no libgfs are involved.

`build_probe(tree, source, exe)` compiles a program against that library (the
fixture generators' probes, which drive private stages of FluidSimulation).

Only the fixture generators under tests/golden/ and the tests use this module.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DROPIN = os.path.join(ROOT, "gridfluidsim3d_gb300", "dropin")
REFCPU = os.path.join(HERE, "refcpu")

# tree file -> file of this repository
REPLACED = {
    "clscalarfield.h": os.path.join(DROPIN, "clscalarfield.h"),
    "particleadvector.h": os.path.join(DROPIN, "particleadvector.h"),
    "clscalarfield.cpp": os.path.join(REFCPU, "clscalarfield_cpu.cpp"),
    "particleadvector.cpp": os.path.join(REFCPU, "particleadvector_cpu.cpp"),
}
# units the simulator library needs (no main.cpp, no C bindings)
SKIP_UNITS = {"main.cpp"}

CXX = ["g++", "-std=c++11", "-fPIC", "-w", "-DNFLUIDSIMDEBUG", "-ffp-contract=off", "-include", "limits"]


def _mirror(src: str, out: str) -> None:
    os.makedirs(out, exist_ok=True)
    for name in os.listdir(src):
        if name in REPLACED or name in ("config.h", "_obj"):
            continue
        s, link = os.path.join(src, name), os.path.join(out, name)
        if os.path.isdir(s):
            if name in ("c_bindings", "pyfluid", "examples", "render", "kernels"):
                continue
            _mirror(s, link)
        elif not os.path.lexists(link):
            os.symlink(s, link)


def _assemble(src: str, out: str) -> None:
    _mirror(src, out)
    for name, target in REPLACED.items():
        link = os.path.join(out, name)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink(target, link)
    cfg = open(os.path.join(src, "config.h.in")).read()
    cfg = re.sub(r"@CONFIG_[A-Z_]*@", os.path.join(out, "_run"), cfg)
    with open(os.path.join(out, "config.h"), "w") as f:
        f.write(cfg)
    for d in ("logs", "savestates", "bakefiles", "temp"):
        os.makedirs(os.path.join(out, "_run", d), exist_ok=True)


def _compile(unit: str, out: str, opt: str) -> str:
    obj = os.path.join(out, "_obj", os.path.basename(unit)[:-4] + ".o")
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    deps = [os.path.realpath(unit)] + [os.path.realpath(p) for p in REPLACED.values()]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    r = subprocess.run(CXX + [opt, "-I" + out, "-c", unit, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {unit}:\n{r.stderr[-4000:]}")
    return obj


def build_cpu_tree(src: str, out: str, opt: str = "-O2", jobs: int | None = None) -> str:
    """Build the reference's simulator library with the CPU backends; returns its path."""
    _assemble(src, out)
    units = [os.path.join(out, f) for f in sorted(os.listdir(out)) if f.endswith(".cpp") and f not in SKIP_UNITS]
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda u: _compile(u, out, opt), units))
    so = os.path.join(out, "libfluidsim_refcpu.so")
    if not os.path.exists(so) or any(os.path.getmtime(o) > os.path.getmtime(so) for o in objs):
        r = subprocess.run(["g++", "-shared", "-o", so] + objs + ["-Wl,--no-undefined", "-lpthread"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libfluidsim_refcpu.so failed:\n{r.stderr[-4000:]}")
    return so


def build_probe(tree: str, source: str, exe: str, opt: str = "-O2") -> str:
    """Compile a probe program against the tree's library."""
    r = subprocess.run(CXX + [opt, "-I" + tree, source, "-o", exe, "-L" + tree, "-lfluidsim_refcpu",
                              "-Wl,-rpath," + tree], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"probe build failed:\n{r.stderr[-4000:]}")
    return exe
