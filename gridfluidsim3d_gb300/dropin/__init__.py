"""C++ drop-in replacements of GridFluidSim3D's PressureSolver, ParticleAdvector
and CLScalarField, forwarding to libgfs (include/gfs.h).

`build_reference_tree(src, out)` builds a GridFluidSim3D source tree with the
three classes replaced: it assembles in `out` a tree of symlinks to `src`
(the reference's `src/` directory, left untouched) in which the replaced
classes' files point at the files of this directory, compiles every
translation unit of the simulator library and its C bindings with g++, and
links them with libgfs.so into `out/libfluidsim_gfs.so` (and, with
`main=True`, the reference's example program into `out/fluidsim`).

    python -m gridfluidsim3d_gb300.dropin --src /path/to/GridFluidSim3D/src --out /tmp/fluidsim_gfs
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_build")

REPLACED = ("pressuresolver", "particleadvector", "clscalarfield")
OURS = [f"{n}.{e}" for n in REPLACED for e in ("h", "cpp")] + ["gfs_dropin.h", "gfs_dropin.cpp"]


def _mirror(src: str, out: str, skip: set) -> None:
    """Real directories, symlinked files (so that "../x.h" from a subdirectory
    resolves inside `out`, where the replaced headers live)."""
    os.makedirs(out, exist_ok=True)
    for name in os.listdir(src):
        if name in skip:
            continue
        s, link = os.path.join(src, name), os.path.join(out, name)
        if os.path.isdir(s):
            _mirror(s, link, set())
        elif not os.path.lexists(link):
            os.symlink(s, link)


def _assemble(src: str, out: str) -> None:
    _mirror(src, out, set(OURS) | {"config.h", "_obj", "_run"})
    for name in OURS:
        link = os.path.join(out, name)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink(os.path.join(HERE, name), link)
    # config.h from config.h.in (the reference's configure step), with throwaway paths
    cfg = open(os.path.join(src, "config.h.in")).read()
    cfg = re.sub(r"@CONFIG_[A-Z_]*@", os.path.join(out, "_run"), cfg)
    with open(os.path.join(out, "config.h"), "w") as f:
        f.write(cfg)


def _units(out: str, main: bool):
    units = [os.path.join(out, f) for f in sorted(os.listdir(out))
             if f.endswith(".cpp") and (main or f != "main.cpp")]
    cb = os.path.join(out, "c_bindings")
    if os.path.isdir(cb):
        units += [os.path.join(cb, f) for f in sorted(os.listdir(cb)) if f.endswith(".cpp")]
    return units


def _compile(unit: str, out: str, opt: str) -> str:
    obj = os.path.join(out, "_obj", os.path.relpath(unit, out).replace(os.sep, "_")[:-4] + ".o")
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    # -include limits: several reference units use std::numeric_limits without
    # including <limits> (g++ 13 no longer pulls it in transitively)
    cmd = ["g++", "-std=c++11", opt, "-fPIC", "-w", "-DNFLUIDSIMDEBUG", "-include", "limits", "-I" + out,
           "-I" + INCLUDE]
    cmd += ["-c", unit, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {unit}:\n{r.stderr[-4000:]}")
    return obj


def build_reference_tree(src: str, out: str, main: bool = False, opt: str = "-O2", jobs: int | None = None) -> dict:
    """Build the reference simulator with the drop-in classes; returns the paths built."""
    lib = os.path.join(LIBDIR, "libgfs.so")
    if not os.path.exists(lib):
        raise RuntimeError("libgfs.so is not built; run gridfluidsim3d_gb300.build.build() first")
    _assemble(src, out)
    units = _units(out, main=False)
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda u: _compile(u, out, opt), units))
    so = os.path.join(out, "libfluidsim_gfs.so")
    cmd = ["g++", "-shared", "-o", so] + objs + ["-L" + LIBDIR, "-lgfs", "-Wl,-rpath," + LIBDIR,
                                                 "-Wl,--no-undefined", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libfluidsim_gfs.so failed:\n{r.stderr[-4000:]}")
    built = {"library": so, "objects": objs}
    if main:
        mobj = _compile(os.path.join(out, "main.cpp"), out, opt)
        exe = os.path.join(out, "fluidsim")
        r = subprocess.run(["g++", "-o", exe, mobj, "-L" + out, "-lfluidsim_gfs", "-Wl,-rpath," + out,
                            "-L" + LIBDIR, "-lgfs", "-Wl,-rpath," + LIBDIR, "-lpthread"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of fluidsim failed:\n{r.stderr[-4000:]}")
        built["program"] = exe
    return built
