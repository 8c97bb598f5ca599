"""The savestate format (FluidSimulationSaveState, fluidsimulationsavestate.cpp)
on the CPU: the oracle's restatement against the fixtures the reference's own
FluidSimulation wrote (tests/golden/make_savestate_golden.py), and libgfs's
header reader, which does file I/O only.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(HERE, "golden"))

from oracle import savestate as S  # noqa: E402

FIN = os.path.join(HERE, "golden", "savestate_in.state")
FREF = os.path.join(HERE, "golden", "savestate_ref.state")


def test_reference_resave_is_byte_identical():
    # the reference loaded the oracle-written file and saved it again: the
    # restatement writes exactly what the reference writes
    assert open(FIN, "rb").read() == open(FREF, "rb").read()


def test_oracle_reads_the_reference_file():
    import make_savestate_golden as G
    mat, pos, vel = G.scene()
    st = S.read_state(FREF)
    assert st["dims"] == G.DIMS and st["dx"] == G.DX and st["frame"] == G.FRAME and not st["brick"]
    assert np.array_equal(st["positions"], pos) and np.array_equal(st["velocities"], vel)
    assert len(st["diffuse_positions"]) == 0 and st["trailing_bytes"] == 0
    # solid cells in the reference's i-fastest order
    assert np.array_equal(st["solid_cells"], S.solid_cells(mat))
    order = st["solid_cells"][:, 0] + 12 * (st["solid_cells"][:, 1] + 10 * st["solid_cells"][:, 2])
    assert np.all(np.diff(order) > 0)
    assert np.array_equal(S.material_from_solid(G.DIMS, st["solid_cells"]), mat)


def test_oracle_round_trip(tmp_path):
    st = S.read_state(FREF)
    out = str(tmp_path / "rt.state")
    S.write_state(out, st["dims"], st["dx"], st["frame"], st["positions"], st["velocities"],
                  S.material_from_solid(st["dims"], st["solid_cells"]))
    assert open(out, "rb").read() == open(FREF, "rb").read()


def test_oracle_diffuse_section_offsets(tmp_path):
    rng = np.random.default_rng(3)
    mat = np.zeros((4, 5, 6), np.uint8)
    mat[0] = S.SOLID
    dif = (rng.random((7, 3), np.float32), rng.random((7, 3), np.float32), rng.random(7, np.float32),
           rng.integers(0, 3, 7).astype(np.int8))
    out = str(tmp_path / "d.state")
    S.write_state(out, (6, 5, 4), 0.5, 2, rng.random((11, 3)), rng.random((11, 3)), mat, diffuse=dif)
    st = S.read_state(out)
    assert np.array_equal(st["diffuse_lifetimes"], dif[2]) and np.array_equal(st["diffuse_types"], dif[3])
    assert len(st["solid_cells"]) == 30 and st["trailing_bytes"] == 0


def test_library_header_reader():
    from gridfluidsim3d_gb300 import FluidSimulationSaveState, GFSError, build
    if not os.path.exists(build.LIB):
        pytest.skip("libgfs.so not built")
    st = FluidSimulationSaveState()
    st.load_state(FREF)
    assert st.get_grid_dimensions() == (12, 10, 9) and st.get_cell_size() == 0.25
    assert st.get_current_frame() == 7 and st.get_num_marker_particles() == 300
    assert st.get_num_diffuse_particles() == 0 and not st.is_fluid_brick_grid_enabled()
    assert st.get_num_solid_cells() == len(S.read_state(FREF)["solid_cells"])
    with pytest.raises(GFSError):
        FluidSimulationSaveState().load_state(os.path.join(HERE, "golden", "no_such.state"))


def test_library_header_reader_truncated(tmp_path):
    from gridfluidsim3d_gb300 import FluidSimulationSaveState, GFSError, build
    if not os.path.exists(build.LIB):
        pytest.skip("libgfs.so not built")
    p = tmp_path / "short.state"
    p.write_bytes(open(FREF, "rb").read()[:20])
    with pytest.raises(GFSError, match="truncated"):
        FluidSimulationSaveState().load_state(str(p))


def test_library_header_reader_matches_oracle(tmp_path):
    """gfs_savestate_read_header (host-only: it opens and parses the file, no
    device work) through pyfluid's FluidSimulationSaveState, on every committed
    savestate fixture; a truncated and a missing file fail with GFSError."""
    import glob
    import shutil

    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no CUDA toolkit")
    from gridfluidsim3d_gb300 import FluidSimulationSaveState, GFSError, build
    build.build()
    files = sorted(glob.glob(os.path.join(HERE, "golden", "*.state")))
    assert len(files) >= 5
    for path in files:
        ref = S.read_state(path)
        st = FluidSimulationSaveState()
        assert st.load_state(path)
        assert st.get_grid_dimensions() == ref["dims"]
        assert st.get_cell_size() == ref["dx"]
        assert st.get_current_frame() == ref["frame"]
        assert st.get_num_marker_particles() == len(ref["positions"])
        assert st.get_num_diffuse_particles() == len(ref["diffuse_positions"])
        assert st.get_num_solid_cells() == len(ref["solid_cells"])
    cut = tmp_path / "cut.state"
    cut.write_bytes(open(files[0], "rb").read()[:20])
    with pytest.raises(GFSError, match="truncated"):
        FluidSimulationSaveState().load_state(str(cut))
    with pytest.raises(GFSError):
        FluidSimulationSaveState().load_state(str(tmp_path / "missing.state"))
