"""Autosave in FluidSimulation.update (FluidSimulation::update and _autosave,
fluidsimulation.cpp:3412-3435; pyfluid's enable_autosave property and
config.set_savestates_directory): with autosave on, every update first writes
`<savestates directory>/autosave.state` with the frame number before the step,
then steps.  Host logic only: the library is replaced by a recorder, so no GPU
is needed (the savestate writer itself is tested on the GPU in
tests/test_gpu_savestate.py).
"""
import os

import pytest

import gridfluidsim3d_gb300 as G
from gridfluidsim3d_gb300 import _lib, config


class Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append((name, args))
            return 0
        return fn


class FakeCtx:
    handle = None


@pytest.fixture
def fake(monkeypatch, tmp_path):
    rec = Recorder()
    monkeypatch.setattr(_lib, "lib", lambda: rec)
    old = config.get_savestates_directory()
    config.set_savestates_directory(tmp_path / "saves")
    yield rec
    config.set_savestates_directory(old)


def names(rec):
    return [c[0] for c in rec.calls if c[0] in ("gfs_sim_save_state", "gfs_sim_step")]


def test_autosave_off_by_default(fake):
    sim = G.FluidSimulation(8, 8, 8, 0.125, 100, ctx=FakeCtx())
    assert sim.enable_autosave is False
    sim.update(0.01)
    assert names(fake) == ["gfs_sim_step"]


def test_autosave_writes_before_each_step(fake, tmp_path):
    sim = G.FluidSimulation(8, 8, 8, 0.125, 100, ctx=FakeCtx())
    sim.enable_autosave = True
    sim.update(0.01)
    sim.update(0.01)
    assert names(fake) == ["gfs_sim_save_state", "gfs_sim_step"] * 2
    saves = [c[1] for c in fake.calls if c[0] == "gfs_sim_save_state"]
    path = os.path.join(str(tmp_path / "saves"), "autosave.state")
    assert [os.fsdecode(a[1]) for a in saves] == [path, path]
    assert [a[2] for a in saves] == [0, 1]        # the frame at the start of each update
    assert os.path.isdir(tmp_path / "saves")
    sim.enable_autosave = False
    sim.update(0.01)
    assert names(fake)[-1] == "gfs_sim_step" and names(fake).count("gfs_sim_save_state") == 2


def test_savestates_directory_roundtrip(tmp_path):
    old = config.get_savestates_directory()
    try:
        config.set_savestates_directory(os.fsencode(str(tmp_path)))
        assert config.get_savestates_directory() == str(tmp_path)
    finally:
        config.set_savestates_directory(old)
