"""Directories the simulation writes to, as pyfluid's config module names them
(pyfluid/config.py, Config::getSavestatesDirectory / setSavestatesDirectory in
config.cpp:46-67).  Only the savestates directory is used here: the autosave of
FluidSimulation.update writes `<savestates directory>/autosave.state`.

The default is `savestates` under the working directory at import time.  The
reference's default is a build-time path (CONFIG_SAVESTATES_DIR).
"""
import os

_savestates_directory = os.path.join(os.getcwd(), "savestates")


def get_savestates_directory() -> str:
    return _savestates_directory


def set_savestates_directory(directory) -> None:
    global _savestates_directory
    _savestates_directory = os.fsdecode(directory)
