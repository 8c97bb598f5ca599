"""Shared pytest configuration.

`-m gpu` tests need a CUDA device and libgfs.so built for sm_103a (they fail,
not skip, without them: there is no CPU fallback); everything else runs on the
CPU (oracle pins, golden fixtures, ABI/symbol checks, host logic).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libgfs.so")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    from gridfluidsim3d_gb300 import build as gb
    gb.build()
    from gridfluidsim3d_gb300 import Context
    return Context(0)
