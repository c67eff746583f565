"""Test configuration: the `gpu` marker and in-tree builds.

Tests marked ``gpu`` need a CUDA device (they run on the GPU machine); the rest
run on any machine.  The library and the oracle are (re)built in-tree once
per session when their sources are newer than the built files.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long statistical run")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from gpusmoldyn_gb300 import build as libbuild
    from oracle import build as obuild

    libbuild.build()
    obuild.build_oracle()
    yield
