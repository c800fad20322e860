"""Shared test helpers. Tests marked ``gpu`` need a GB300 and the built
libns3d.so; everything else runs on the CPU (oracle, fixtures, ABI surface)."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libns3d.so")


@pytest.fixture(scope="session")
def ns3d():
    """The product package (ctypes binding over libns3d.so)."""
    return importlib.import_module("3d_navier_stokes_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O
