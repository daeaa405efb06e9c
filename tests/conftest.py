"""Test configuration: the `gpu` marker and in-tree builds of the CPU parts.

GPU tests (marked ``gpu``) call the CUDA library through its C ABI and check it
against the CPU oracle (``oracle/``).  CPU tests cover the oracle against the
reference's golden vectors, the mesh builder, host logic and the ABI surface.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from hydro_rs_gb300 import build as B
    from oracle import oracle as O

    B.build_mesh()
    O.build()
    yield


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; fails (no skip) when absent."""
    from hydro_rs_gb300 import build as B
    from hydro_rs_gb300 import gpu as G

    B.build_gpu()
    return G.load_library()
