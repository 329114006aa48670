"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and call the GB300 path through the C ABI
(libhsr.so); everything else runs on the CPU (oracle against the golden fixtures, host
logic, and that the library loads and exports its symbols).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "hana-softwarerenderer_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

# the library build script sits beside the package
sys.path.insert(0, os.path.join(ROOT, "hana-softwarerenderer_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libhsr.so")


@pytest.fixture(scope="session")
def gpu():
    """Initialise the library on device 0 once per session."""
    import hsr

    hsr.init(0)
    yield hsr
