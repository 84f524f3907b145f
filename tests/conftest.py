"""Test configuration: import paths, the `gpu` marker, and build helpers.

CPU tests (-m "not gpu") check the oracle against the reference's golden
fixtures, the host-side input handling and the C-ABI library's exports.  GPU
tests (-m gpu) are the parity tests proper: CUDA path vs oracle through the
C ABI."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "energy-stability_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (CUDA path parity tests)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle_py
    if not os.path.exists(oracle_py.LIB_PATH):
        oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def sclet_lib():
    """The CUDA library (built if missing).  Loading needs no GPU."""
    import build_ext
    build_ext.build()
    import sclet_gb300
    sclet_gb300.lib()
    return sclet_gb300


@pytest.fixture(scope="session")
def gpu_available():
    try:
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=60)
        return r.returncode == 0 and "GPU" in r.stdout
    except Exception:
        return False
