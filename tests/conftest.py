"""Shared pytest configuration.

* ``gpu`` marks tests that need a GB300 (they call the CUDA path through the C ABI).
* The repository root (for ``oracle``) and ``incremental-fluids_gb300`` (for the
  ``ifluids`` package) are put on ``sys.path``.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "incremental-fluids_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (CUDA path through the C ABI)")


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import torch
            return torch.cuda.is_available()
        except Exception:
            return False
    n = ctypes.c_int(0)
    return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def ifl():
    """The built CUDA library (builds it when missing); GPU tests only."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ifluids_build", os.path.join(PKG, "build.py"))
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    pkg_build.build()
    import ifluids
    ifluids.load_library()
    return ifluids
