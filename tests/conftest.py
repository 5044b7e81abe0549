"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def goldens():
    return json.loads((ROOT / "tests" / "golden" / "transport_goldens.json").read_text())


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.load()
    return pyoracle


@pytest.fixture(scope="session")
def nsdg_lib():
    """The in-tree CUDA library (built if missing).  No CPU fallback exists."""
    from nextsimdg_gb300 import build, _lib
    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


def gpu_available() -> bool:
    import ctypes
    try:
        rt = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    n = ctypes.c_int(0)
    if rt.cuInit(0) != 0:
        return False
    if rt.cuDeviceGetCount(ctypes.byref(n)) != 0:
        return False
    return n.value > 0


@pytest.fixture(scope="session")
def gpu(nsdg_lib):
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return nsdg_lib


@pytest.fixture(scope="session")
def ref_goldens():
    """(case definitions module, read-outs) of tests/golden/ref_dynamics.npz:
    the reference's own dynamics code run on the cases of ref_cases.py."""
    import numpy as np
    gdir = ROOT / "tests" / "golden"
    if str(gdir) not in sys.path:
        sys.path.insert(0, str(gdir))
    import ref_cases
    z = np.load(gdir / "ref_dynamics.npz")
    data = {}
    for key in z.files:
        if "/" in key:
            case, name = key.split("/", 1)
            data.setdefault(case, {})[name] = z[key]
    return ref_cases, data
