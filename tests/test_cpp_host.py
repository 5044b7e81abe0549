"""The C++17 host class (include/nsdg_dynamics_kernel.hpp) compiles against the
C ABI, and on the GPU gives exactly what the Python mirror gives."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "host_kernel_test.cpp"


def _compile(tmp_path, nsdg_lib):
    exe = tmp_path / "host_kernel_test"
    libdir = ROOT / "nextsimdg_gb300"
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), str(SRC),
           "-L", str(libdir), "-l:libnsdg_gb300.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_host_class_compiles(tmp_path, nsdg_lib):
    assert _compile(tmp_path, nsdg_lib).exists()


@pytest.mark.gpu
def test_cpp_host_class_matches_python(tmp_path, gpu):
    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel

    exe = _compile(tmp_path, gpu)
    n, steps = 16, 2
    box = BoxTest(n)
    box.coords().tofile(tmp_path / "coords.bin")
    box.mask().ravel().tofile(tmp_path / "mask.bin")
    for name, arr in box.initial_fields().items():
        np.asarray(arr, dtype=np.float64).tofile(tmp_path / f"{name}.bin")
    for s in range(steps):
        uw, vw = box.wind(s * box.dt)
        uw.tofile(tmp_path / f"uwind_{s}.bin")
        vw.tofile(tmp_path / f"vwind_{s}.bin")
    r = subprocess.run([str(exe), str(tmp_path), str(n), str(steps)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    k = MEVPDynamicsKernel(dg_comp=6, alpha=300.0, beta=300.0)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    for s in range(steps):
        uw, vw = box.wind(s * box.dt)
        k.setData("uwind", uw)
        k.setData("vwind", vw)
        k.update(s * box.dt, box.dt)
    for name in ("hice", "cice", "u", "v", "uiostress", "viostress"):
        cpp = np.fromfile(tmp_path / f"out_{name}.bin")
        np.testing.assert_array_equal(cpp, k.getDG0Data(name))
