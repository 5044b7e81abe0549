"""Build recipe for the GB300 dynamics library (libnsdg_gb300.so).

Compiles the CUDA kernels for sm_103a with nvcc and the host-side C++
(FP64 precompute, C ABI) with g++, in parallel, and links one in-tree shared
library next to this file.  No PyTorch, no CMake.

    python -m nextsimdg_gb300.build [--verbose] [--ptxas]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libnsdg_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))

CU_SOURCES = ["nsdg_kernels.cu", "nsdg_stress_pairs.cu", "nsdg_forcing.cu", "nsdg_noalloc.cu", "nsdg_surrogate.cu", "nsdg_ice_growth.cu"]
CXX_SOURCES = ["nsdg_host.cpp", "nsdg_capi.cpp", "nsdg_transport_capi.cpp", "nsdg_ice_growth_capi.cpp",
               "nsdg_restart.cpp", "nsdg_restart_write.cpp", "nsdg_restart_capi.cpp"]
# per-file nvcc flags: the column thermodynamics and the benchmark forcing
# round every product and sum separately (no fused multiply-add), as the
# reference's and the oracle's arithmetic does
CU_FLAGS = {"nsdg_ice_growth.cu": ["--fmad=false"], "nsdg_forcing.cu": ["--fmad=false"]}


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _cxx() -> str:
    return os.environ.get("CXX", shutil.which("g++") or "g++")


def _sources_newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas: bool = False, force: bool = False) -> Path:
    """Compiles (if needed) and returns the path of libnsdg_gb300.so."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "nsdg.h"]
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [CSRC / src] + headers):
            cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", *CU_FLAGS.get(src, []), *inc, "-c", str(CSRC / src),
                   "-o", str(obj)]
            if ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [CSRC / src] + headers):
            cmd = [_cxx(), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                   "-Wno-unused-function", *inc, "-I", str(CUDA_HOME / "include"),
                   "-c", str(CSRC / src), "-o", str(obj)]
            jobs.append(cmd)
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if out and (verbose or ptxas or p.returncode):
            print(out, end="", flush=True)
        if p.returncode:
            failed.append(cmd[-3])
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, ptxas="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(LIB)
