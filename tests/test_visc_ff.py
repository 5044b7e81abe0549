"""The float-float viscosity (nextsimdg_gb300/csrc/nsdg_visc_ff.hpp) on the
host: the same header the device compiles, built here with g++ and
-ffp-contract=off, so its IEEE FP32/FP64 operations round as on the GPU.

P/(8 alpha Delta) by one Newton step from a shared FP32 seed, in FP64 (the
stress kernels' form) and with float pairs on the FP32 pipe: over 7 M seeded
cases (strain invariants 0 to 1e-4 s^-2, subnormal ones, pressure terms from
FP64 subnormals to 1e6, four DeltaMin, seeds up to 3 ulps off) the two agree
except near rounding midpoints (bar: 1e-5 of the cases, measured 2e-6) and
never by more than one FP32 ulp, and both are within one ulp of
P / sqrt(inv + DeltaMin^2) correctly rounded."""
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "visc_ff_test.cpp"


def test_float_float_viscosity_matches_the_fp64_form(tmp_path):
    exe = tmp_path / "visc_ff_test"
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-Wall", "-ffp-contract=off",
           "-I", str(ROOT / "nextsimdg_gb300" / "csrc"), str(SRC), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    r = {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert r["samples"] == 7_000_000
    assert r["nonfinite"] == 0
    assert r["max_ulp_ab"] <= 1
    assert r["mismatch_ab"] <= 1e-5 * r["samples"], r
    assert r["max_ulp_fp64_ref"] <= 1 and r["max_ulp_ff_ref"] <= 1, r
