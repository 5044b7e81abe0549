"""The float-float viscosity (nextsimdg_gb300/csrc/nsdg_visc_ff.hpp) on the
host: the same header the device compiles, built here with g++ and
-ffp-contract=off, so its IEEE FP32/FP64 operations round as on the GPU.

P/(8 alpha Delta) by one Newton step from a shared FP32 seed, in FP64 (the
stress kernels' form) and with float pairs on the FP32 pipe: over 7 M seeded
cases (strain invariants 0 to 1e-4 s^-2, subnormal ones, pressure terms from
FP64 subnormals to 1e6, four DeltaMin, seeds up to 3 ulps off) the two agree
except near rounding midpoints (bar: 1e-5 of the cases, measured 2e-6) and
never by more than one FP32 ulp, and both are within one ulp of
P / sqrt(inv + DeltaMin^2) correctly rounded.  The checked float-float form
(the kernels' form 4) reports where its result is provably the FP64 form's:
there it is bitwise equal, over the random cases and over 3 M cases aimed at
float rounding midpoints.  On the GPU: the device build
against form 2, and the stress kernel with form 3 (time_kernel id 8)."""
import shutil
import subprocess
from pathlib import Path

import pytest

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
    # the checked form (the kernels' form 4): where it reports exact, bitwise
    # the FP64 form, including on values aimed at rounding midpoints; every
    # value within 2^-40 of a midpoint (11 of the 15 offsets) goes to the
    # FP64 form; on physical pressure terms it falls back rarely
    assert r["checked_wrong"] == 0, r
    assert r["adv_wrong"] == 0, r
    assert r["adv_fallback"] >= 11 * r["adv_samples"] // 15, r
    assert r["phys_fallback"] <= 5e-4 * r["phys_samples"], r


@pytest.mark.gpu
def test_float_float_viscosity_on_the_gpu(gpu):
    """The device build of the same header: form 3 against form 2 on the GPU
    (same rsqrtf seed), then the parallelogram stress kernel with form 3
    (time_kernel id 8) on a 64^2 box, after which the handle still steps."""
    import numpy as np

    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel, selftest_viscosity, selftest_viscosity_ff
    rng = np.random.default_rng(5)
    n = 1 << 18
    inv = np.concatenate([[0.0, 1e-45, 1e-40, 1.1754942e-38, 4e-18],
                          10.0 ** rng.uniform(-36, -4, n - 5)]).astype(np.float32)
    pa = np.concatenate([[0.0, 1e-300, 1e-31, 12.5, 1e3], 10.0 ** rng.uniform(-3, 4, n - 5)])
    f2 = selftest_viscosity(inv, pa, 2e-9)[2]
    f3 = selftest_viscosity_ff(inv, pa, 2e-9)
    assert np.all(np.isfinite(f3))
    d = np.abs(f3.astype(np.float64) - f2.astype(np.float64))
    assert np.all(d <= np.spacing(np.abs(f2)).astype(np.float64))
    assert np.mean(d == 0) >= 1 - 1e-4, np.mean(d == 0)

    box = BoxTest(64)
    k = MEVPDynamicsKernel(dg_comp=6, alpha=300.0, beta=300.0, n_steps=100, precision=1)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    k.update(0.0, box.dt)
    ms, name = k.time_kernel(8, 5)
    assert ms > 0 and name == "kMevpStress32Affine"
    k.update(box.dt, box.dt)
    assert np.all(np.isfinite(k.getDG0Data("u")))
    k.close()
