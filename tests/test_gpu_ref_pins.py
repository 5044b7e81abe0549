"""The GPU path against the reference's own results, through the C ABI.

The fixture tests/golden/ref_dynamics.npz holds the read-outs of the
reference's dynamics code (its unmodified sources built with the project's
Eigen subset, oracle/_ref) on the cases of tests/golden/ref_cases.py: box
tests with land holes, sea-surface height, unequal alpha and beta,
degenerate grids and masks, general quadrilaterals, and spherical patches.  The FP64 path must match every read-out within
1e-10 of the reference's magnitude; the mixed-precision path within its
stated tolerance (velocity RMS <= 1e-5 m/s, h and A RMS <= 1e-6).
"""
import numpy as np
import pytest

from nextsimdg_gb300.dynamics import BBMDynamicsKernel, MEVPDynamicsKernel

pytestmark = pytest.mark.gpu

TOL = 1e-10

ALL = ["mevp_dg6_a300_12x12", "mevp_dg3_a300_17x18", "mevp_dg1_a300_16x16", "mevp_dg6_a1500_32x32",
       "mevp_dg6_a1500_20x15_holes", "mevp_dg6_a300_64x64", "mevp_dg3_a1500_64x64", "bbm_dg6_14x14",
       "bbm_dg3_16x12", "mevp_dg6_a1500_256x256", "mevp_dg6_a1500_24x20_ssh", "bbm_dg6_16x14_ssh",
       "mevp_sph_dg3_a1500_20x16", "mevp_sph_dg6_a1500_20x16", "mevp_dg6_a300_20x18_distorted",
       "mevp_dg3_a1500_16x16_distorted", "bbm_dg6_14x12_distorted", "mevp_dg6_a300_b1500_18x16",
       "mevp_dg3_a1500_b300_16x18"]


def _kernel(case, precision):
    if case["rheology"] == 1:
        return BBMDynamicsKernel(dg_comp=case["dg"], n_steps=case["sub"], precision=precision)
    return MEVPDynamicsKernel(dg_comp=case["dg"], alpha=case["alpha"], beta=case.get("beta", case["alpha"]),
                              n_steps=case["sub"], precision=precision)


@pytest.mark.parametrize("stress", ["fma", "pairs", "pairs_tma"])
@pytest.mark.parametrize("name", ALL)
def test_fp64_matches_reference(gpu, ref_goldens, name, stress, monkeypatch):
    """FP64 GPU path vs the reference build: h, A (and damage) in every DG
    component, u, v and the ice-ocean stress, 1e-10 relative.  The 256 x 256
    case (alpha = beta = 1500) runs the 7 steps over which the reference's
    own sensitivity to h x (1 + 1e-14) stays below 1e-11.  Both mEVP stress
    kernels of the FP64 path: FP64 FMA (the default) and float-pair products
    with operators from global memory or staged by TMA
    (NSDG_FP64_STRESS=pairs, pairs_tma)."""
    monkeypatch.setenv("NSDG_FP64_STRESS", stress)
    cases, data = ref_goldens
    case = cases.CASES[name]
    k = _kernel(case, 0)
    got = cases.readouts(cases.run(k, case), case)
    k.close()
    worst = cases.compare(got, data[name])
    assert max(worst.values()) <= TOL, worst


DEGENERATE = ["mevp_dg6_a300_9x2", "mevp_dg3_a300_2x7", "mevp_dg6_a300_7x6_one", "mevp_dg6_a300_33x3_checker",
              "bbm_dg6_10x8_checker"]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", DEGENERATE)
def test_degenerate_cases_match_reference(gpu, ref_goldens, name, precision):
    """Two-row and two-column grids, one ice cell in land, a checkerboard of
    ice and land (mEVP and BBM) against the reference build: FP64 within
    1e-10 of every read-out; mixed precision within its stated tolerance."""
    cases, data = ref_goldens
    case = cases.CASES[name]
    k = _kernel(case, precision)
    got = cases.readouts(cases.run(k, case), case)
    k.close()
    ref = data[name]
    if precision == 0:
        worst = cases.compare(got, ref)
        assert max(worst.values()) <= TOL, worst
    else:
        rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
        du = rms(np.hypot(got["dg0_u"] - ref["dg0_u"], got["dg0_v"] - ref["dg0_v"]))
        dh = rms(got["dg0_hice"] - ref["dg0_hice"])
        da = rms(got["dg0_cice"] - ref["dg0_cice"])
        assert du <= 1e-5 and dh <= 1e-6 and da <= 1e-6, (du, dh, da)


DISTORTED = ["mevp_dg6_a300_20x18_distorted", "mevp_dg3_a1500_16x16_distorted", "bbm_dg6_14x12_distorted"]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", DISTORTED)
def test_general_quadrilaterals_match_reference(gpu, ref_goldens, name, precision):
    """General quadrilaterals (the box's vertices displaced as in the
    reference's distorted advection mesh) against the reference build: the
    per-element operator kernels of both paths, FP64 within 1e-10 of every
    read-out, mixed precision within its stated tolerance."""
    test_degenerate_cases_match_reference(gpu, ref_goldens, name, precision)


@pytest.mark.parametrize("name", ["mevp_dg6_a300_12x12", "mevp_dg6_a1500_32x32", "mevp_dg6_a300_64x64",
                                  "mevp_dg3_a1500_64x64", "mevp_dg3_a300_17x18", "mevp_dg1_a300_16x16",
                                  "mevp_dg6_a1500_20x15_holes", "mevp_dg6_a1500_24x20_ssh", "bbm_dg6_14x14",
                                  "bbm_dg3_16x12", "bbm_dg6_16x14_ssh", "mevp_sph_dg3_a1500_20x16",
                                  "mevp_sph_dg6_a1500_20x16", "mevp_dg6_a300_b1500_18x16",
                                  "mevp_dg3_a1500_b300_16x18"])
def test_mixed_precision_within_stated_tolerance_of_reference(gpu, ref_goldens, name):
    """Mixed precision (FP32 bulk; FP64 conservation sums, inverse mass
    matrices, Delta and viscosity) against the reference's FP64 results."""
    cases, data = ref_goldens
    case = cases.CASES[name]
    k = _kernel(case, 1)
    cases.run(k, case)
    ref = data[name]
    rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
    du = rms(np.hypot(k.getDG0Data("u") - ref["dg0_u"], k.getDG0Data("v") - ref["dg0_v"]))
    dh = rms(k.getDG0Data("hice") - ref["dg0_hice"])
    da = rms(k.getDG0Data("cice") - ref["dg0_cice"])
    k.close()
    print(f"{name} mixed vs reference: velocity RMS {du:.2e} m/s, h RMS {dh:.2e} m, A RMS {da:.2e}")
    assert du <= 1e-5 and dh <= 1e-6 and da <= 1e-6, (du, dh, da)
