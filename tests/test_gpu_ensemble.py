"""Batched uneven ensembles: one graph per step, the mEVP sub-cycle of all
members in one element launch and one node launch per iteration.  Each
member must evolve exactly as it would alone (same arithmetic per element)."""
import numpy as np
import pytest

from nextsimdg_gb300.boxtest import BoxTest
from nextsimdg_gb300.dynamics import Ensemble, MEVPDynamicsKernel, NsdgError

pytestmark = pytest.mark.gpu

PRM = dict(alpha=300.0, beta=300.0, n_steps=40, precision=1)


def _member(box):
    k = MEVPDynamicsKernel(dg_comp=6, **PRM)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    return k


def _boxes():
    # uneven grids, perturbed cyclone tracks and thickness noise (seeded)
    sides = [(16, 16), (24, 20), (40, 33), (9, 70)]
    out = []
    for i, (nx, ny) in enumerate(sides):
        out.append(BoxTest(nx, ny, seed=i + 1, h_noise=0.02, start=(0.5e5 * (i + 4), 2.6e5),
                           wind_speed=8.0 + i))
    return out


def test_ensemble_members_match_single_runs(gpu):
    boxes = _boxes()
    ens_members = [_member(b) for b in boxes]
    solo = [_member(b) for b in boxes]
    ens = Ensemble(ens_members)
    for s in range(3):
        for b, k in zip(boxes, ens_members):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
        ens.update(s * 120.0, 120.0)
        for b, k in zip(boxes, solo):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
            k.update(s * 120.0, 120.0)
    ens.synchronize()
    for a, b in zip(ens_members, solo):
        for name in ("u", "v", "hice", "cice"):
            np.testing.assert_array_equal(a.getDG0Data(name), b.getDG0Data(name))
    for i in range(len(boxes)):
        w, h = ens.tile(i)
        # an autotuned 2-D tile of 64 elements, or 32 consecutive elements
        # for the TMA-staged and the parallelogram element kernels
        assert (w * h == 64 and w in (64, 32, 16, 8)) or (w, h) == (32, 1)
    assert ens.launches_per_update() < 2 * PRM["n_steps"] + 20 * len(boxes)


@pytest.mark.parametrize("kernel", ["affine", "tma", "global"])
def test_ensemble_both_element_kernels_match_single_runs(gpu, kernel, monkeypatch):
    """Each element kernel of the batched sub-cycle, forced through
    NSDG_STRESS_KERNEL, reproduces the members' single runs bitwise."""
    monkeypatch.setenv("NSDG_STRESS_KERNEL", kernel)
    boxes = [BoxTest(24, seed=1), BoxTest(40, 33, seed=2)]
    ens_members = [_member(b) for b in boxes]
    solo = [_member(b) for b in boxes]
    ens = Ensemble(ens_members)
    for s in range(2):
        for k, b in zip(ens_members, boxes):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
        ens.update(s * 120.0, 120.0)
        for k, b in zip(solo, boxes):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
            k.update(s * 120.0, 120.0)
    ens.synchronize()
    for a, b in zip(ens_members, solo):
        for name in ("u", "v", "hice", "cice"):
            np.testing.assert_array_equal(a.getDG0Data(name), b.getDG0Data(name))
    w, h = ens.tile(0)
    if kernel in ("tma", "affine"):
        assert (w, h) == (32, 1)
    else:
        assert w * h == 64
    assert ens_members[0].stress_variant()[0] == kernel


def test_ensemble_of_box_members_takes_the_parallelogram_kernel(gpu):
    """Without NSDG_STRESS_KERNEL, box members take the parallelogram
    coefficient kernel in their single runs and in the ensemble."""
    boxes = [BoxTest(24, seed=1), BoxTest(40, 33, seed=2)]
    members = [_member(b) for b in boxes]
    assert all(m.stress_variant()[0] == "affine" for m in members)
    ens = Ensemble(members)
    assert ens.tile(0) == (32, 1) and ens.tile(1) == (32, 1)


def test_ensemble_rejects_fp64_members(gpu):
    k = MEVPDynamicsKernel(dg_comp=6, n_steps=10)
    k.initialise(BoxTest(8).coords(), False, BoxTest(8).mask())
    with pytest.raises(NsdgError):
        Ensemble([k])


def test_persistent_subcycle_matches_the_per_phase_launches(gpu):
    """The sub-cycle as one persistent cooperative launch per step
    (nsdg_ensemble_set_persistent): bitwise the same as the per-phase
    launches and as the members stepped alone."""
    boxes = _boxes()
    persistent = [_member(b) for b in boxes]
    solo = [_member(b) for b in boxes]
    ens = Ensemble(persistent)
    ens.set_persistent(True)
    for s in range(3):
        for b, k in zip(boxes, persistent):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
        ens.update(s * 120.0, 120.0)
        for b, k in zip(boxes, solo):
            uw, vw = b.wind(s * b.dt)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
            k.update(s * 120.0, 120.0)
    ens.synchronize()
    for a, b in zip(persistent, solo):
        for name in ("u", "v", "hice", "cice", "uiostress"):
            np.testing.assert_array_equal(a.getDG0Data(name), b.getDG0Data(name))
    # one launch for the whole sub-cycle (plus its barrier reset)
    assert ens.launches_per_update() < 2 + 20 * len(boxes)
    ens.close()


def test_persistent_needs_parallelogram_members(gpu):
    box = BoxTest(16, distort=0.05)
    k = _member(box)
    ens = Ensemble([k])
    with pytest.raises(NsdgError) as e:
        ens.set_persistent(True)
    assert e.value.status == 6  # NSDG_ERR_UNSUPPORTED
    ens.close()
