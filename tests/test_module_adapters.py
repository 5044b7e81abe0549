"""The dynamics modules (IDynamics implementations) on the reference's own
module framework.

`make -C oracle module` compiles the reference's module layer (IDynamics,
ModelComponent and the shared array store, the configuration layer against
the project's Boost.ProgramOptions subset in oracle/boost_min) and its
MEVPDynamics and BBMDynamics modules, unmodified, next to the product's
adapters GPUMEVPDynamics and GPUBBMDynamics (nextsimdg_gb300/module/),
linked against the product library with every symbol resolved.
oracle/module_harness.cpp drives a module as the model does
(PrognosticData.cpp:60-118): setData with the initial state, then per step
the forcing in the shared store, update, and the updated damage handed back.

* The reference's modules give exactly what their kernels give when driven
  by the same calls directly (the module step is MEVPDynamics.cpp:59-95 /
  BBMDynamics.cpp:63-104 around the kernel), so the harness drives modules
  correctly.
* The adapters read their precision through the reference's configuration
  layer (Configured::getConfiguration), and an invalid value is an error.
* The adapters run the same module step on the GB300 kernel: where a GPU is
  present they match the reference's modules (FP64: 1e-10 relative, the
  bar of the kernel-level tests); without one, the kernel creation's error
  reaches the caller through the module.

These need the reference sources, so they run where those are and skip
elsewhere.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from nextsimdg_gb300.boxtest import BoxTest
from oracle import pyref

pytestmark = pytest.mark.skipif(pyref.reference_root() is None, reason="needs the reference sources")

READS = ("hice", "cice", "u", "v", "taux", "tauy")


@pytest.fixture(scope="module")
def modlib():
    from nextsimdg_gb300 import _lib
    _lib.load()  # the product library the adapters link against
    pyref.build()
    if pyref.build_module() is None:
        pytest.skip("module build unavailable")
    return pyref.load_module()


def _gpu_present() -> bool:
    try:
        cudart = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import torch
            return bool(torch.cuda.is_available())
        except Exception:
            return False
    n = ctypes.c_int(0)
    return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


def drive_module(m: pyref.DynamicsModule, b: BoxTest, steps: int, damage=None) -> dict:
    f = b.initial_fields()
    m.set_state(b.coords(), b.mask(), f["hice"], f["cice"], f["u"], f["v"], damage=damage)
    for s in range(steps):
        uw, vw = b.wind(s * b.dt)
        m.step(s * b.dt, b.dt, uw, vw, f["uocean"], f["vocean"], f["ssh"])
    out = {n: m.get(n) for n in READS}
    if m.kind.endswith("BBMDynamics"):
        out["damage"] = m.get("damage")
    return out


def drive_kernel(k, b: BoxTest, steps: int, bbm: bool, damage=None) -> dict:
    """The same calls made on a kernel directly: MEVPDynamics::setData /
    BBMDynamics::setData, then per step the module's setData calls, update,
    and the DG0 read-outs that become the next step's h, A (and damage)."""
    f = b.initial_fields()
    k.initialise(b.coords(), False, b.mask())
    for n in ("hice", "cice", "u", "v"):
        k.setData(n, f[n])
    # without a damage field the model starts from damage 1 everywhere
    # (PrognosticData.cpp:70-75); each update sets the damage the model holds
    d = (damage if damage is not None else np.ones(b.nelements)) if bbm else None
    if bbm:
        k.setData("damage", d)
    h, a = f["hice"], f["cice"]
    for s in range(steps):
        k.setData("hice", h)
        k.setData("cice", a)
        if bbm:
            k.setData("damage", d)
        uw, vw = b.wind(s * b.dt)
        for n, v in (("uwind", uw), ("vwind", vw), ("uocean", f["uocean"]), ("vocean", f["vocean"]),
                     ("ssh", f["ssh"])):
            k.setData(n, v)
        k.update(s * b.dt, b.dt)
        h, a = k.getDG0Data("hice"), k.getDG0Data("cice")
        if bbm:
            d = k.getDG0Data("damage")
    out = {"hice": h, "cice": a, "u": k.getDG0Data("u"), "v": k.getDG0Data("v"),
           "taux": k.getDG0Data("uiostress"), "tauy": k.getDG0Data("viostress")}
    if bbm:
        out["damage"] = d
    return out


@pytest.mark.parametrize("kind,bbm", [("MEVPDynamics", False), ("BBMDynamics", True)])
def test_reference_module_equals_its_kernel(modlib, kind, bbm):
    b = BoxTest(12)
    m = pyref.DynamicsModule(kind, 12, 12)
    got = drive_module(m, b, 3)
    m.close()
    k = pyref.RefKernel(rheology=1 if bbm else 0, dg_comp=6)
    want = drive_kernel(k, b, 3, bbm)
    k.close()
    for n, w in want.items():
        np.testing.assert_array_equal(got[n], w, err_msg=n)
    assert np.abs(got["u"]).max() > 1e-3  # the ice moved


@pytest.mark.parametrize("kind", ["GPUMEVPDynamics", "GPUBBMDynamics"])
def test_adapter_reads_its_precision_from_the_configuration(modlib, kind):
    m = pyref.DynamicsModule(kind, 8, 8)
    m.configure("")
    assert m.precision == 0  # the default: FP64, the reference's arithmetic
    m.configure("[GPUDynamics]\nprecision = mixed\n")
    assert m.precision == 1
    m.configure("[GPUDynamics]\nprecision = fp64  # comment\n")
    assert m.precision == 0
    with pytest.raises(RuntimeError, match="precision"):
        m.configure("[GPUDynamics]\nprecision = half\n")
    m.close()


def test_reference_module_configure_selects_no_healing(modlib):
    m = pyref.DynamicsModule("MEVPDynamics", 8, 8)
    m.configure("")  # Module<IDamageHealing>::setImplementation("Nextsim::NoHealing")
    m.close()


@pytest.mark.parametrize("kind,ref_kind", [("GPUMEVPDynamics", "MEVPDynamics"), ("GPUBBMDynamics", "BBMDynamics")])
def test_adapter_module_step(modlib, kind, ref_kind):
    b = BoxTest(12)
    if not _gpu_present():
        m = pyref.DynamicsModule(kind, 12, 12)
        f = b.initial_fields()
        with pytest.raises(RuntimeError) as e:
            m.set_state(b.coords(), b.mask(), f["hice"], f["cice"], f["u"], f["v"])
        assert "create" in str(e.value) or "initialise" in str(e.value)
        m.close()
        return
    r = pyref.DynamicsModule(ref_kind, 12, 12)
    want = drive_module(r, b, 3)
    r.close()
    m = pyref.DynamicsModule(kind, 12, 12)
    got = drive_module(m, b, 3)
    m.close()
    for n, w in want.items():
        scale = max(float(np.abs(w).max()), 1e-300)
        assert float(np.abs(got[n] - w).max()) / scale <= 1e-10, n
