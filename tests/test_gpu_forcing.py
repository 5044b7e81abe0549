"""The benchmark forcing computed on the device (nsdg_kernel_benchmark_ocean,
nsdg_kernel_benchmark_atmosphere) against the same fields computed on the
host by the oracle's restatement and passed with setData: the dynamics
driven either way agree to rounding, in FP64 and in mixed precision."""
import numpy as np
import pytest

from nextsimdg_gb300 import _lib
from nextsimdg_gb300.boxtest import BoxTest
from nextsimdg_gb300.dynamics import MEVPDynamicsKernel

pytestmark = pytest.mark.gpu


def _run(box, f, device, oracle, precision, steps=4):
    k = MEVPDynamicsKernel(dg_comp=6, alpha=1500.0, beta=1500.0, n_steps=100, precision=precision)
    k.initialise(box.coords(), False, box.mask())
    for name in ("hice", "cice", "u", "v", "ssh"):
        k.setData(name, box.initial_fields()[name])
    if device:
        k.benchmark_ocean(f)
    else:
        _, _, uo, vo = oracle.benchmark_forcing_fields(box.nx, box.ny, f, 0.0)
        k.setData("uocean", uo)
        k.setData("vocean", vo)
    for s in range(steps):
        t = s * box.dt
        if device:
            k.benchmark_atmosphere(f, t)
        else:
            uw, vw, _, _ = oracle.benchmark_forcing_fields(box.nx, box.ny, f, t)
            k.setData("uwind", uw)
            k.setData("vwind", vw)
        k.update(t, box.dt)
    out = {n: k.getDG0Data(n) for n in ("u", "v", "hice", "uiostress")}
    k.close()
    return out


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["reference", "box"])
def test_device_forcing_matches_host_forcing(gpu, oracle, precision, which):
    box = BoxTest(48, 40)
    f = _lib.benchmark_forcing(512e3, 512e3) if which == "reference" else box.device_forcing()
    a = _run(box, f, True, oracle, precision)
    b = _run(box, f, False, oracle, precision)
    for n in a:
        scale = np.abs(b[n]).max()
        assert np.abs(a[n] - b[n]).max() <= 1e-11 * scale, n
    assert np.abs(b["u"]).max() > 1e-3


def test_device_forcing_errors(gpu):
    k = MEVPDynamicsKernel(dg_comp=6)
    f = _lib.benchmark_forcing()
    with pytest.raises(Exception):
        k.benchmark_atmosphere(f, 0.0)  # not initialised
    box = BoxTest(8)
    k.initialise(box.coords(), False, box.mask())
    bad = _lib.benchmark_forcing(0.0, 512e3)
    with pytest.raises(Exception):
        k.benchmark_ocean(bad)
    k.close()
