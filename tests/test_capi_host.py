"""The C-ABI library loads and exports every entry point of include/nsdg.h;
host-side argument validation works without touching a GPU."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from nextsimdg_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "nsdg.h"


def header_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nsdg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    fns = header_functions()
    for required in ("nsdg_kernel_create", "nsdg_kernel_initialise", "nsdg_kernel_set_data",
                     "nsdg_kernel_get_dg0", "nsdg_kernel_get_dg", "nsdg_kernel_update",
                     "nsdg_transport_step"):
        assert required in fns


def test_library_exports_every_header_symbol(nsdg_lib):
    missing = [f for f in header_functions() if not hasattr(nsdg_lib, f)]
    assert not missing, missing
    declared = {name for name, _, _ in _lib.SIGNATURES}
    assert set(header_functions()) == declared


def test_version_and_status_strings(nsdg_lib):
    assert b"sm_103a" in nsdg_lib.nsdg_version()
    assert nsdg_lib.nsdg_status_string(_lib.NSDG_ERR_UNKNOWN_FIELD) == b"unknown field"


def test_default_params_equal_oracle(nsdg_lib, oracle):
    p = _lib.default_params()
    q = oracle.default_params()
    for name, _ in _lib.Params._fields_:
        assert getattr(p, name) == getattr(q, name), name


def test_create_validates_arguments(nsdg_lib):
    h = ctypes.c_void_p()
    p = _lib.default_params()
    assert nsdg_lib.nsdg_kernel_create(7, 6, ctypes.byref(p), ctypes.byref(h)) == _lib.NSDG_ERR_BAD_ARG
    assert nsdg_lib.nsdg_kernel_create(0, 5, ctypes.byref(p), ctypes.byref(h)) == _lib.NSDG_ERR_BAD_ARG
    bad = _lib.default_params()
    bad.n_steps = 0
    assert nsdg_lib.nsdg_kernel_create(0, 6, ctypes.byref(bad), ctypes.byref(h)) == _lib.NSDG_ERR_BAD_ARG
    mixed = _lib.default_params()
    mixed.precision = 7
    assert nsdg_lib.nsdg_kernel_create(0, 6, ctypes.byref(mixed), ctypes.byref(h)) == _lib.NSDG_ERR_UNSUPPORTED
    assert nsdg_lib.nsdg_kernel_create(0, 6, ctypes.byref(p), ctypes.byref(h)) == _lib.NSDG_OK
    # calls before initialise fail cleanly, with a message
    buf = (ctypes.c_double * 4)()
    assert nsdg_lib.nsdg_kernel_set_data(h, b"hice", buf, 4, 1) == _lib.NSDG_ERR_BAD_ARG
    assert b"not initialised" in nsdg_lib.nsdg_kernel_last_error(h)
    assert nsdg_lib.nsdg_kernel_update(h, 0.0, 120.0) == _lib.NSDG_ERR_BAD_ARG
    assert nsdg_lib.nsdg_kernel_destroy(h) == _lib.NSDG_OK


def test_python_mirror_raises(nsdg_lib):
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel, NsdgError
    with pytest.raises(NsdgError):
        MEVPDynamicsKernel(dg_comp=4)
    k = MEVPDynamicsKernel(dg_comp=6)
    with pytest.raises(NsdgError):
        k.update(0.0, 120.0)
    k.close()


def test_parallelogram_mismatch_on_the_host(nsdg_lib):
    """Host only: operators rebuilt from parallelogram coefficients match the
    exact ones to FP64 rounding on box and sheared meshes, and not on a
    distorted mesh (which keeps the operator-streaming kernels)."""
    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import NsdgError, parallelogram_mismatch
    for n in (8, 33):
        b = BoxTest(n, n + 3)
        assert parallelogram_mismatch(b.coords(), n, n + 3) < 1e-12
    n = 12
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1))
    sheared = np.stack([(1000.0 * i + 300.0 * j).ravel(), (-200.0 * i + 900.0 * j).ravel()], axis=1)
    for dg in (1, 3, 6):
        assert parallelogram_mismatch(sheared, n, n, dg) < 1e-12
    rng = np.random.default_rng(4)
    distorted = sheared + rng.normal(0.0, 30.0, sheared.shape)
    assert parallelogram_mismatch(distorted, n, n) > 1e-3
    with pytest.raises(ValueError):
        parallelogram_mismatch(sheared[:-1], n, n)
    with pytest.raises(NsdgError):
        parallelogram_mismatch(sheared, n, n, 2)


def test_parallelogram_checks_on_the_host(nsdg_lib):
    """Host only: the checks behind the tiled transport and the parallelogram
    BBM kernel.  On box and sheared meshes the transport cell operators and
    the BBM projection and divergence operators rebuilt from the unit
    square's match the exact ones to FP64 rounding and M^{-1} is diagonal (the
    Legendre basis, constant J); a distorted mesh fails each check, as
    expected."""
    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import parallelogram_checks, parallelogram_mismatch
    n = 12
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1))
    sheared = np.stack([(1000.0 * i + 300.0 * j).ravel(), (-200.0 * i + 900.0 * j).ravel()], axis=1)
    for coords, nx, ny in ((BoxTest(9, 14).coords(), 9, 14), (sheared, n, n)):
        for dg in (1, 3, 6):
            c = parallelogram_checks(coords, nx, ny, dg)
            assert c["stress"] < 1e-12 and c["transport_cell"] < 1e-12, c
            assert c["minv_offdiag"] < 1e-13 and c["bbm"] < 1e-12, c
            assert c["stress"] == parallelogram_mismatch(coords, nx, ny, dg)
    rng = np.random.default_rng(4)
    distorted = sheared + rng.normal(0.0, 30.0, sheared.shape)
    c = parallelogram_checks(distorted, n, n, 6)
    assert c["stress"] > 1e-3 and c["transport_cell"] > 1e-3 and c["bbm"] > 1e-3, c
    assert c["minv_offdiag"] > 1e-6, c  # a general quadrilateral's mass matrix is not diagonal


def test_ice_growth_create_validates_arguments(nsdg_lib):
    """Host-side checks of the column-thermodynamics handle (no GPU call is
    made before they pass); the defaults equal the oracle's."""
    from oracle import pyoracle
    from nextsimdg_gb300.ice_growth import default_params
    p = default_params()
    o = pyoracle.ice_growth_params()
    for name, _ in p._fields_:
        assert getattr(p, name) == getattr(o, name), name
    assert _lib.ICE_GROWTH_FIELDS == pyoracle.IG_FIELDS
    h = ctypes.c_void_p()
    for bad in (dict(h0=0.0), dict(healing_time=-1.0), dict(thermo_model=3), dict(ks=float("nan"))):
        q = default_params(**bad)
        assert nsdg_lib.nsdg_ice_growth_create(4, None, ctypes.byref(q), ctypes.byref(h)) == _lib.NSDG_ERR_BAD_ARG
    assert nsdg_lib.nsdg_ice_growth_create(0, None, ctypes.byref(p), ctypes.byref(h)) == _lib.NSDG_ERR_BAD_ARG
    assert nsdg_lib.nsdg_ice_growth_exchange(None, None, 0) == _lib.NSDG_ERR_BAD_ARG
