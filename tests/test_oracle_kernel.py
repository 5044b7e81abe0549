"""CPU-only checks of the oracle's dynamics kernel (the parity reference)."""
import numpy as np
import pytest

from nextsimdg_gb300.boxtest import BoxTest


def _run(oracle, n=12, dg=6, steps=2, rheology=0, threads=None, **kw):
    if threads:
        oracle.set_threads(threads)
    box = BoxTest(n)
    k = oracle.OracleKernel(rheology, dg, alpha=300.0, beta=300.0, n_steps=kw.pop("n_steps", 20), **kw)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    if rheology == 1:
        k.setData("damage", box.damage())
    for s in range(steps):
        uw, vw = box.wind(s * box.dt)
        k.setData("uwind", uw)
        k.setData("vwind", vw)
        k.update(s * box.dt, box.dt)
    return k


def test_default_params_match_reference(oracle):
    p = oracle.default_params()
    assert p.rho_ice == 900.0 and p.Pstar == 27500.0 and p.DeltaMin == 2e-9
    assert p.alpha == 1500.0 and p.beta == 1500.0 and p.n_steps == 100
    assert p.F_ocean == pytest.approx(5.5e-3 * 1026.0) and p.F_atm == pytest.approx(1.2e-3 * 1.3)
    assert p.young == 5.96e8 and p.nu0 == pytest.approx(1 / 3)


@pytest.mark.parametrize("dg", [1, 3, 6])
def test_mevp_runs_and_is_thread_independent(oracle, dg):
    a = _run(oracle, dg=dg, threads=1)
    b = _run(oracle, dg=dg, threads=4)
    for name in ("u", "v", "hice", "cice"):
        x, y = a.getDG0Data(name), b.getDG0Data(name)
        assert np.all(np.isfinite(x))
        np.testing.assert_array_equal(x, y)
    assert np.abs(a.getDG0Data("u")).max() > 1e-4  # the wind moves the ice


def test_bbm_runs(oracle):
    k = _run(oracle, rheology=1, steps=2)
    d = k.getDG0Data("damage")
    assert np.all(np.isfinite(d)) and d.max() <= 1.0 + 1e-12


def test_ma2dg_truncation(oracle):
    """setData with a DG0 array zeroes the higher components (DGModelArray.hpp:20-32)."""
    box = BoxTest(6)
    k = oracle.OracleKernel(0, 6)
    k.initialise(box.coords(), False, box.mask())
    full = np.random.default_rng(1).standard_normal((36, 6))
    k.setData("hice", full)
    np.testing.assert_array_equal(k.getDGData("hice"), full)
    k.setData("hice", full[:, 0])
    g = k.getDGData("hice")
    np.testing.assert_array_equal(g[:, 0], full[:, 0])
    assert not g[:, 1:].any()
    with pytest.raises(KeyError):
        k.getDG0Data("nonexistent")
    k.setData("tracer", full[:, 0])
    np.testing.assert_array_equal(k.getDG0Data("tracer"), full[:, 0])


def test_tables_match_formulas(oracle):
    import ctypes
    out = np.empty(8 * 9)
    oracle.load().oracle_table(b"PSI", 8, 3, out.ctypes.data_as(ctypes.c_void_p))
    gp = 0.5 + np.array([-np.sqrt(3 / 20), 0.0, np.sqrt(3 / 20)])
    x = np.tile(gp, 3)
    y = np.repeat(gp, 3)
    assert np.allclose(out[0:9], 1.0)
    assert np.allclose(out[9:18], x - 0.5)
    assert np.allclose(out[18:27], y - 0.5)
    assert np.allclose(out[63:72], (x - 0.5) * ((y - 0.5) ** 2 - 1 / 12))
