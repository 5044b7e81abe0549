"""GPU column thermodynamics (IceGrowth + ThermoIce0 or ThermoWinton +
HiblerSpread + ConstantHealing) against the CPU oracle, through the C ABI.

The bar is bit-identity: the kernel is element-local FP64 arithmetic in the
reference's operation order, compiled without fused multiply-adds, so every
slot (inputs, outputs, the heat fluxes and damage it modifies, and the
outputs an update leaves untouched) must equal the oracle's exactly, over
several steps, at the 512 x 512 benchmark size and on the edge cases the
reference guards (no ice, ice below the minima, no snow, land)."""
import numpy as np
import pytest

from nextsimdg_gb300._lib import ICE_GROWTH_FIELDS, NsdgError, NSDG_ERR_BAD_ARG, NSDG_ERR_SIZE_MISMATCH
from nextsimdg_gb300._lib import NSDG_ERR_UNKNOWN_FIELD

pytestmark = pytest.mark.gpu

INPUTS = ("hice", "cice", "hsnow", "tice", "qia", "dqia_dt", "qow", "qio", "sublim", "snowfall", "penSW", "sst",
          "tf", "mlbhc", "damage", "tice_1", "tice_2")


def _inputs(n, rng, po):
    """Seeded forcing and state with the reference's edge cases mixed in."""
    cice = rng.uniform(0.0, 1.0, n)
    cice[rng.random(n) < 0.05] = 0.0
    cice[rng.random(n) < 0.02] = 1e-13          # below c_min
    cice[rng.random(n) < 0.05] = 1.0
    hice = rng.uniform(0.0, 3.0, n) * cice
    hice[rng.random(n) < 0.05] = 0.0
    thin = rng.random(n) < 0.03
    hice[thin] = 0.004 * cice[thin]                # true thickness below h_min
    hsnow = rng.uniform(0.0, 0.4, n) * cice
    hsnow[rng.random(n) < 0.2] = 0.0
    sss = rng.uniform(30.0, 35.0, n)
    tf = np.array([po.unesco_freezing(s) for s in sss[:64]])[rng.integers(0, 64, n)]
    qio = rng.uniform(0.0, 200.0, n)
    qio[rng.random(n) < 0.01] = 5e4                # complete melt
    return dict(hice=hice, cice=cice, hsnow=hsnow, tice=rng.uniform(-30.0, 0.0, n), qia=rng.uniform(-100, 400, n),
                dqia_dt=rng.uniform(0.0, 30.0, n), qow=rng.uniform(-200.0, 400.0, n), qio=qio,
                sublim=rng.uniform(-1e-5, 1e-5, n), snowfall=rng.uniform(0.0, 1e-4, n) * (rng.random(n) < 0.5),
                penSW=rng.uniform(0.0, 50.0, n), sst=tf + rng.uniform(-0.2, 2.0, n), tf=tf,
                mlbhc=4186.84e3 * rng.uniform(5.0, 50.0, n), damage=rng.uniform(0.0, 1.0, n),
                tice_1=rng.uniform(-25.0, -0.5, n), tice_2=rng.uniform(-15.0, -0.3, n))


def _pair(n, mask, oracle_mod, **params):
    from nextsimdg_gb300.ice_growth import IceGrowth
    g = IceGrowth(n, mask=mask, **params)
    o = oracle_mod.OracleIceGrowth(n, mask=mask, **params)
    return g, o


def _compare_all(g, o):
    for name in ICE_GROWTH_FIELDS:
        np.testing.assert_array_equal(g.getData(name), o.getData(name), err_msg=name)


@pytest.mark.parametrize("params", [
    {}, dict(thermo_model=1), dict(lateral_model=1), dict(healing_model=1), dict(use_thermo=0),
    dict(flooding=0), dict(thermo_model=1, lateral_model=1), dict(thermo_model=2), dict(thermo_model=2, flooding=0)])
def test_ice_growth_bitwise_equals_oracle(gpu, oracle, params):
    from oracle import pyoracle as po
    rng = np.random.default_rng(4)
    n = 20_000
    mask = (rng.random(n) > 0.1).astype(np.float64)
    g, o = _pair(n, mask, po, **params)
    for step, dt in enumerate((600.0, 3600.0, 86400.0, 120.0)):
        fresh = _inputs(n, rng, po)
        for name in INPUTS if step == 0 else ("qia", "dqia_dt", "qow", "qio", "sublim", "snowfall", "penSW",
                                              "sst", "tf"):
            g.setData(name, fresh[name])
            o.setData(name, fresh[name])
        if step > 0:  # the next step starts from the cell averages of this one (PrognosticData)
            for k in (g, o):
                c = k.getData("cice_updated")
                k.setData("hice", k.getData("hice_updated") * c)
                k.setData("hsnow", k.getData("hsnow_updated") * c)
                k.setData("cice", c)
                k.setData("tice", k.getData("tice_updated"))
                k.setData("tice_1", k.getData("tice_updated_1"))
                k.setData("tice_2", k.getData("tice_updated_2"))
        g.update(dt)
        o.update(dt)
        _compare_all(g, o)
    if params.get("use_thermo", 1):
        assert np.count_nonzero(g.getData("newice")) > 100
    if params.get("thermo_model") == 2:
        assert np.all(np.isfinite(g.getData("tice_updated_1")))
    if not params:
        assert np.count_nonzero(g.getData("snow_to_ice")) > 10
        assert np.count_nonzero(g.getData("delta_cmelt")) > 100


def test_ice_growth_full_size_bitwise(gpu, oracle):
    """The 512 x 512 benchmark size: every slot bit-identical after one step."""
    from oracle import pyoracle as po
    rng = np.random.default_rng(9)
    n = 512 * 512
    g, o = _pair(n, None, po)
    for name, arr in _inputs(n, rng, po).items():
        g.setData(name, arr)
        o.setData(name, arr)
    g.update(600.0)
    o.update(600.0)
    _compare_all(g, o)


@pytest.mark.parametrize("case", ["new_ice", "melting", "freezing"])
def test_reference_known_answers_on_gpu(gpu, case):
    """physics/test/IceGrowth_test.cpp cases through the GPU handle."""
    from oracle import pyoracle as po
    from nextsimdg_gb300.ice_growth import IceGrowth
    c = {"new_ice": (0.5, 0.1, 0.0, -2.0, 305.288, 4.5036, 307.546, 0.0, 0.0, -1.5, 124.689, 86400.0),
         "melting": (0.5, 0.1, 0.01, -1.0, -84.5952, 19.7016, -109.923, -7.3858e-06, 0.0, -1.0, 53717.8, 600.0),
         "freezing": (0.5, 0.1, 0.01, -9.0, 42.2955, 16.7615, 143.266, 2.15132e-6, 1e-3, -1.75, 73.9465, 600.0)}[case]
    cice, hice, hsnow, tice, qia, dqia, qow, subl, snow, sst, qio, dt = c
    g = IceGrowth(1)
    for k, v in dict(cice=cice, hice=hice, hsnow=hsnow, tice=tice, qia=qia, dqia_dt=dqia, qow=qow, sublim=subl,
                     snowfall=snow, sst=sst, tf=po.unesco_freezing(32.0), mlbhc=1000.0 * 4186.84 * 10.25, qio=qio,
                     damage=1.0).items():
        g.setData(k, v)
    g.update(dt)
    ap = lambda a, b: abs(a - b) < 1e-5 * (1 + max(abs(a), abs(b)))  # noqa: E731 (doctest Approx)
    ci = g.getData("cice_updated")[0]
    hc = g.getData("hice_updated")[0] * ci
    sc = g.getData("hsnow_updated")[0] * ci
    ni = g.getData("newice")[0]
    if case == "new_ice":
        assert ap(ni, 0.0258264)
    elif case == "melting":
        assert ap(ci, 0.368269) and ap(hc, 0.0473078) and ap(sc, 0.00720977) and ni == 0.0
    else:
        assert ap(ci, 0.5002) and ap(hc, 0.100039) and ap(sc, 0.0109012) and ap(ni, 6.79906e-5)


@pytest.mark.parametrize("rheology", ["mevp", "bbm"])
def test_exchange_with_dynamics(gpu, rheology):
    """PrognosticData's round trip on the device: the dynamics' DG0 h, A (and
    BBM damage) into the growth step, the updated cell averages back as
    one-component fields (higher DG components zero), with the same values
    the host round trip would give."""
    from oracle import pyoracle as po
    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import BBMDynamicsKernel, MEVPDynamicsKernel
    from nextsimdg_gb300.ice_growth import IceGrowth
    box = BoxTest(16)
    cls = BBMDynamicsKernel if rheology == "bbm" else MEVPDynamicsKernel
    k = cls(dg_comp=6, n_steps=10)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    if rheology == "bbm":
        k.setData("damage", np.full(box.nx * box.ny, 0.7))
    uw, vw = box.wind(0.0)
    k.setData("uwind", uw)
    k.setData("vwind", vw)
    k.update(0.0, 120.0)
    n = box.nx * box.ny
    rng = np.random.default_rng(2)
    forcing = _inputs(n, rng, po)
    g = IceGrowth(n, mask=box.mask())
    for name in INPUTS:
        if name not in ("hice", "cice") and not (name == "damage" and rheology == "bbm"):
            g.setData(name, forcing[name])
    g.exchange(k, 0)
    np.testing.assert_array_equal(g.getData("hice"), k.getDG0Data("hice"))
    np.testing.assert_array_equal(g.getData("cice"), k.getDG0Data("cice"))
    if rheology == "bbm":
        np.testing.assert_array_equal(g.getData("damage"), k.getDG0Data("damage"))
    g.update(600.0)
    g.exchange(k, 1)
    c = g.getData("cice_updated")
    np.testing.assert_array_equal(k.getDG0Data("hice"), g.getData("hice_updated") * c)
    np.testing.assert_array_equal(k.getDG0Data("cice"), c)
    assert np.all(k.getDGData("hice", ncomp=6)[:, 1:] == 0.0)
    # the host round trip (setData with one-component arrays) gives the same state
    k2 = cls(dg_comp=6, n_steps=10)
    k2.initialise(box.coords(), False, box.mask())
    k2.restore(k.snapshot())
    k2.setData("hice", g.getData("hice_updated") * c)
    k2.setData("cice", c)
    np.testing.assert_array_equal(k2.getDGData("hice", ncomp=6), k.getDGData("hice", ncomp=6))
    k.update(120.0, 120.0)  # the dynamics steps on from the exchanged state
    assert np.all(np.isfinite(k.getDG0Data("u")))


def test_ice_growth_argument_errors(gpu):
    from nextsimdg_gb300.ice_growth import IceGrowth
    g = IceGrowth(8)
    with pytest.raises(NsdgError) as e:
        g.setData("nonsense", np.zeros(8))
    assert e.value.status == NSDG_ERR_UNKNOWN_FIELD
    with pytest.raises(NsdgError) as e:
        g._check(g._l.nsdg_ice_growth_set_field(g._h, b"qia", np.zeros(4).ctypes.data, 4))
    assert e.value.status == NSDG_ERR_SIZE_MISMATCH
    for dt in (0.0, -1.0, float("nan")):
        with pytest.raises(NsdgError) as e:
            g.update(dt)
        assert e.value.status == NSDG_ERR_BAD_ARG
