"""The column-thermodynamics oracle (oracle/ice_growth_oracle.cpp) against the
reference's own known-answer tests of IceGrowth, ThermoIce0, ThermoWinton and
ConstantHealing (physics/test/IceGrowth_test.cpp, ThermoIce0_test.cpp,
ThermoWintonTemperature_test.cpp, DamageHealing_test.cpp), with doctest's
Approx semantics:
|a - b| < eps (1 + max(|a|, |b|)).

The inputs are those the tests set through their boundary modules:
UniformOcean(sst, sss, mld) gives tf = UnescoFreezing(sss) and the mixed
layer bulk heat capacity rho_w cp_w mld (UniformOcean.cpp:17-23); the
penetrating short wave is zero.  Not pinned: ThermoIce0Temperature_test.cpp
(not built by the reference: it uses a retired array-store API, and its
expected conductive flux predates the factor gamma = 1.065) and the
"Zero thickness" case (it installs a test-only thermodynamics module); the
complete-melt case below drives the same IceGrowth branches with ThermoIce0.
"""
import pytest

from oracle import pyoracle as po

RHO_CP_WATER = 1000.0 * 4186.84  # Water::rho * Water::cp (constants.hpp:102,114)


def approx(a, b, eps=1e-5):
    return abs(a - b) < eps * (1.0 + max(abs(a), abs(b)))


def _run(cice, hice, hsnow, tice0, qia, dqia, qow, subl, snow, ocean, qio, dt, **params):
    sst, sss, mld = ocean
    g = po.OracleIceGrowth(1, **params)
    for k, v in dict(cice=cice, hice=hice, hsnow=hsnow, tice=tice0, qia=qia, dqia_dt=dqia, qow=qow, sublim=subl,
                     snowfall=snow, penSW=0.0, sst=sst, tf=po.unesco_freezing(sss), mlbhc=RHO_CP_WATER * mld,
                     qio=qio, damage=1.0).items():
        g.setData(k, v)
    g.update(dt)
    c = g.getData("cice_updated")[0]
    return dict(cice=c, hc=g.getData("hice_updated")[0] * c, sc=g.getData("hsnow_updated")[0] * c,
                newice=g.getData("newice")[0], g=g)


def test_unesco_freezing_point():
    # Fofonoff and Millard (1983) at 32 PSU, zero pressure:
    # 32 (-0.0575 + 1.710523e-3 sqrt(32) - 2.154996e-4 32)
    assert approx(po.unesco_freezing(32.0), -1.7510339, 1e-7)
    assert po.unesco_freezing(0.0) == 0.0


def test_new_ice_formation():
    """IceGrowth_test.cpp:30-110 (one day)."""
    r = _run(0.5, 0.1, 0.0, -2.0, 305.288, 4.5036, 307.546, 0.0, 0.0, (-1.5, 32.0, 10.25), 124.689, 86400.0)
    assert approx(r["newice"], 0.0258264)


def test_melting_conditions():
    """IceGrowth_test.cpp:112-203 (600 s)."""
    r = _run(0.5, 0.1, 0.01, -1.0, -84.5952, 19.7016, -109.923, -7.3858e-06, 0.0, (-1.0, 32.0, 10.25), 53717.8,
             600.0)
    assert approx(r["cice"], 0.368269)
    assert approx(r["hc"], 0.0473078)
    assert approx(r["sc"], 0.00720977)
    assert r["newice"] == 0.0


def test_freezing_conditions():
    """IceGrowth_test.cpp:205-296 (600 s, snowfall)."""
    r = _run(0.5, 0.1, 0.01, -9.0, 42.2955, 16.7615, 143.266, 2.15132e-6, 1e-3, (-1.75, 32.0, 10.25), 73.9465,
             600.0)
    assert approx(r["cice"], 0.5002)
    assert approx(r["hc"], 0.100039)
    assert approx(r["sc"], 0.0109012)
    assert approx(r["newice"], 6.79906e-5)


def test_dummy_modules_keep_the_ice():
    """IceGrowth_test.cpp:298-399: DummyIceThermodynamics + DummyIceSpread."""
    r = _run(0.5, 0.1, 0.01, -5.0, 0.0, 0.0, 0.0, 0.0, 0.0, (-1.0, 35.0, 10.0), 0.0, 600.0,
             thermo_model=1, lateral_model=1)
    assert r["cice"] == 0.5 and r["hc"] == 0.1 and r["sc"] == 0.01 and r["newice"] == 0.0


def test_thermo_switched_off():
    """IceGrowth_test.cpp:502-617: nextsim_thermo.use_thermo_forcing = false."""
    r = _run(0.5, 0.1, 0.01, -9.0, 42.2955, 16.7615, 143.266, 2.15132e-6, 1e-3, (-1.75, 32.0, 10.25), 73.9465,
             600.0, use_thermo=0)
    assert r["cice"] == 0.5 and r["hc"] == 0.1 and r["sc"] == 0.01 and r["newice"] == 0.0


def test_threshold_ice_is_removed():
    """ThermoIce0_test.cpp:30-160: ThermoIce0 alone removes 1 mm of ice at
    99 % concentration (true thickness 0.001 / 0.99)."""
    sst = po.unesco_freezing(32.0)
    g = po.OracleIceGrowth(1)
    h = 0.001 / 0.99
    for k, v in dict(cice_updated=0.99, hice_updated=h, hice_initial=h, hsnow_updated=0.0, tice=-9.0, sst=sst,
                     tf=sst, mlbhc=4.29151e7).items():
        g.setData(k, v)
    g.thermo_only(600.0)
    assert g.getData("hice_updated")[0] == 0.0 and g.getData("cice_updated")[0] == 0.0


def test_removed_ice_refreezes_with_its_latent_heat():
    """The same ice through the whole IceGrowth::update: applyLimits removes
    it and returns its latent heat to the open-water flux, which (sea at the
    freezing point) refreezes exactly that volume as new ice spread at
    thickness h0 by HiblerSpread."""
    sst = po.unesco_freezing(32.0)
    g = po.OracleIceGrowth(1)
    for k, v in dict(cice=0.99, hice=0.001, hsnow=0.0, tice=-9.0, sst=sst, tf=sst, mlbhc=4.29151e7).items():
        g.setData(k, v)
    g.update(600.0)
    assert approx(g.getData("newice")[0], 0.001, 1e-12)
    assert approx(g.getData("hice_updated")[0], 0.25, 1e-12)
    assert approx(g.getData("cice_updated")[0], 0.004, 1e-12)


def test_complete_melt():
    """A day of the melting conditions: ThermoIce0 melts all the ice
    (the hice < h_min branch), so concentration and thickness are zero and no
    new ice forms (the outcome IceGrowth_test.cpp:401-500 checks)."""
    r = _run(0.5, 0.1, 0.01, -1.0, -84.5952, 19.7016, -109.923, -7.3858e-06, 0.0, (-1.0, 32.0, 10.25), 53717.8,
             86400.0)
    assert r["newice"] == 0.0 and r["hc"] == 0.0 and r["cice"] == 0.0
    assert r["g"].getData("tice_updated")[0] == 0.0


@pytest.mark.parametrize("cice,dci,damage,expect", [
    (0.6, 0.3, 0.0, 0.55), (0.6, 0.3, 0.5, 0.80), (0.5, 0.1, 0.5, 0.65), (1.0, 0.1, 1.0, 1.0), (0.5, -0.5, 0.5, 0.55)])
def test_constant_healing_new_ice(cice, dci, damage, expect):
    """DamageHealing_test.cpp:66-169 (t_d = 20 days, one day)."""
    d = po.constant_healing(damage, cice, dci, 86400.0, 20 * 86400.0)
    assert d <= 1.0 and approx(d, expect, 1e-8)


def test_constant_healing_time_scale():
    """DamageHealing_test.cpp:17-64: 0.5 -> 0.55, 0.99 -> 1 (capped)."""
    assert approx(po.constant_healing(0.5, 0.5, 0.0, 86400.0, 20 * 86400.0), 0.55, 1e-8)
    assert po.constant_healing(0.99, 0.5, 0.0, 86400.0, 20 * 86400.0) == 1.0


@pytest.mark.parametrize("case,expect", [
    ("melting", (0.0, -0.999261, -0.275)), ("freezing", (-10.5129, -9.00726, -8.20454))])
def test_thermo_winton_temperatures(case, expect):
    """ThermoWintonTemperature_test.cpp:32-233: ThermoWinton alone for 600 s on
    true thicknesses 0.2 m ice, 0.02 m snow; UniformOcean(sst, 32 PSU,
    4.29151e7 / (rho_w cp_w)); the three temperature levels."""
    t0, qio, qia, dqia, subl, pensw = {
        "melting": (-1.0, 53717.8, -85.6364, 19.7016, -7.3858e-06, 1.04125),
        "freezing": (-9.0, 73.9465, 42.2955, 16.7615, 2.15132e-6, 0.0)}[case]
    g = po.OracleIceGrowth(1, thermo_model=2)
    for k, v in dict(cice_updated=0.5, hice_updated=0.2, hice_initial=0.2, hsnow_updated=0.02, tice=t0, tice_1=t0,
                     tice_2=t0, tf=po.unesco_freezing(32.0), qio=qio, qia=qia, dqia_dt=dqia, sublim=subl,
                     penSW=pensw).items():
        g.setData(k, v)
    g.thermo_only(600.0)
    got = [g.getData(n)[0] for n in ("tice_updated", "tice_updated_1", "tice_updated_2")]
    assert all(approx(a, b) for a, b in zip(got, expect)), got


def test_thermo_winton_no_ice():
    """ThermoWintonTemperature_test.cpp:235-346: no ice stays no ice."""
    g = po.OracleIceGrowth(1, thermo_model=2)
    for k, v in dict(cice=0.0, hice=0.0, hsnow=0.0, tice=0.0, sst=1.75, tf=po.unesco_freezing(32.0),
                     mlbhc=4.29151e7, qow=143.266, qia=42.2955, dqia_dt=16.7615, sublim=2.15132e-6).items():
        g.setData(k, v)
    g.update(600.0)
    assert g.getData("hice_updated")[0] == 0.0 and g.getData("cice_updated")[0] == 0.0
