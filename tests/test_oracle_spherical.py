"""The oracle's spherical geometry (rotation of the poles, longitude
continuity, cos(lat) area weight) against the exact spherical area.

The kernel rotates the (lon, lat) mesh so that its poles sit in Greenland /
Antarctica; a rotation preserves areas, so the integral of a constant field
over a lon/lat rectangle (Tools::MeanValue with cos(lat) weights, in
radians^2) must approach the rectangle's area on the unit sphere,
(lon1 - lon0)(sin lat1 - sin lat0), to the second order of the bilinear
elements."""
import numpy as np


def _mean_value(oracle, nx, ny, lon, lat, dg=6):
    lo = np.linspace(lon[0], lon[1], nx + 1)
    la = np.linspace(lat[0], lat[1], ny + 1)
    X, Y = np.meshgrid(lo, la)
    coords = np.stack([X.ravel(), Y.ravel()], 1)
    k = oracle.OracleKernel(0, dg, n_steps=10)
    k.initialise(coords, True, np.ones((ny, nx)))
    k.setData("hice", np.ones(nx * ny))
    return k.meanValue("hice")


def test_spherical_area_of_a_rectangle(oracle):
    lon, lat = (-0.4, 0.5), (0.9, 1.25)
    exact = (lon[1] - lon[0]) * (np.sin(lat[1]) - np.sin(lat[0]))
    e1 = abs(_mean_value(oracle, 12, 10, lon, lat) - exact) / exact
    e2 = abs(_mean_value(oracle, 24, 20, lon, lat) - exact) / exact
    assert e1 < 1e-3, e1
    assert e2 < 0.35 * e1, (e1, e2)  # second order in the element size


def test_spherical_area_across_the_dateline(oracle):
    """A rectangle straddling lon = +-pi (coordinates jump from +pi to -pi)
    keeps its area: the longitudes of each element are made continuous."""
    nx, ny = 16, 10
    lo = np.linspace(np.pi - 0.3, np.pi + 0.3, nx + 1)
    lo = np.where(lo > np.pi, lo - 2 * np.pi, lo)
    la = np.linspace(-0.2, 0.2, ny + 1)
    X, Y = np.meshgrid(lo, la)
    coords = np.stack([X.ravel(), Y.ravel()], 1)
    k = oracle.OracleKernel(0, 3, n_steps=10)
    k.initialise(coords, True, np.ones((ny, nx)))
    k.setData("hice", np.ones(nx * ny))
    exact = 0.6 * (np.sin(0.2) - np.sin(-0.2))
    assert abs(k.meanValue("hice") - exact) / exact < 1e-3
