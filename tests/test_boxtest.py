"""The synthetic box-test generator (inputs shared by the GPU kernel and the oracle)."""
import math

import numpy as np

from nextsimdg_gb300.boxtest import BoxTest


def test_shapes_and_mask():
    b = BoxTest(16)
    assert b.coords().shape == (17 * 17, 2)
    m = b.mask()
    assert m.shape == (16, 16) and m[0].sum() == 0 and m[:, -1].sum() == 0 and m[1:-1, 1:-1].all()
    assert b.coords()[-1].tolist() == [512e3, 512e3]
    for name, a in b.initial_fields().items():
        assert a.shape == (256,), name


def test_thickness_and_ocean_formulas():
    b = BoxTest(64)
    h = b.hice().reshape(64, 64)
    dx = 512e3 / 64
    assert h[0, 3] == 0.3 + 0.005 * (math.sin(6e-5 * 3 * dx) + math.sin(0.0))
    u, v = b.ocean()
    assert np.isclose(u.reshape(64, 64)[0, 0], -0.1) and np.isclose(v.reshape(64, 64)[0, 0], 0.1)


def test_cyclone_maximum_wind_and_motion():
    b = BoxTest(512)
    u, v = b.wind(0.0)
    s = np.hypot(u, v)
    assert abs(s.max() - 15.0) < 0.01
    # maximum at ~100 km from the centre
    x = (np.arange(512) * b.dx)[None, :].repeat(512, 0).ravel()
    y = (np.arange(512) * b.dy)[:, None].repeat(512, 1).ravel()
    r = np.hypot(x - 256e3, y - 256e3)
    assert abs(r[np.argmax(s)] - 100e3) < 2 * b.dx
    # after one hour the centre moved 36 km along the diagonal
    u1, v1 = b.wind(3600.0)
    assert not np.allclose(u, u1)


def test_seeded_perturbations():
    a, b = BoxTest(8, seed=3, h_noise=0.02), BoxTest(8, seed=3, h_noise=0.02)
    np.testing.assert_array_equal(a.hice(), b.hice())
    assert not np.array_equal(a.hice(), BoxTest(8, seed=4, h_noise=0.02).hice())
    assert np.array_equal(BoxTest(8).hice(), BoxTest(8, seed=0).hice())
