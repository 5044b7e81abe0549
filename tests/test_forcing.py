"""The benchmark forcing restated in numpy (oracle.pyoracle) against the
box-test generator that feeds every other test, on the CPU: with the box
test's constants the reference's formulas (BenchmarkAtmosphere.cpp:29-77,
BenchmarkOcean.cpp:15-39) give the same fields."""
import numpy as np

from nextsimdg_gb300 import _lib
from nextsimdg_gb300.boxtest import BoxTest


def test_reference_defaults(oracle):
    f = _lib.benchmark_forcing(512e3, 512e3)
    assert (f.wind_A, f.wind_vmax, f.wind_k, f.wind_angle_deg, f.ocean_vmax) == (1e-5, 30.0, 1e-5, 72.0, 0.01)
    assert (f.centre_x, f.centre_y) == (256e3, 256e3)
    # the centre reaches the far corner after 5 days (BenchmarkAtmosphere.cpp:41-58)
    assert abs(f.centre_x + f.centre_vx * 5 * 86400.0 - 512e3) < 1e-6
    uw, vw, uo, vo = oracle.benchmark_forcing_fields(64, 64, f, 0.0)
    # cyclone: |wind| = A vmax r exp(-k r), largest (30/e m/s) at r = 1/k
    assert abs(np.hypot(uw, vw).max() - 30.0 / np.e) < 0.05
    assert np.isclose(uo.max(), 0.01 * (2 * 63 / 64 - 1)) and np.isclose(vo.max(), 0.01)


def test_box_test_constants_give_the_box_test_fields(oracle):
    for box in (BoxTest(48), BoxTest(40, seed=3, start=(230e3, 280e3), wind_speed=9.0)):
        f = box.device_forcing()
        for step in (0, 7, 100):
            t = step * box.dt
            uw, vw, uo, vo = oracle.benchmark_forcing_fields(box.nx, box.ny, f, t)
            bw, bv = box.wind(t)
            bo, bp = box.ocean()
            scale = np.abs(bw).max()
            assert np.abs(uw - bw).max() <= 1e-13 * scale and np.abs(vw - bv).max() <= 1e-13 * scale
            assert np.abs(uo - bo).max() <= 1e-15 and np.abs(vo - bp).max() <= 1e-15
