"""The CPU oracle against the reference's own golden values.

Advection_test.cpp:274-301 and AdvectionPeriodicBC_test.cpp:281-290 check
the L2 error after transporting a bump (resp. a ring profile) for DG 1/3/6 at
two resolutions, with relative tolerance 1e-7.  Matching them pins the
oracle's transport, limiters, Function2DG, L2ErrorFunctionDG, mesh geometry
and basis tables.
"""
import ctypes

import pytest

CASES = [(dg, it) for dg in (1, 3, 6) for it in (0, 1)]


@pytest.mark.parametrize("dg,it", CASES)
@pytest.mark.parametrize("key,distort", [("advection_regular", 0.0), ("advection_distorted", 0.05)])
def test_advection_goldens(oracle, goldens, key, distort, dg, it):
    ml = ctypes.c_double()
    err = oracle.load().oracle_advection_golden(dg, distort, it, ctypes.byref(ml))
    ref = goldens[key][str(dg)][it]
    assert err == pytest.approx(ref, rel=goldens["tolerance"])


@pytest.mark.parametrize("dg,it", CASES)
def test_periodic_goldens(oracle, goldens, dg, it):
    ml = ctypes.c_double()
    err = oracle.load().oracle_periodic_golden(dg, it, ctypes.byref(ml))
    assert err == pytest.approx(goldens["periodic"][str(dg)][it], rel=goldens["tolerance"])
