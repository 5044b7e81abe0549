"""GPU DG transport (kTransportStage, kNormalVelocity) through the C ABI.

1. The reference's golden values (Advection_test.cpp, AdvectionPeriodicBC_test.cpp)
   reproduced on the GPU, tolerance 1e-7 as in the reference tests.
2. Bitwise-close parity with the CPU oracle on random data, land masks and
   all DG orders / RK schemes (FP64: relative 1e-12 of the field scale).
"""
import numpy as np
import pytest

from nextsimdg_gb300.dynamics import DGTransport

pytestmark = pytest.mark.gpu


def _run_golden(oracle, dg, verts, dirichlet, periodic, nx, ny, fn_phi, fn_vx, fn_vy, param, dt, NT,
                limit=False):
    o = oracle.OracleTransport(dg, nx, ny, verts, dirichlet, periodic)
    phi = o.function2dg(fn_phi, param)
    if limit:  # LimitMax(phi, 1.0) after the initial projection
        phi = o.limit(phi, limit_max=1.0)
    vx, vy = o.function2dg(fn_vx, param), o.function2dg(fn_vy, param)
    t = DGTransport(dg, nx, ny, verts, dirichlet, periodic, scheme="rk2" if dg < 3 else "rk3")
    t.setVelocity(vx, vy)
    t.reinitnormalvelocity()
    if limit:
        out = t.step(dt, phi, NT, limit_max=1.0, limit_min=0.0)
    else:
        out = t.step(dt, phi, NT)
    # the reference's mass check (Tools::MeanValue) on the GPU, FP64
    m_gpu, m_cpu = t.meanValue(out), o.meanValue(out)
    assert m_gpu == pytest.approx(m_cpu, rel=1e-12)
    return np.sqrt(o.l2error(fn_phi, param, out)), out


@pytest.mark.parametrize("dg,it", [(dg, it) for dg in (1, 3, 6) for it in (0, 1)])
@pytest.mark.parametrize("key,distort", [("advection_regular", 0.0), ("advection_distorted", 0.05)])
def test_gpu_advection_goldens(gpu, oracle, goldens, key, distort, dg, it):
    Lx, Ly = 409600.0, 512000.0
    nx, ny = 12 << it, 13 << it
    deg = {1: 0, 3: 1, 6: 2}[dg]
    NT = 100 * (deg + 1) ** 2 * (1 << it)
    verts, dirichlet, periodic = oracle.rectangle_mesh(Lx, Ly, nx, ny, distort)
    err, _ = _run_golden(oracle, dg, verts, dirichlet, periodic, nx, ny, oracle.SMOOTH_BUMP, oracle.ROT_VX,
                         oracle.ROT_VY, Lx, Lx / NT, NT)
    assert err / Lx == pytest.approx(goldens[key][str(dg)][it], rel=goldens["tolerance"])


@pytest.mark.parametrize("dg,it", [(dg, it) for dg in (1, 3, 6) for it in (0, 1)])
def test_gpu_periodic_goldens(gpu, oracle, goldens, dg, it):
    R0, R1 = 100000.0, 250000.0
    nx, ny = 32 << it, 4 << it
    deg = {1: 0, 3: 1, 6: 2}[dg]
    NT = 50 * (deg + 1) ** 2 * (1 << it)
    verts, dirichlet, periodic = oracle.ring_mesh(R0, R1, nx, ny)
    err, _ = _run_golden(oracle, dg, verts, dirichlet, periodic, nx, ny, oracle.PACKMAN, oracle.RING_VX,
                         oracle.RING_VY, R1, R1 / NT, NT, limit=True)
    assert err / R0 == pytest.approx(goldens["periodic"][str(dg)][it], rel=goldens["tolerance"])


@pytest.mark.parametrize("dg,scheme", [(1, "rk2"), (3, "rk1"), (3, "rk3"), (6, "rk2"), (6, "rk3"), (8, "rk2")])
def test_gpu_transport_matches_oracle_random(gpu, oracle, dg, scheme):
    rng = np.random.default_rng(dg * 10 + len(scheme))
    nx, ny = 19, 14
    verts, dirichlet, _ = oracle.rectangle_mesh(3e5, 2.5e5, nx, ny, 0.04)
    land = np.ones(nx * ny, dtype=np.uint8)
    land[rng.choice(nx * ny, 20, replace=False)] = 0  # land holes: edges next to them are skipped
    phi = rng.standard_normal((nx * ny, dg))
    vx, vy = 0.3 * rng.standard_normal((nx * ny, dg)), 0.3 * rng.standard_normal((nx * ny, dg))
    o = oracle.OracleTransport(dg, nx, ny, verts, dirichlet, [], landmask=land, scheme=scheme)
    t = DGTransport(dg, nx, ny, verts, dirichlet, [], landmask=land, scheme=scheme)
    for tr in (o, t):
        tr.setVelocity(vx, vy)
        tr.reinitnormalvelocity()
    lim = dict(limit_max=1.5, limit_min=-1.5) if dg in (1, 3, 6) else {}
    a = o.step(2000.0, phi, 5, **lim)
    b = t.step(2000.0, phi, 5, **lim)
    scale = np.abs(a).max()
    assert np.abs(a - b).max() <= 1e-12 * scale
