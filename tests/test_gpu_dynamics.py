"""The GPU dynamics kernel (mEVP and BBM) against the CPU oracle, through the C ABI.

Parity bar for the FP64 path: max |gpu - oracle| <= 1e-10 * max |oracle| for
thickness, concentration, damage (all DG components), velocity and ice-ocean
stress (DG0 read-out) after several full model steps of the box test.
"""
import numpy as np
import pytest

from nextsimdg_gb300.boxtest import BoxTest
from nextsimdg_gb300.dynamics import BBMDynamicsKernel, MEVPDynamicsKernel, NsdgError

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _make(cls_or_oracle, box, dg, rheology, **params):
    k = cls_or_oracle(dg_comp=dg, **params) if rheology is None else cls_or_oracle(rheology, dg, **params)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    return k


def _advance(k, box, steps, start=0):
    for s in range(start, start + steps):
        uw, vw = box.wind(s * box.dt)
        k.setData("uwind", uw)
        k.setData("vwind", vw)
        k.update(s * box.dt, box.dt)


def _rel(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def _compare(g, o, names, dg):
    worst = {}
    for n in names:
        if n in ("hice", "cice", "damage") and dg > 1:
            a, b = g.getDGData(n), o.getDGData(n)
        else:
            a, b = g.getDG0Data(n), o.getDG0Data(n)
        assert np.all(np.isfinite(a)), n
        worst[n] = _rel(a, b)
    return worst


MEVP_CASES = [(12, 6, 3), (17, 3, 3), (16, 1, 2), (32, 6, 4)]


@pytest.mark.parametrize("n,dg,steps", MEVP_CASES)
def test_mevp_matches_oracle(gpu, oracle, n, dg, steps):
    box = BoxTest(n, n + (1 if n == 17 else 0))
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, dg, None, **prm)
    o = _make(oracle.OracleKernel, box, dg, 0, **prm)
    _advance(g, box, steps)
    _advance(o, box, steps)
    worst = _compare(g, o, ["hice", "cice", "u", "v", "uiostress", "viostress"], dg)
    assert all(v <= TOL for v in worst.values()), worst
    assert np.abs(o.getDG0Data("u")).max() > 1e-3  # the test moves the ice


@pytest.mark.parametrize("nx,ny,mask_kind", [(2, 7, "ice"), (9, 2, "ice"), (2, 2, "ice"), (6, 5, "land"),
                                              (7, 6, "one cell"), (33, 3, "checker")])
def test_degenerate_grids_match_oracle(gpu, oracle, nx, ny, mask_kind):
    """Two-column and two-row grids, a 2 x 2 grid, an all-land mask, one ice
    cell in land and a checkerboard of ice and land (every ice cell's edges
    closed): FP64 within 1e-10 of the oracle after two steps, the mixed path
    (parallelogram kernels, tiled transport) finite and within 1e-5 m/s of
    it.  A single row or column is refused at initialise."""
    if nx == 2 and ny == 7:
        k = MEVPDynamicsKernel(dg_comp=6)
        with pytest.raises(NsdgError, match="nx >= 2"):
            k.initialise(BoxTest(1, 7).coords(), False, np.ones((7, 1)))
        k.close()
    box = BoxTest(nx, ny)
    if mask_kind != "ice":
        m = np.zeros((ny, nx))
        if mask_kind == "one cell":
            m[ny // 2, nx // 2] = 1.0
        elif mask_kind == "checker":
            m[(np.add.outer(np.arange(ny), np.arange(nx)) % 2) == 0] = 1.0
        box.mask = lambda m=m: m
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    g = _make(MEVPDynamicsKernel, box, 6, None, **prm)
    x = _make(MEVPDynamicsKernel, box, 6, None, precision=1, **prm)
    for k in (o, g, x):
        _advance(k, box, 2)
    names = ["hice", "cice", "u", "v", "uiostress", "viostress"]
    worst = _compare(g, o, names, 6)
    assert all(v <= TOL for v in worst.values()), worst
    for n in ("u", "v"):
        a, b = x.getDG0Data(n), o.getDG0Data(n)
        assert np.all(np.isfinite(a)) and float(np.sqrt(np.mean((a - b) ** 2))) <= 1e-5, n
    g.close()
    x.close()


def test_mevp_land_holes_matches_oracle(gpu, oracle):
    box = BoxTest(20, 15)
    m = box.mask()
    rng = np.random.default_rng(5)
    for _ in range(12):
        m[rng.integers(1, 14), rng.integers(1, 19)] = 0.0
    box.mask = lambda m=m: m
    prm = dict(alpha=1500.0, beta=1500.0, n_steps=60)
    g = _make(MEVPDynamicsKernel, box, 6, None, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    _advance(g, box, 3)
    _advance(o, box, 3)
    worst = _compare(g, o, ["hice", "cice", "u", "v"], 6)
    assert all(v <= TOL for v in worst.values()), worst


def test_bbm_matches_oracle(gpu, oracle):
    box = BoxTest(14)
    prm = dict(n_steps=50)
    g = _make(BBMDynamicsKernel, box, 6, None, **prm)
    o = _make(oracle.OracleKernel, box, 6, 1, **prm)
    for k in (g, o):
        k.setData("damage", box.damage())
    _advance(g, box, 3)
    _advance(o, box, 3)
    worst = _compare(g, o, ["hice", "cice", "damage", "u", "v", "uiostress"], 6)
    assert all(v <= TOL for v in worst.values()), worst


def test_full_size_matches_oracle(gpu, oracle):
    """256 x 256 DG2 box test (the benchmark grid), two full steps with the
    reference's default relaxation alpha = beta = 1500: FP64 parity 1e-10."""
    box = BoxTest(256)
    prm = dict(alpha=1500.0, beta=1500.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, 6, None, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    _advance(g, box, 2)
    _advance(o, box, 2)
    worst = _compare(g, o, ["hice", "cice", "u", "v"], 6)
    assert all(v <= TOL for v in worst.values()), worst


@pytest.mark.parametrize("dg,alpha,steps", [(3, 300.0, 30), (6, 300.0, 30), (6, 1500.0, 100)])
def test_long_horizon_matches_oracle(gpu, oracle, dg, alpha, steps):
    """64 x 64 box test over the longest horizons on which the oracle's own
    sensitivity to h x (1 + 1e-14) stays near 1e-13 (30 steps at alpha = 300:
    between steps 35 and 40 a clamp/limiter switch amplifies it to 4e-5;
    100 steps at alpha = 1500): FP64 parity 1e-10 for h, A (all DG
    components), u, v and the ice-ocean stress."""
    box = BoxTest(64)
    prm = dict(alpha=alpha, beta=alpha, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, dg, None, **prm)
    o = _make(oracle.OracleKernel, box, dg, 0, **prm)
    _advance(g, box, steps)
    _advance(o, box, steps)
    worst = _compare(g, o, ["hice", "cice", "u", "v", "uiostress", "viostress"], dg)
    assert all(v <= TOL for v in worst.values()), worst
    assert np.abs(o.getDG0Data("u")).max() > 1e-2


@pytest.mark.parametrize("dg", [3, 6])
def test_one_day_64_matches_oracle(gpu, oracle, dg):
    """The CPU-runnable box test for a full simulated day: 64 x 64 cells,
    DG1 (3 components) or DG2 transport, CG2 velocity, 100 mEVP iterations,
    alpha = beta = 300, 720 steps of 120 s, the oracle on the same inputs.
    The bar is 1e-10 relative where the oracle's own sensitivity (to h scaled
    by 1 + 1e-14) stays below 1e-11; otherwise 10x that sensitivity (over a
    day it is ~1e-4 for u: see test_long_horizon_matches_oracle)."""
    box = BoxTest(64)
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, dg, None, **prm)
    o = _make(oracle.OracleKernel, box, dg, 0, **prm)
    o2 = oracle.OracleKernel(0, dg, **prm)
    o2.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        o2.setData(name, arr * (1.0 + 1e-14) if name == "hice" else arr)
    for k in (g, o, o2):
        _advance(k, box, 720)
    worst = _compare(g, o, ["hice", "cice", "u", "v", "uiostress", "viostress"], dg)
    sens = max(_compare(o2, o, ["hice", "cice", "u", "v"], dg).values())
    bar = TOL if sens < 1e-11 else 10.0 * sens
    print(f"one day 64x64 DG{dg}: gpu vs oracle {worst}, oracle sensitivity {sens:.3e}, bar {bar:.1e}")
    assert all(v <= bar for v in worst.values()), (worst, sens)
    assert np.abs(o.getDG0Data("u")).max() > 1e-2


def test_full_size_alpha300_within_oracle_sensitivity(gpu, oracle):
    """With alpha = beta = 300 on 2 km cells the mEVP iteration amplifies
    rounding (alpha*beta is far below its stability bound), so no 1e-10 bar
    can hold between two correct FP64 implementations.  The GPU must then stay
    within the oracle's own sensitivity to a 1e-14 relative perturbation of h."""
    box = BoxTest(256)
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, 6, None, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    o2 = oracle.OracleKernel(0, 6, **prm)
    o2.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        o2.setData(name, arr * (1.0 + 1e-14) if name == "hice" else arr)
    for k in (g, o, o2):
        _advance(k, box, 2)
    ug, uo, up = g.getDG0Data("u"), o.getDG0Data("u"), o2.getDG0Data("u")
    sensitivity = _rel(up, uo)
    assert sensitivity > 1e-6  # the configuration is ill-conditioned
    assert _rel(ug, uo) <= 10.0 * sensitivity
    assert np.all(np.isfinite(ug))


def test_bitwise_reproducible(gpu):
    box = BoxTest(24)
    outs = []
    for _ in range(2):
        g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=50)
        _advance(g, box, 3)
        outs.append(np.concatenate([g.getDG0Data("u"), g.getDGData("hice").ravel()]))
        g.close()
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("cls,extra", [(MEVPDynamicsKernel, {}), (BBMDynamicsKernel, {"damage": True})])
def test_snapshot_resume_is_bitwise(gpu, cls, extra):
    box = BoxTest(16)
    a = _make(cls, box, 6, None, n_steps=30)
    if extra:
        a.setData("damage", box.damage())
    _advance(a, box, 4)
    ref = a.getDG0Data("u"), a.getDGData("hice")
    b = _make(cls, box, 6, None, n_steps=30)
    if extra:
        b.setData("damage", box.damage())
    _advance(b, box, 2)
    blob = b.snapshot()
    c = cls(dg_comp=6, n_steps=30)
    c.initialise(box.coords(), False, box.mask())
    c.restore(blob)
    _advance(c, box, 2, start=2)
    np.testing.assert_array_equal(c.getDG0Data("u"), ref[0])
    np.testing.assert_array_equal(c.getDGData("hice"), ref[1])


def test_mean_value_matches_oracle(gpu, oracle):
    box = BoxTest(20)
    g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=20)
    o = _make(oracle.OracleKernel, box, 6, 0, n_steps=20)
    _advance(g, box, 2)
    _advance(o, box, 2)
    assert g.meanValue("hice") == pytest.approx(o.meanValue("hice"), rel=1e-12)


def test_errors_surface_and_gpu_stays_usable(gpu):
    box = BoxTest(10)
    g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=10)
    with pytest.raises(KeyError):
        g.getDG0Data("no_such_field")
    with pytest.raises(NsdgError):
        g.setData("hice", np.ones(7))
    # a non-finite forcing is reported as a numeric fault, not a crash
    bad = np.full(box.nelements, np.nan)
    g.setData("uwind", bad)
    g.update(0.0, box.dt)
    with pytest.raises(NsdgError) as ei:
        g.getDG0Data("u")
    assert ei.value.status == 5
    # the same handle is re-initialised and runs normally afterwards
    g.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        g.setData(name, arr)
    _advance(g, box, 1)
    assert np.all(np.isfinite(g.getDG0Data("u")))
    with pytest.raises(NsdgError):
        g.initialise(box.coords() * np.nan, False, box.mask())  # non-finite coordinates


def test_other_fields_are_stored_not_advected(gpu):
    box = BoxTest(8)
    g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=5)
    tracer = np.arange(box.nelements, dtype=float)
    g.setData("tracer", tracer)
    _advance(g, box, 1)
    np.testing.assert_array_equal(g.getDG0Data("tracer"), tracer)
    np.testing.assert_array_equal(g.getDGData("tracer", ncomp=1), tracer)


@pytest.mark.parametrize("n,steps,dg,kernel", [(32, 5, 6, None), (64, 3, 6, None), (32, 5, 3, None),
                                               (32, 5, 1, None), (32, 5, 6, "tma"), (32, 5, 6, "global")])
def test_mixed_precision_close_to_oracle(gpu, oracle, n, steps, dg, kernel, monkeypatch):
    """FP32 bulk with FP64 Delta/viscosity, lumped-mass inverse and
    conservation sums: RMS error against the FP64 oracle, stated bars.  The
    box mesh takes the parallelogram stress kernel; NSDG_STRESS_KERNEL forces
    the operator-streaming ones."""
    if kernel:
        monkeypatch.setenv("NSDG_STRESS_KERNEL", kernel)
    box = BoxTest(n)
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, dg, None, precision=1, **prm)
    o = _make(oracle.OracleKernel, box, dg, 0, **prm)
    _advance(g, box, steps)
    _advance(o, box, steps)
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
    du = rms(g.getDG0Data("u"), o.getDG0Data("u"))
    dv = rms(g.getDG0Data("v"), o.getDG0Data("v"))
    dh = rms(g.getDG0Data("hice"), o.getDG0Data("hice"))
    da = rms(g.getDG0Data("cice"), o.getDG0Data("cice"))
    assert max(du, dv) <= 1e-5, (du, dv)       # m/s
    assert dh <= 1e-6 and da <= 1e-6, (dh, da)  # m, fraction
    assert np.abs(o.getDG0Data("u")).max() > 1e-3
    # the ice-ocean stress read-out (FP32 on this path): 5 % of its RMS, a
    # bar the velocity bar above implies (tau ~ |u - uo| (u - uo))
    for n in ("uiostress", "viostress"):
        ref = o.getDG0Data(n)
        assert rms(g.getDG0Data(n), ref) <= 0.05 * float(np.sqrt(np.mean(ref ** 2))), n
    assert g.stress_variant()[0] == (kernel or "affine")
    assert g.transport_variant()[0] == "tiled"


@pytest.mark.parametrize("nx,ny,dg,holes", [(45, 37, 6, True), (64, 64, 6, False), (33, 17, 3, True),
                                            (31, 9, 1, True), (8, 40, 6, False)])
def test_tiled_transport_matches_per_element_kernel(gpu, nx, ny, dg, holes, monkeypatch):
    """The parallelogram-mesh transport stage (tiles of 32 x 8 cells, each
    interior edge flux evaluated once into shared memory, the cell term from
    the Jacobian coefficients, diagonal M^{-1}) against the per-element
    kernel (NSDG_TRANSPORT_KERNEL=element) on grids that are not multiples
    of the tile, with land cells.  The first update starts from rest (no
    transport), so both handles reach the same velocity bit for bit; the
    second transports h and A by it, and they differ by rounding only (FP32
    fluxes; the diagonal M^{-1} also in the transport velocity's projection):
    1e-6 of their largest value; the velocity then follows within 1e-4."""
    box = BoxTest(nx, ny)
    if holes:
        m = box.mask()
        rng = np.random.default_rng(nx + ny)
        for _ in range(max(4, nx * ny // 60)):
            m[rng.integers(1, ny - 1), rng.integers(1, nx - 1)] = 0.0
        box.mask = lambda m=m: m
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    t = _make(MEVPDynamicsKernel, box, dg, None, precision=1, **prm)
    monkeypatch.setenv("NSDG_TRANSPORT_KERNEL", "element")
    e = _make(MEVPDynamicsKernel, box, dg, None, precision=1, **prm)
    monkeypatch.delenv("NSDG_TRANSPORT_KERNEL")
    kind, cell_mismatch, offdiag = t.transport_variant()
    assert kind == "tiled" and 0 <= cell_mismatch <= 1e-9 and 0 <= offdiag <= 1e-12, t.transport_variant()
    assert e.transport_variant()[0] == "element"
    _advance(t, box, 1)
    _advance(e, box, 1)
    np.testing.assert_array_equal(t.getDG0Data("u"), e.getDG0Data("u"))
    h1 = t.getDGData("hice")
    _advance(t, box, 1, start=1)
    _advance(e, box, 1, start=1)
    for n in ("hice", "cice"):
        a, b = t.getDGData(n), e.getDGData(n)
        assert np.all(np.isfinite(a)), n
        assert _rel(a, b) <= 1e-6, (n, _rel(a, b))
    for n in ("u", "v"):
        assert _rel(t.getDG0Data(n), e.getDG0Data(n)) <= 1e-4, n
    # the transport moved something: the thickness changed
    assert _rel(t.getDGData("hice"), h1) > 1e-9


def test_mixed_precision_distorted_mesh_close_to_oracle(gpu, oracle):
    """A mesh of general quadrilaterals (interior vertices moved by up to 8 %
    of a cell) is not a parallelogram mesh: the mixed path streams the
    element operators (TMA or global kernel, chosen by timing); stated bars
    against the FP64 oracle."""
    box = BoxTest(40, 36)
    c = box.coords().copy()
    rng = np.random.default_rng(11)
    ix = np.tile(np.arange(41), 37)
    iy = np.repeat(np.arange(37), 41)
    inner = (ix > 0) & (ix < 40) & (iy > 0) & (iy < 36)
    c[inner] += rng.uniform(-0.08, 0.08, (inner.sum(), 2)) * (box.L / 40)
    box.coords = lambda c=c: c
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, 6, None, precision=1, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    kind, mismatch = g.stress_variant()
    assert kind in ("tma", "global") and mismatch > 1e-3, (kind, mismatch)
    # not a parallelogram mesh: the transport checks are not even evaluated
    assert g.transport_variant() == ("element", -1.0, -1.0)
    _advance(g, box, 4)
    _advance(o, box, 4)
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
    err = {f: rms(g.getDG0Data(f), o.getDG0Data(f)) for f in ("u", "v", "hice", "cice")}
    print(f"distorted 40x36 mixed ({kind}): RMS vs oracle {err}")
    assert max(err["u"], err["v"]) <= 1e-5, err
    assert err["hice"] <= 1e-6 and err["cice"] <= 1e-6, err
    assert np.abs(o.getDG0Data("u")).max() > 1e-3


def test_parallelogram_kernel_on_a_sheared_mesh(gpu, oracle):
    """A sheared (non-rectangular) parallelogram mesh takes the coefficient
    kernel and stays within the mixed-precision bars of the FP64 oracle."""
    box = BoxTest(36, 30)
    c = box.coords().copy()
    c[:, 0] += 0.3 * c[:, 1]
    c[:, 1] -= 0.1 * c[:, 0]
    box.coords = lambda c=c: c
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, 6, None, precision=1, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    kind, mismatch = g.stress_variant()
    assert kind == "affine" and 0 <= mismatch < 1e-12, (kind, mismatch)
    _advance(g, box, 4)
    _advance(o, box, 4)
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
    err = {f: rms(g.getDG0Data(f), o.getDG0Data(f)) for f in ("u", "v", "hice", "cice")}
    print(f"sheared 36x30 mixed (affine): RMS vs oracle {err}")
    assert max(err["u"], err["v"]) <= 1e-5, err
    assert err["hice"] <= 1e-6 and err["cice"] <= 1e-6, err
    assert np.abs(o.getDG0Data("u")).max() > 1e-3


def test_fp64_viscosity_forms_agree(gpu):
    """P/(8 alpha Delta) by CUDA's rsqrt(double) and by the Newton-Raphson
    forms (FP32 seed, one FP64 step; conversions by the FP64 unit or on the
    integer pipe): within one FP32 ulp, equal in almost every case, over
    strain invariants from 0 (and denormals) to 1e-4 s^-2."""
    from nextsimdg_gb300.dynamics import selftest_viscosity
    rng = np.random.default_rng(2)
    n = 1 << 18
    inv = np.concatenate([[0.0, 1e-45, 1e-40, 1.1754942e-38, 1.1754944e-38],
                          10.0 ** rng.uniform(-36, -4, n - 5)]).astype(np.float32)
    pa = np.concatenate([[0.0, 1e-300, 5.0, 12.5, 1e3], 10.0 ** rng.uniform(-3, 4, n - 5)])
    pa[rng.integers(5, n, 100)] = 0.0
    out = selftest_viscosity(inv, pa, 2e-9)
    ref = out[0].astype(np.float64)
    for k in (1, 2):
        d = np.abs(out[k].astype(np.float64) - ref)
        ulp = np.spacing(np.abs(out[0])).astype(np.float64)
        assert np.all(d <= ulp), (k, np.max(d / np.maximum(ulp, 1e-45)))
        assert np.mean(d == 0) > 0.99, (k, np.mean(d == 0))
    assert np.all(out[:, pa == 0.0] == 0.0)
    assert np.all(np.isfinite(out))


def test_checked_float_pair_viscosity_is_form_2(gpu):
    """Form 4 (float pairs checked against form 2's rounding, form 2 where
    the check fails) is bitwise form 2 on the device: random strain
    invariants and pressure terms, and pressure terms aimed at float
    rounding midpoints of the result (where form 3 alone may differ)."""
    from nextsimdg_gb300.dynamics import selftest_viscosity, selftest_viscosity_checked
    rng = np.random.default_rng(11)
    n = 1 << 18
    inv = np.concatenate([[0.0, 1e-45, 1e-40, 1.1754942e-38, 4e-18],
                          10.0 ** rng.uniform(-36, -4, n - 5)]).astype(np.float32)
    pa = np.concatenate([[0.0, 1e-300, 1e-31, 12.5, 1e3], 10.0 ** rng.uniform(-3, 4, n - 5)])
    # aimed: Pa = midpoint / (1 / sqrt(inv + DeltaMin^2)) in extended
    # precision, so that the result lies within about 2^-43 of a midpoint
    m = n // 2
    dmin = 2e-9
    t = inv[:m].astype(np.longdouble) + np.longdouble(dmin) * np.longdouble(dmin)
    z0 = (10.0 ** rng.uniform(-2, 3, m)).astype(np.float32)
    mid = (z0.astype(np.longdouble) + np.nextafter(z0, np.float32(np.inf)).astype(np.longdouble)) / 2
    pa[:m] = (mid * np.sqrt(t)).astype(np.float64)
    f2 = selftest_viscosity(inv, pa, dmin)[2]
    f4 = selftest_viscosity_checked(inv, pa, dmin)
    assert np.array_equal(f4.view(np.uint32), f2.view(np.uint32)), int(np.sum(f4 != f2))


def test_checked_float_pair_viscosity_steps_like_form_2(gpu, monkeypatch):
    """The parallelogram stress kernel with form 4 (NSDG_VISC_FORM=4) and
    with form 2: the same model steps, bitwise."""
    from nextsimdg_gb300.boxtest import step_forcing
    box = BoxTest(96)
    out = {}
    for form in ("2", "4"):
        monkeypatch.setenv("NSDG_VISC_FORM", form)
        k = MEVPDynamicsKernel(dg_comp=6, alpha=300.0, beta=300.0, n_steps=100, precision=1)
        k.initialise(box.coords(), False, box.mask())
        for name, arr in box.initial_fields().items():
            k.setData(name, arr)
        for s in range(4):
            step_forcing(k, box, s)
            k.update(s * box.dt, box.dt)
        out[form] = {f: k.getDG0Data(f) for f in ("u", "v", "hice", "cice", "uiostress")}
        assert k.stress_variant()[0] == "affine"
        k.close()
    for f in out["2"]:
        assert np.array_equal(out["2"][f], out["4"][f]), f
    assert np.abs(out["4"]["u"]).max() > 1e-3


@pytest.mark.parametrize("n,steps", [(14, 3), (48, 3)])
def test_bbm_mixed_precision_close_to_oracle(gpu, oracle, n, steps):
    """BBM in the mixed mode (FP32 stress/damage arithmetic and transport
    fluxes, FP64 fields, inverse mass matrices and momentum): RMS error
    against the FP64 oracle, stated bars."""
    box = BoxTest(n)
    prm = dict(n_steps=50)
    g = _make(BBMDynamicsKernel, box, 6, None, precision=1, **prm)
    o = _make(oracle.OracleKernel, box, 6, 1, **prm)
    for k in (g, o):
        k.setData("damage", box.damage())
    _advance(g, box, steps)
    _advance(o, box, steps)
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
    err = {f: rms(g.getDG0Data(f), o.getDG0Data(f)) for f in ("u", "v", "hice", "cice", "damage")}
    print(f"BBM mixed {n}x{n}, {steps} steps: RMS vs oracle {err}")
    assert max(err["u"], err["v"]) <= 1e-5, err           # m/s
    assert err["hice"] <= 1e-6 and err["cice"] <= 1e-6, err
    assert err["damage"] <= 1e-5, err
    assert np.abs(o.getDG0Data("u")).max() > 1e-3
    kind, mismatch = g.stress_variant()  # the box takes the parallelogram BBM kernel
    assert kind == "affine" and 0 <= mismatch <= 1e-9, (kind, mismatch)


def test_bbm_parallelogram_kernel_matches_per_element_operators(gpu, monkeypatch):
    """The mixed BBM stress kernel on a parallelogram mesh (5 coefficients
    per element, the unit square's strain, projection and divergence
    operators in constant memory) against the same kernel streaming each
    element's FP32 operators (NSDG_BBM_STRESS_KERNEL=general), on a sheared
    grid with land holes: FP32 rounding of the operators only (velocity
    1e-6 m/s, damage 1e-6 RMS after three steps)."""
    box = BoxTest(33, 20)
    c = box.coords().copy()
    c[:, 0] += 0.3 * c[:, 1]  # sheared: still parallelograms
    box.coords = lambda c=c: c
    m = box.mask()
    m[5, 7] = m[12, 20] = m[3, 30] = 0.0
    box.mask = lambda m=m: m
    prm = dict(n_steps=50)
    a = _make(BBMDynamicsKernel, box, 6, None, precision=1, **prm)
    monkeypatch.setenv("NSDG_BBM_STRESS_KERNEL", "general")
    b = _make(BBMDynamicsKernel, box, 6, None, precision=1, **prm)
    monkeypatch.delenv("NSDG_BBM_STRESS_KERNEL")
    assert a.stress_variant()[0] == "affine" and b.stress_variant()[0] == "global"
    for k in (a, b):
        k.setData("damage", box.damage())
    _advance(a, box, 3)
    _advance(b, box, 3)
    rms = lambda x, y: float(np.sqrt(np.mean((x - y) ** 2)))  # noqa: E731
    for f, bar in (("u", 1e-6), ("v", 1e-6), ("hice", 1e-7), ("cice", 1e-7), ("damage", 1e-6)):
        assert rms(a.getDG0Data(f), b.getDG0Data(f)) <= bar, f
    assert np.abs(b.getDG0Data("u")).max() > 1e-4
    a.close()
    b.close()


def test_mixed_precision_snapshot_and_reproducible(gpu):
    box = BoxTest(16)
    a = _make(MEVPDynamicsKernel, box, 6, None, precision=1, n_steps=30)
    _advance(a, box, 2)
    blob = a.snapshot()
    _advance(a, box, 2, start=2)
    b = MEVPDynamicsKernel(dg_comp=6, precision=1, n_steps=30)
    b.initialise(box.coords(), False, box.mask())
    b.restore(blob)
    _advance(b, box, 2, start=2)
    np.testing.assert_array_equal(a.getDG0Data("u"), b.getDG0Data("u"))


# ---------------------------------------------------------------------------
# Spherical coordinates (x = lon, y = lat in radians; the poles are moved to
# Greenland / Antarctica by the kernel, as DynamicsKernel::initialise does)
# ---------------------------------------------------------------------------
def _sphere_case(nx=20, ny=16, lon=(-0.3, 0.3), lat=(1.0, 1.3), seed=3):
    lo = np.linspace(lon[0], lon[1], nx + 1)
    la = np.linspace(lat[0], lat[1], ny + 1)
    X, Y = np.meshgrid(lo, la)
    coords = np.stack([X.ravel(), Y.ravel()], 1)
    mask = np.ones((ny, nx))
    mask[0, :] = mask[-1, :] = 0
    mask[:, 0] = mask[:, -1] = 0
    rng = np.random.default_rng(seed)
    N = nx * ny
    cx = 0.5 * (lo[:-1] + lo[1:])
    cy = 0.5 * (la[:-1] + la[1:])
    CX, CY = np.meshgrid(cx, cy)
    fields = {
        "hice": (0.3 + 0.05 * np.sin(9 * CX) * np.cos(7 * CY)).ravel() + 0.01 * rng.standard_normal(N),
        "cice": np.full(N, 0.95), "u": np.zeros(N), "v": np.zeros(N),
        "uocean": 0.05 * np.cos(5 * CY).ravel(), "vocean": np.zeros(N),
        "ssh": np.zeros(N),
    }
    wind = lambda s: (12.0 * np.cos(4 * CY + 0.01 * s).ravel(), 6.0 * np.sin(3 * CX - 0.02 * s).ravel())  # noqa: E731
    return coords, mask, fields, wind


def _sphere_make(k, case, damage=False):
    coords, mask, fields, _ = case
    k.initialise(coords, True, mask)
    for name, arr in fields.items():
        k.setData(name, arr)
    if damage:
        k.setData("damage", np.ones(mask.size))
    return k


def _sphere_advance(k, case, steps):
    wind = case[3]
    for s in range(steps):
        uw, vw = wind(s)
        k.setData("uwind", uw)
        k.setData("vwind", vw)
        k.update(s * 120.0, 120.0)


@pytest.mark.parametrize("dg", [3, 6])
def test_spherical_mevp_matches_oracle(gpu, oracle, dg):
    case = _sphere_case()
    prm = dict(alpha=1500.0, beta=1500.0, n_steps=100)
    g = _sphere_make(MEVPDynamicsKernel(dg_comp=dg, **prm), case)
    o = _sphere_make(oracle.OracleKernel(0, dg, **prm), case)
    _sphere_advance(g, case, 3)
    _sphere_advance(o, case, 3)
    worst = _compare(g, o, ["hice", "cice", "u", "v", "uiostress", "viostress"], dg)
    assert all(v <= TOL for v in worst.values()), worst
    assert np.abs(o.getDG0Data("u")).max() > 1e-3
    assert abs(g.meanValue("hice") - o.meanValue("hice")) <= 1e-12 * abs(o.meanValue("hice"))


def test_spherical_bbm_is_refused(gpu):
    """The BBM's element size (sqrt of the area of the raw vertex coordinates)
    would be in radians on a sphere; the oracle restated from the reference
    diverges in its first step there.  The library refuses the combination."""
    case = _sphere_case(14, 12)
    with pytest.raises(NsdgError) as e:
        _sphere_make(BBMDynamicsKernel(dg_comp=6, n_steps=50), case, damage=True)
    assert e.value.status == 6  # NSDG_ERR_UNSUPPORTED


@pytest.mark.parametrize("rheology,kernel", [("mevp", "tma"), ("mevp", "global")])
def test_spherical_mixed_precision_close_to_oracle(gpu, oracle, rheology, kernel, monkeypatch):
    """Both FP32 element kernels (NSDG_STRESS_KERNEL forces the choice)."""
    monkeypatch.setenv("NSDG_STRESS_KERNEL", kernel)
    case = _sphere_case(24, 18)
    bbm = rheology == "bbm"
    prm = dict(n_steps=50) if bbm else dict(alpha=1500.0, beta=1500.0, n_steps=100)
    cls = BBMDynamicsKernel if bbm else MEVPDynamicsKernel
    g = _sphere_make(cls(dg_comp=6, precision=1, **prm), case, damage=bbm)
    o = _sphere_make(oracle.OracleKernel(1 if bbm else 0, 6, **prm), case, damage=bbm)
    _sphere_advance(g, case, 3)
    _sphere_advance(o, case, 3)
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
    err = {f: rms(g.getDG0Data(f), o.getDG0Data(f)) for f in ("u", "v", "hice", "cice")}
    print(f"spherical {rheology} mixed ({kernel} element kernel): RMS vs oracle {err}")
    assert max(err["u"], err["v"]) <= 1e-5, err
    assert err["hice"] <= 1e-6 and err["cice"] <= 1e-6, err


def test_bounded_wait_runs_out_and_the_gpu_stays_usable(gpu):
    """Failure detection without a GPU fault: a device wait on an mbarrier
    that nothing completes gives up after its time limit and reports it."""
    import ctypes
    import time
    from nextsimdg_gb300 import _lib
    lib = _lib.load()
    flag = ctypes.c_int(-1)
    t0 = time.perf_counter()
    assert lib.nsdg_selftest_bounded_wait(0.02, ctypes.byref(flag)) == _lib.NSDG_OK
    assert flag.value == 1
    assert time.perf_counter() - t0 < 10.0
    assert lib.nsdg_selftest_bounded_wait(0.0, ctypes.byref(flag)) == _lib.NSDG_ERR_BAD_ARG
    box = BoxTest(8)
    g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=5, precision=1)
    _advance(g, box, 1)
    assert np.all(np.isfinite(g.getDG0Data("u")))


@pytest.mark.parametrize("precision", [0, 1])
def test_zero_thickness_is_handled(gpu, precision):
    """Open water everywhere (h = 0, A = 0): the clamps of prepareIteration
    (H, A >= 1e-4) keep the momentum finite; nothing is flagged."""
    box = BoxTest(12)
    g = _make(MEVPDynamicsKernel, box, 6, None, n_steps=20, precision=precision)
    g.setData("hice", np.zeros(box.nelements))
    g.setData("cice", np.zeros(box.nelements))
    _advance(g, box, 2)
    g.synchronize()
    for f in ("u", "v", "hice", "cice"):
        assert np.all(np.isfinite(g.getDG0Data(f))), f
    assert np.all(g.getDG0Data("hice") == 0.0)


@pytest.mark.parametrize("precision", [0, 1])
def test_sea_surface_height_gradient_matches_oracle(gpu, oracle, precision):
    """A non-zero sea surface height (the box test's is zero): the CG1
    gradient, its boundary extension and the CG1 -> CG2 interpolation
    (CGDynamicsKernel.cpp:126-258) enter the momentum balance."""
    box = BoxTest(20, 18)
    x = (np.arange(box.nelements) % box.nx + 0.5) / box.nx
    y = (np.arange(box.nelements) // box.nx + 0.5) / box.ny
    ssh = 0.4 * np.sin(2 * np.pi * x) * np.cos(np.pi * y) + 0.2 * y
    prm = dict(alpha=1500.0, beta=1500.0, n_steps=60)
    g = _make(MEVPDynamicsKernel, box, 6, None, precision=precision, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    for k in (g, o):
        k.setData("ssh", ssh)
    _advance(g, box, 3)
    _advance(o, box, 3)
    if precision == 0:
        worst = _compare(g, o, ["hice", "cice", "u", "v"], 6)
        assert all(v <= TOL for v in worst.values()), worst
    else:
        rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))  # noqa: E731
        assert rms(g.getDG0Data("u"), o.getDG0Data("u")) <= 1e-5
    # the gradient matters: without the ssh the velocity differs
    o2 = _make(oracle.OracleKernel, box, 6, 0, **prm)
    _advance(o2, box, 3)
    assert np.abs(o2.getDG0Data("u") - o.getDG0Data("u")).max() > 1e-4



@pytest.mark.parametrize("precision,alpha", [(0, 1500.0), (0, 300.0), (1, 300.0)])
def test_full_size_512_within_oracle_sensitivity(gpu, oracle, precision, alpha):
    """The 512 x 512 DG2 box test (1 km cells; the mixed-precision benchmark
    grid), two full steps, FP64 or mixed precision, against the oracle on the
    same inputs.  On 1 km cells both relaxations amplify rounding within two
    steps (the oracle's own response to h x (1 + 1e-14) reaches ~1e-6 in u),
    so the bar per field is 10x that response (h and A follow through
    advection by the perturbed velocity); 1e-10 where the response stays
    below 1e-11, and never below 1e-6 for the mixed-precision path."""
    box = BoxTest(512)
    prm = dict(alpha=alpha, beta=alpha, n_steps=100)
    g = _make(MEVPDynamicsKernel, box, 6, None, precision=precision, **prm)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    o2 = oracle.OracleKernel(0, 6, **prm)
    o2.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        o2.setData(name, arr * (1.0 + 1e-14) if name == "hice" else arr)
    for k in (g, o, o2):
        _advance(k, box, 2)
    names = ["hice", "cice", "u", "v"]
    worst = _compare(g, o, names, 6)
    sens = _compare(o2, o, names, 6)
    floor = 1e-6 if precision else TOL
    print(f"512x512 precision {precision} alpha {alpha}: gpu vs oracle {worst}, oracle sensitivity {sens}")
    for n in names:
        bar = TOL if sens[n] < 1e-11 else 10.0 * sens[n]
        assert worst[n] <= max(bar, floor), (n, worst, sens)
    assert np.abs(o.getDG0Data("u")).max() > 1e-3


def test_largest_grid_within_oracle_sensitivity(gpu, oracle):
    """The 1024 x 1024 DG2 box test (0.5 km cells, the learned warm start's
    evaluation grid and the largest the bench runs), one step, FP64 and mixed
    precision against the oracle on the same inputs.  One step already
    amplifies the oracle's own response to h x (1 + 1e-14) to about 3e-3 of
    u (alpha = beta = 1500 is far from converged on 0.5 km cells), so the bar
    per field is 10x that response, as on 512 x 512."""
    box = BoxTest(1024)
    prm = dict(alpha=1500.0, beta=1500.0, n_steps=100)
    o = _make(oracle.OracleKernel, box, 6, 0, **prm)
    o2 = oracle.OracleKernel(0, 6, **prm)
    o2.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        o2.setData(name, arr * (1.0 + 1e-14) if name == "hice" else arr)
    gs = [_make(MEVPDynamicsKernel, box, 6, None, precision=p, **prm) for p in (0, 1)]
    for k in [o, o2] + gs:
        _advance(k, box, 1)
    names = ["hice", "cice", "u", "v"]
    sens = _compare(o2, o, names, 6)
    assert sens["u"] > 1e-6  # the configuration is ill-conditioned
    for p, g in zip((0, 1), gs):
        worst = _compare(g, o, names, 6)
        print(f"1024x1024 precision {p}: gpu vs oracle {worst}, oracle sensitivity {sens}")
        for n in names:
            bar = TOL if sens[n] < 1e-11 else 10.0 * sens[n]
            assert worst[n] <= max(bar, 1e-6 if p else TOL), (p, n, worst, sens)
        assert np.all(np.isfinite(g.getDG0Data("u")))
        g.close()


def test_host_arrays_moved_by_kernel_match_copies(gpu, monkeypatch):
    """Pageable host arrays (numpy) moved by the direct-access kernel
    (set_data, get_dg0 and module_step; on a GPU that reads pageable host
    memory) give bitwise the results of the copy-engine path
    (NSDG_HOST_DIRECT=0), and page-locked arrays keep the copies."""
    box = BoxTest(40, 36)
    prm = dict(alpha=300.0, beta=300.0, n_steps=100)
    d = _make(MEVPDynamicsKernel, box, 6, None, precision=1, **prm)
    monkeypatch.setenv("NSDG_HOST_DIRECT", "0")
    c = _make(MEVPDynamicsKernel, box, 6, None, precision=1, **prm)
    monkeypatch.delenv("NSDG_HOST_DIRECT")
    assert not c.host_direct()
    print("direct host access:", d.host_direct())
    outs = ["hice", "cice", "u", "v", "uiostress", "viostress"]
    for s in range(3):
        uw, vw = box.wind(s * box.dt)
        for k in (d, c):
            k.setData("uwind", uw)
            k.setData("vwind", vw)
            k.update(s * box.dt, box.dt)
        for n in outs:
            np.testing.assert_array_equal(d.getDG0Data(n), c.getDG0Data(n), err_msg=f"step {s}: {n}")
    for s in range(3, 5):
        uw, vw = box.wind(s * box.dt)
        inputs = {"uwind": uw, "vwind": vw, "hice": d.getDG0Data("hice"), "cice": d.getDG0Data("cice")}
        a = d.module_step(s * box.dt, box.dt, inputs, outs)
        b = c.module_step(s * box.dt, box.dt, inputs, outs)
        for n in outs:
            np.testing.assert_array_equal(a[n], b[n], err_msg=f"module step {s}: {n}")
    d.close()
    c.close()


@pytest.mark.parametrize("rheology,precision", [("mevp", 0), ("mevp", 1), ("bbm", 0)])
def test_module_step_matches_separate_calls(gpu, rheology, precision):
    """nsdg_kernel_module_step (the module step in one call: the inputs,
    update, the read-outs, one wait) gives bitwise what the separate setData,
    update and getDG0Data calls give, including a stored (not advected)
    field passed through; an unknown output is refused before anything is
    copied."""
    box = BoxTest(40, 36)
    bbm = rheology == "bbm"
    cls = BBMDynamicsKernel if bbm else MEVPDynamicsKernel
    prm = dict(n_steps=50) if bbm else dict(alpha=300.0, beta=300.0, n_steps=100)
    ks = []
    for _ in range(2):
        k = cls(dg_comp=6, precision=precision, **prm)
        k.initialise(box.coords(), False, box.mask())
        for name, arr in box.initial_fields().items():
            k.setData(name, arr)
        if bbm:
            k.setData("damage", box.damage())
        ks.append(k)
    sep, bat = ks
    outs = ["hice", "cice", "u", "v", "uiostress", "viostress"] + (["damage"] if bbm else [])
    tracer = np.linspace(0.0, 1.0, box.nelements)
    for s in range(3):
        uw, vw = box.wind(s * box.dt)
        h, a = sep.getDG0Data("hice"), sep.getDG0Data("cice")
        inputs = {"hice": h, "cice": a, "uwind": uw, "vwind": vw, "tracer": tracer + s}
        for name, arr in inputs.items():
            sep.setData(name, arr)
        sep.update(s * box.dt, box.dt)
        want = {n: sep.getDG0Data(n) for n in outs + ["tracer"]}
        got = bat.module_step(s * box.dt, box.dt, inputs, outs + ["tracer"])
        for n in want:
            np.testing.assert_array_equal(got[n], want[n], err_msg=f"step {s}: {n}")
    with pytest.raises(KeyError):  # NSDG_ERR_UNKNOWN_FIELD, as getDG0Data raises it
        bat.module_step(0.0, box.dt, {"uwind": uw}, ["not_a_field"])
    for k in ks:
        k.close()
