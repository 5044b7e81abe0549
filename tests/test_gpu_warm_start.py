"""Learned warm start of the mixed-precision mEVP sub-cycle, through the C ABI.

The plain sub-cycle (100 iterations) is the audit: a warm sub-cycle (network
+ K iterations) is compared with it from the same state, next to the cold
sub-cycle with the same K iterations and no network.  The fallback (restore
the state at the start of the sub-cycle, run the full count) must reproduce
the plain update bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 96
K = 40


def _box(**kw):
    from nextsimdg_gb300.boxtest import BoxTest
    return BoxTest(N, **kw)


def _kernel(box, precision=1, n_steps=100, alpha=1500.0):
    from nextsimdg_gb300.boxtest import setup_kernel
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel
    return setup_kernel(MEVPDynamicsKernel(dg_comp=6, alpha=alpha, beta=alpha, n_steps=n_steps,
                                           precision=precision), box)


def _run(k, box, steps, start=0):
    from nextsimdg_gb300.boxtest import step_forcing
    for s in range(start, start + steps):
        step_forcing(k, box, s)
        k.update(s * box.dt, box.dt)


def _rms(a):
    return float(np.sqrt(np.mean(a * a)))


@pytest.fixture(scope="module")
def trained(gpu):
    """A network trained on a trajectory other than the evaluation one."""
    from nextsimdg_gb300 import surrogate
    from nextsimdg_gb300.boxtest import step_forcing
    tb = _box(seed=1, start=(0.42 * 512e3, 0.47 * 512e3), wind_speed=9.0, h_noise=0.01)
    k = _kernel(tb)
    net = surrogate.warm_net(N, N, max_batch=2, seed=3)
    nsamp = 80
    net.dataset_reserve(nsamp)
    ratios = []
    for s in range(nsamp):
        step_forcing(k, tb, s)
        ratios.append(k.warm_sample(s * tb.dt, tb.dt, K, net, s))
    net.dataset_normalise(nsamp)
    first = net.train(nsamp, 40, batch=2, lr=1e-3, seed=0)
    net.train(nsamp, 500, batch=2, lr=1e-3, seed=1)
    last = net.train(nsamp, 400, batch=2, lr=2e-4, seed=2)
    k.close()
    return net, max(ratios), first, last


def test_warm_sample_is_a_plain_update(gpu):
    """Recording a sample does not change the step: bitwise equal to update()."""
    from nextsimdg_gb300 import surrogate
    from nextsimdg_gb300.boxtest import step_forcing
    box = _box()
    a, b = _kernel(box), _kernel(box)
    net = surrogate.warm_net(N, N)
    net.dataset_reserve(3)
    for s in range(3):
        step_forcing(a, box, s)
        a.update(s * box.dt, box.dt)
        step_forcing(b, box, s)
        r = b.warm_sample(s * box.dt, box.dt, K, net, s)
        assert np.isfinite(r) and 0 < r < 1
    for f in ("u", "v", "hice", "cice"):
        np.testing.assert_array_equal(a.getDG0Data(f), b.getDG0Data(f))


def test_training_reduces_loss(trained):
    _, _, first, last = trained
    assert last < 0.5 * first, (first, last)


def test_warm_start_beats_cold_start(trained):
    """Network + K iterations lands closer to the plain 100-iteration result
    than K iterations alone, on states of the evaluation trajectory."""
    net, kappa, _, _ = trained
    box = _box()
    plain = _kernel(box)
    _run(plain, box, 30)
    warm, cold = _kernel(box), _kernel(box, n_steps=K)
    warm.set_warm_start(net, K, kappa * 10.0)
    from nextsimdg_gb300.boxtest import step_forcing
    ew, ec = [], []
    for s in range(30, 36):
        snap = plain.snapshot()
        u0, v0 = plain.getDG0Data("u"), plain.getDG0Data("v")
        res = {}
        for name, kk in (("warm", warm), ("cold", cold)):
            kk.restore(snap)
            step_forcing(kk, box, s)
            kk.update(s * box.dt, box.dt)
            res[name] = (kk.getDG0Data("u"), kk.getDG0Data("v"))
        step_forcing(plain, box, s)
        plain.update(s * box.dt, box.dt)
        up, vp = plain.getDG0Data("u"), plain.getDG0Data("v")
        scale = _rms(np.hypot(up - u0, vp - v0))
        ew.append(_rms(np.hypot(res["warm"][0] - up, res["warm"][1] - vp)) / scale)
        ec.append(_rms(np.hypot(res["cold"][0] - up, res["cold"][1] - vp)) / scale)
    st = warm.warm_stats()
    assert st["fallbacks"] == 0 and st["accepted"] == 6
    # the gain of the trained network over the method without it
    assert max(ew) < 0.5 * min(ec), (ew, ec)


def test_fallback_reproduces_plain_update(trained):
    """kappa = 0 rejects every warm sub-cycle: the update must equal the plain
    mixed-precision update exactly (restore + full iteration count)."""
    net, _, _, _ = trained
    box = _box()
    a, b = _kernel(box), _kernel(box)
    b.set_warm_start(net, K, 0.0)
    _run(a, box, 3)
    _run(b, box, 3)
    for f in ("u", "v", "hice", "cice"):
        np.testing.assert_array_equal(a.getDG0Data(f), b.getDG0Data(f))
    st = b.warm_stats()
    assert (st["accepted"], st["fallbacks"]) == (0, 3) and st["last_ratio"] > 0


def test_nonfinite_network_falls_back(trained):
    """A network producing NaN increments is rejected on the device (its
    numeric fault stays private to the warm attempt) and the step is the
    plain one."""
    from nextsimdg_gb300 import surrogate
    net, kappa, _, _ = trained
    bad = surrogate.warm_net(N, N, seed=5)
    p = net.get_params()
    p[-32] = np.nan  # bias of output channel 0 (u increment at the first owned node)
    bad.set_params(p)
    bad.set_normalisation(net.get_normalisation())
    box = _box()
    a, b = _kernel(box), _kernel(box)
    b.set_warm_start(bad, K, kappa * 10.0)
    _run(a, box, 2)
    _run(b, box, 2)
    b.synchronize()
    for f in ("u", "v"):
        np.testing.assert_array_equal(a.getDG0Data(f), b.getDG0Data(f))
    st = b.warm_stats()
    assert (st["accepted"], st["fallbacks"]) == (0, 2)


def test_audited_updates_keep_the_plain_result(trained):
    """audit_every = 1: every update runs warm and plain from the same start
    and keeps the plain result (bitwise the plain update)."""
    net, kappa, _, _ = trained
    box = _box()
    a, b = _kernel(box), _kernel(box)
    b.set_warm_start(net, K, kappa * 10.0, audit_every=1, audit_tol=1.0)
    _run(a, box, 3)
    _run(b, box, 3)
    for f in ("u", "v", "hice", "cice"):
        np.testing.assert_array_equal(a.getDG0Data(f), b.getDG0Data(f))
    st = b.warm_stats()
    assert st["audited"] == 3 and st["audit_rejected"] == 0 and st["enabled"] == 1
    assert 0 < st["last_audit_error"] < 1.0


def test_failed_audit_disables_warm_start(trained):
    """audit_tol = 0 fails the first audit: the next updates fall back
    (plain result) until the next audit."""
    net, kappa, _, _ = trained
    box = _box()
    a, b = _kernel(box), _kernel(box)
    b.set_warm_start(net, K, kappa * 10.0, audit_every=3, audit_tol=0.0)
    _run(a, box, 3)
    _run(b, box, 3)
    for f in ("u", "v", "hice", "cice"):
        np.testing.assert_array_equal(a.getDG0Data(f), b.getDG0Data(f))
    st = b.warm_stats()
    assert (st["audited"], st["audit_rejected"], st["accepted"], st["fallbacks"], st["enabled"]) == (1, 1, 0, 2, 0)


def test_detach_restores_plain_graph(trained):
    net, kappa, _, _ = trained
    box = _box()
    a, b = _kernel(box), _kernel(box)
    b.set_warm_start(net, K, kappa * 10.0)
    _run(b, box, 1)
    b.set_warm_start(None)
    a.restore(b.snapshot())
    _run(a, box, 2, start=1)
    _run(b, box, 2, start=1)
    np.testing.assert_array_equal(a.getDG0Data("u"), b.getDG0Data("u"))


def test_warm_start_argument_errors(trained):
    from nextsimdg_gb300 import surrogate
    from nextsimdg_gb300._lib import NsdgError, NSDG_ERR_UNSUPPORTED, NSDG_ERR_SIZE_MISMATCH, NSDG_ERR_BAD_ARG
    net, _, _, _ = trained
    box = _box()
    with pytest.raises(NsdgError) as e:
        _kernel(box, precision=0).set_warm_start(net, K, 1.0)
    assert e.value.status == NSDG_ERR_UNSUPPORTED
    k = _kernel(box)
    with pytest.raises(NsdgError) as e:
        k.set_warm_start(surrogate.warm_net(N + 2, N), K, 1.0)
    assert e.value.status == NSDG_ERR_SIZE_MISMATCH
    for kk, kap, je, jt in ((0, 1.0, 0, 0.0), (101, 1.0, 0, 0.0), (K, -1.0, 0, 0.0), (K, float("nan"), 0, 0.0),
                            (K, 1.0, -1, 0.0), (K, 1.0, 5, float("inf"))):
        with pytest.raises(NsdgError) as e:
            k.set_warm_start(net, kk, kap, je, jt)
        assert e.value.status == NSDG_ERR_BAD_ARG
    with pytest.raises(NsdgError) as e:
        k.warm_sample(0.0, 120.0, K, net, 10_000)
    assert e.value.status == NSDG_ERR_BAD_ARG
