"""The network oracle (numpy) against finite differences (CPU)."""
import numpy as np

from oracle import cnn_oracle as co


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    chans = [3, 4, 2]
    Ws = [rng.standard_normal((3, 3, chans[i], chans[i + 1])) * 0.4 for i in range(2)]
    bs = [rng.standard_normal(chans[i + 1]) * 0.1 for i in range(2)]
    x = rng.standard_normal((2, 5, 6, 3))
    t = rng.standard_normal((2, 5, 6, 2))
    m = (rng.random((2, 5, 6)) > 0.3).astype(float)
    loss, gWs, gbs, _ = co.loss_and_grads(x, t, m, Ws, bs)
    eps = 1e-6
    for li in range(2):
        for idx in [(0, 0, 0, 0), (1, 2, 1, 1), (2, 1, chans[li] - 1, 0)]:
            Wp = [w.copy() for w in Ws]
            Wp[li][idx] += eps
            lp = co.loss_and_grads(x, t, m, Wp, bs)[0]
            Wp[li][idx] -= 2 * eps
            lm = co.loss_and_grads(x, t, m, Wp, bs)[0]
            assert abs((lp - lm) / (2 * eps) - gWs[li][idx]) < 1e-6 * max(1.0, abs(gWs[li][idx]))
        bp = [b.copy() for b in bs]
        bp[li][0] += eps
        lp = co.loss_and_grads(x, t, m, Ws, bp)[0]
        bp[li][0] -= 2 * eps
        lm = co.loss_and_grads(x, t, m, Ws, bp)[0]
        assert abs((lp - lm) / (2 * eps) - gbs[li][0]) < 1e-6


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 1e-30])
    r = co.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
