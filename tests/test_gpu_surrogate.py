"""GPU network kernels (BF16 products, FP32 accumulation) against the numpy
oracle: forward output, loss, weight and bias gradients, with the
convolutions on tcgen05 (the default) and by mma.sync (NSDG_CONV=mma); the
two against each other on the warm start's network shape; and a short
training run."""
import numpy as np
import pytest

from oracle import cnn_oracle as co

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.parametrize("conv", ["tcgen05", "tcgen05_m128", "mma"])
@pytest.mark.parametrize("chans,H,W,B,used", [([16, 32, 32, 16], 10, 13, 2, 12), ([48, 48, 32], 9, 70, 1, 26),
                                              ([64, 48, 64, 32], 5, 131, 2, 20)])
def test_net_gradients_match_oracle(gpu, monkeypatch, conv, chans, H, W, B, used):
    """tcgen05: the weight gradient's MMAs with the input channels as 64 rows
    (the default); tcgen05_m128: as 128 rows (NSDG_WGRAD_M=128); mma: every
    convolution on mma.sync."""
    from nextsimdg_gb300.surrogate import Net
    if conv == "mma":
        monkeypatch.setenv("NSDG_CONV", "mma")
    else:
        monkeypatch.delenv("NSDG_CONV", raising=False)
    if conv == "tcgen05_m128":
        monkeypatch.setenv("NSDG_WGRAD_M", "128")
    else:
        monkeypatch.delenv("NSDG_WGRAD_M", raising=False)
    rng = np.random.default_rng(11)
    net = Net(chans, H, W, max_batch=B, used_outputs=used, seed=5)
    p = net.get_params()
    p[:] = (rng.standard_normal(p.size) * 0.2).astype(np.float32)  # nonzero biases too
    net.set_params(p)
    Ws, bs = net.unpack(p)
    x = rng.standard_normal((B, H, W, chans[0])).astype(np.float32)
    t = np.zeros((B, H, W, chans[-1]), dtype=np.float32)
    t[..., :used] = rng.standard_normal((B, H, W, used))
    m = (rng.random((B, H, W)) > 0.2).astype(np.float32)
    net.set_batch(x, t, m)
    out = net.forward()
    loss_g = net.loss_backward()
    g = net.get_grads()
    gWs, gbs = net.unpack(g)
    loss_o, gWo, gbo, out_o = co.loss_and_grads_bf16(x.astype(np.float64), t[..., :used].astype(np.float64),
                                                      m.astype(np.float64), Ws, bs)
    assert _rel(out, out_o) < 1e-3
    assert abs(loss_g - loss_o) <= 1e-3 * loss_o
    for l in range(len(Ws)):
        assert _rel(gWs[l], gWo[l]) < 2e-2, l
        assert _rel(gbs[l], gbo[l]) < 2e-2, l


def test_net_training_reduces_loss(gpu):
    """Fit a smooth target map (a fixed random 3x3 linear filter of the input)."""
    from nextsimdg_gb300.surrogate import Net
    rng = np.random.default_rng(2)
    H = W = 24
    net = Net([16, 32, 32, 16], H, W, max_batch=4, used_outputs=4, seed=1)
    K = rng.standard_normal((3, 3, 16, 16)) * 0.1
    x = rng.standard_normal((4, H, W, 16))
    t = co.conv3x3(x, K, np.zeros(16)).astype(np.float32)
    t[..., 4:] = 0
    m = np.ones((4, H, W), dtype=np.float32)
    net.set_batch(x, t, m)
    losses = []
    for _ in range(300):
        net.forward()
        losses.append(net.loss_backward())
        net.adam_step(lr=3e-3)
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])


def test_tensor_core_convolutions_match_mma_sync(gpu, monkeypatch):
    """The warm start's network (64-48-48-48-48-48-32) on a 3 x 40 x 200 batch
    (two 128-pixel tiles per row, the second partial): forward output and
    gradients with tcgen05 against mma.sync, and the tcgen05 forward run to
    run bitwise reproducible."""
    from nextsimdg_gb300 import surrogate
    rng = np.random.default_rng(4)
    H, W, B = 40, 200, 3
    out, grads = {}, {}
    for conv in ("mma", "tcgen05"):
        if conv == "mma":
            monkeypatch.setenv("NSDG_CONV", "mma")
        else:
            monkeypatch.delenv("NSDG_CONV", raising=False)
        net = surrogate.Net(list(surrogate.WARM_CHANNELS), H, W, max_batch=B, used_outputs=26, seed=3)
        x = rng.standard_normal((B, H, W, net.channels[0])).astype(np.float32) if conv == "mma" else x
        t = np.zeros((B, H, W, net.channels[-1]), dtype=np.float32)
        t[..., :26] = 0.3
        m = np.ones((B, H, W), dtype=np.float32)
        net.set_batch(x, t, m)
        out[conv] = net.forward()
        if conv == "tcgen05":
            assert np.array_equal(net.forward(), out[conv])
        net.loss_backward()
        grads[conv] = net.get_grads()
        net.close()
    assert np.all(np.isfinite(out["tcgen05"]))
    assert _rel(out["tcgen05"], out["mma"]) < 2e-3
    assert _rel(grads["tcgen05"], grads["mma"]) < 2e-2
