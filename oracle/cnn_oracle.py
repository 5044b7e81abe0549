"""CPU reference of the warm-start network (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the checker for the GPU network kernels
(nextsimdg_gb300/csrc/nsdg_surrogate.cu).  The network is a stack of 3x3
convolutions with "same" zero padding on a channels-last grid:

    z_l = conv3x3(x_l, W_l) + b_l,   x_{l+1} = relu(z_l)  (identity after the last layer)
    conv3x3(x, W)[b, y, x, o] = sum_{dy, dx, c} x[b, y + dy - 1, x + dx - 1, c] * W[dy, dx, c, o]

and the training loss is the masked mean squared error
    L = sum_{b,y,x,o} m[b,y,x] (out - target)^2 / (sum m * C_out).
"""
from __future__ import annotations

import numpy as np


def conv3x3(x, W, b):
    B, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.broadcast_to(b, (B, H, Wd, W.shape[3])).astype(np.float64).copy()
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("bhwc,co->bhwo", xp[:, dy:dy + H, dx:dx + Wd, :], W[dy, dx])
    return out


def conv3x3_backward(x, W, gout):
    """Gradients of sum(gout * conv3x3(x, W, b)) w.r.t. x, W and b."""
    B, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    gxp = np.zeros_like(xp)
    gW = np.zeros_like(W, dtype=np.float64)
    for dy in range(3):
        for dx in range(3):
            gxp[:, dy:dy + H, dx:dx + Wd, :] += np.einsum("bhwo,co->bhwc", gout, W[dy, dx])
            gW[dy, dx] = np.einsum("bhwc,bhwo->co", xp[:, dy:dy + H, dx:dx + Wd, :], gout)
    return gxp[:, 1:-1, 1:-1, :], gW, gout.sum(axis=(0, 1, 2))


def forward(x, weights, biases):
    """Returns the activations of every layer (inputs of the next) and the output."""
    acts = [x]
    for i, (W, b) in enumerate(zip(weights, biases)):
        z = conv3x3(acts[-1], W, b)
        acts.append(np.maximum(z, 0.0) if i < len(weights) - 1 else z)
    return acts


def loss_and_grads(x, target, mask, weights, biases):
    acts = forward(x, weights, biases)
    out = acts[-1]
    cout = out.shape[-1]
    denom = mask.sum() * cout
    diff = (out - target) * mask[..., None]
    loss = float((diff * (out - target)).sum() / denom)
    g = 2.0 * diff / denom
    gWs, gbs = [None] * len(weights), [None] * len(weights)
    for i in range(len(weights) - 1, -1, -1):
        if i < len(weights) - 1:
            g = g * (acts[i + 1] > 0)
        gx, gWs[i], gbs[i] = conv3x3_backward(acts[i], weights[i], g)
        g = gx
    return loss, gWs, gbs, acts


def bf16_round(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a32 = np.asarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def loss_and_grads_bf16(x, target, mask, weights, biases):
    """The same computation with the GPU kernels' BF16 rounding points: the
    input, the weights used in the products, the stored hidden activations,
    the loss gradient and the back-propagated gradients are rounded to
    bfloat16; sums are exact (FP64) here and FP32 on the GPU."""
    q = bf16_round
    Wq = [q(W) for W in weights]
    acts = [q(x)]
    L = len(weights)
    for i in range(L):
        z = conv3x3(acts[-1], Wq[i], biases[i])
        acts.append(q(np.maximum(z, 0.0)) if i < L - 1 else z)
    out = acts[-1]
    cout = target.shape[-1]
    denom = mask.sum() * cout
    d = out[..., :cout] - target
    loss = float((mask[..., None] * d * d).sum() / denom)
    g = np.zeros_like(out)
    g[..., :cout] = q(2.0 * mask[..., None] * d / denom)
    gWs, gbs = [None] * L, [None] * L
    for i in range(L - 1, -1, -1):
        gx, gWs[i], gbs[i] = conv3x3_backward(acts[i], Wq[i], g)
        if i > 0:
            g = q(gx * (acts[i] > 0))
    return loss, gWs, gbs, out
