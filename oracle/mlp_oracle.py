"""CPU oracle of the warm-start network (test infrastructure only: the tests
load it to check the GPU kernels; the product never calls it).

The network has no counterpart in the reference: this module restates the
library's own definition (k_mlp.cu) in numpy -- standardised inputs padded to
64 columns, hidden layers z = h W^T + b with SiLU, a linear output layer,
mean-squared error over the 5 outputs -- and its exact backward pass.  With
`bf16=True` it rounds what the GPU rounds to BF16 (inputs, weights, hidden
activations, the output gradient and every back-propagated pre-activation
gradient), accumulating in float32; with `bf16=False` it runs in float64 for
finite-difference checks of the backward formulas.
"""
from __future__ import annotations

import numpy as np

NIN, NIN_PAD, NOUT, NOUT_PAD = 7, 64, 5, 128


def to_bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x, bf16=True):
    """params: list of (W [out x in], b [out]) with the padded shapes of the
    library; x: B x 7 standardised inputs.  Returns (out B x 5, cache)."""
    dt = np.float32 if bf16 else np.float64
    rnd = to_bf16 if bf16 else (lambda a: np.asarray(a, dt))
    B = x.shape[0]
    h = np.zeros((B, NIN_PAD), dt)
    h[:, :NIN] = x
    h = rnd(h)
    hs, zs = [h], []
    for l, (W, b) in enumerate(params):
        z = (h.astype(dt) @ rnd(W).astype(dt).T + b.astype(dt)).astype(dt)
        if l < len(params) - 1:
            zs.append(z)
            h = rnd(silu(z).astype(dt))
            hs.append(h)
        else:
            out = z
    return out[:, :NOUT], (hs, zs, out)


def loss_grad(params, x, y, bf16=True):
    """MSE over the 5 outputs and the gradients of every (W, b)."""
    dt = np.float32 if bf16 else np.float64
    rnd = to_bf16 if bf16 else (lambda a: np.asarray(a, dt))
    out5, (hs, zs, out) = forward(params, x, bf16)
    B = x.shape[0]
    e = out5 - y
    loss = float(np.mean(e.astype(np.float64) ** 2))
    d = np.zeros_like(out)
    d[:, :NOUT] = 2.0 * e / (B * NOUT)
    d = rnd(d)
    grads = [None] * len(params)
    for l in range(len(params) - 1, -1, -1):
        W, _ = params[l]
        h = hs[l]
        grads[l] = ((d.T.astype(dt) @ h.astype(dt)).astype(dt), d.sum(axis=0, dtype=dt))
        if l == 0:
            break
        dh = (d.astype(dt) @ rnd(W).astype(dt)).astype(dt)
        d = rnd((dh * dsilu(zs[l - 1])).astype(dt))
    return loss, grads


def fd_check(params, x, y, layer, idx, eps=1e-6):
    """Central finite difference of the float64 loss w.r.t. W[layer][idx]."""
    p = [(W.astype(np.float64).copy(), b.astype(np.float64).copy()) for W, b in params]
    W = p[layer][0]
    w0 = W[idx]
    W[idx] = w0 + eps
    lp, _ = loss_grad(p, x, y, bf16=False)
    W[idx] = w0 - eps
    lm, _ = loss_grad(p, x, y, bf16=False)
    W[idx] = w0
    return (lp - lm) / (2 * eps)
