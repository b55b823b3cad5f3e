"""The CPU oracle of the warm-start network: its backward pass against central
finite differences (float64), and its BF16 mode against its float64 mode."""
import numpy as np

import mlp_oracle as mo


def _params(width=128, hidden=2, seed=0):
    rng = np.random.default_rng(seed)
    shapes = [(width, mo.NIN_PAD)] + [(width, width)] * (hidden - 1) + [(mo.NOUT_PAD, width)]
    ps = []
    for l, (r, c) in enumerate(shapes):
        W = np.zeros((r, c))
        rt = mo.NOUT if l == len(shapes) - 1 else r
        ct = mo.NIN if l == 0 else c
        W[:rt, :ct] = rng.uniform(-1, 1, (rt, ct)) * np.sqrt(6.0 / ct)
        b = np.zeros(r)
        b[:rt] = rng.normal(0, 0.1, rt)
        ps.append((W, b))
    return ps


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    ps = _params()
    x = rng.normal(size=(8, mo.NIN))
    y = rng.normal(size=(8, mo.NOUT))
    _, g = mo.loss_grad(ps, x, y, bf16=False)
    for layer, idx in [(0, (3, 2)), (0, (10, 6)), (1, (5, 7)), (2, (1, 9)), (2, (4, 100))]:
        fd = mo.fd_check(ps, x, y, layer, idx)
        assert abs(fd - g[layer][0][idx]) <= 1e-7 * max(1.0, abs(fd)), (layer, idx, fd, g[layer][0][idx])


def test_bf16_mode_close_to_float64():
    rng = np.random.default_rng(2)
    ps = _params()
    x = rng.normal(size=(64, mo.NIN))
    y = rng.normal(size=(64, mo.NOUT))
    l64, g64 = mo.loss_grad(ps, x, y, bf16=False)
    l16, g16 = mo.loss_grad([(W.astype(np.float32), b.astype(np.float32)) for W, b in ps],
                            x.astype(np.float32), y.astype(np.float32), bf16=True)
    assert abs(l16 - l64) <= 2e-2 * l64
    for (a, _), (b, _) in zip(g64, g16):
        assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(a)


def test_bf16_rounding():
    # BF16 keeps 8 significant bits: ulp(1) = 2^-7; halfway cases go to even
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0078125 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 0.0], np.float32)
    r = mo.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == 1.0078125 and r[4] == -2.5
