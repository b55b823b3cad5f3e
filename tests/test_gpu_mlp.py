"""The learned warm start on the GPU: forward/backward kernels against the CPU
oracle of the network, training on solved fields, and what the warm start
gains over the freestream start of the same cases."""
import numpy as np
import pytest

import mlp_oracle as mo
from helpers import small_case

pytestmark = pytest.mark.gpu


def test_mlp_loss_and_gradients_match_oracle(gpu_lib):
    net = gpu_lib.WarmStartNet(hidden=3, width=128, seed=7)
    rng = np.random.default_rng(3)
    params = [net.get_weights(l) for l in range(net.nlin)]
    # non-zero biases so every term of the backward pass is exercised
    for l, (W, b) in enumerate(params):
        rows = mo.NOUT if l == net.nlin - 1 else W.shape[0]
        b = b.copy()
        b[:rows] = rng.normal(0, 0.1, rows).astype(np.float32)
        net.set_weights(l, W, b)
        params[l] = (W, b)
    x = rng.normal(size=(512, mo.NIN)).astype(np.float32)
    y = rng.normal(size=(512, mo.NOUT)).astype(np.float32)
    loss = net.loss_grad(x, y)
    lo, go = mo.loss_grad(params, x, y, bf16=True)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for l in range(net.nlin):
        gw, gb = net.get_grads(l)
        ow, ob = go[l]
        assert np.linalg.norm(gw - ow) <= 2e-2 * np.linalg.norm(ow), l
        assert np.linalg.norm(gb - ob) <= 2e-2 * np.linalg.norm(ob) + 1e-12, l
    # padded rows/columns carry no gradient
    assert np.all(net.get_grads(0)[0][:, mo.NIN:] == 0.0)
    assert np.all(net.get_grads(net.nlin - 1)[0][mo.NOUT:, :] == 0.0)


def _family(n, seed, nx=65, ny=17):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        M, aoa = rng.uniform(0.4, 0.6), rng.uniform(0.0, 4.0)
        out.append(small_case(nx=nx, ny=ny, Ma=M, AoA=aoa, Re=1.0e6, If_viscous=1, Iflag_turbulence_model=2,
                              Iflag_flux=4, Iflag_Scheme=5, CFL=5.0, first=2e-4))
    return out


def test_training_on_solved_fields_and_warm_start_gain(gpu_lib):
    """12 SA cases (M 0.4-0.6, AoA 0-4 deg) solved for 3000 steps train the
    network (6 hidden layers of 256); on 4 held-out cases the warm start must
    reach a 1e-4 drop of the freestream start's first residual in at most 70 %
    of the steps the freestream start needs (measured: about 45 %)."""
    train = _family(12, seed=11)
    s = gpu_lib.Solver(train)
    s.set_lusgs_precision(32)
    s.init_flow()
    s.step(3000)
    net = gpu_lib.WarmStartNet(hidden=6, width=256, seed=5)
    net.add_samples(s)
    assert net.num_samples() == 12 * 64 * 16
    net.fit_normalization()
    l0 = net.train(1, batch=8192, lr=1e-3)
    net.train(1800, batch=8192, lr=1e-3)
    l1 = net.train(1200, batch=8192, lr=3e-4)
    assert l1 < 0.05 * l0, (l0, l1)
    s.close()

    held = _family(4, seed=12)
    # freestream start: the reference residual is its first step's
    a = gpu_lib.Solver(held)
    a.set_lusgs_precision(32)
    a.init_flow()
    a.step(1)
    r0 = np.array([a.norms(c)[1][0] for c in range(1, 5)])
    n_free, ratio_a, _ = a.run_to_drop(drop=1e-4, r0=r0, max_steps=20000, check_every=10)
    b = gpu_lib.Solver(held)
    b.set_lusgs_precision(32)
    assert net.warm_start(b) == 0
    n_warm, ratio_b, _ = b.run_to_drop(drop=1e-4, r0=r0, max_steps=20000, check_every=10)
    assert ratio_a <= 1e-4 and ratio_b <= 1e-4
    assert n_warm <= 0.7 * (n_free + 1), (n_warm, n_free)


def test_tcgen05_gemm_matches_mma_sync(gpu_lib):
    """The tcgen05 GEMM path (TMEM accumulators) against the mma.sync path on
    the same weights and batch: loss and every gradient agree to FP32
    accumulation-order round-off (BF16 activations may differ by one ulp)."""
    rng = np.random.default_rng(9)
    x = rng.normal(size=(1024, mo.NIN)).astype(np.float32)
    y = rng.normal(size=(1024, mo.NOUT)).astype(np.float32)
    res = []
    for kind in (0, 1):
        net = gpu_lib.WarmStartNet(hidden=3, width=256, seed=3)
        net.set_gemm(kind)
        loss = net.loss_grad(x, y)
        res.append((loss, [net.get_grads(l) for l in range(net.nlin)]))
        net.close()
    (l0, g0), (l1, g1) = res
    assert abs(l1 - l0) <= 1e-4 * abs(l0), (l0, l1)
    for (a, ab), (b, bb) in zip(g0, g1):
        assert np.linalg.norm(a - b) <= 5e-3 * np.linalg.norm(a)
        assert np.linalg.norm(ab - bb) <= 5e-3 * np.linalg.norm(ab) + 1e-12
