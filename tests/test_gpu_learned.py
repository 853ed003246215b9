"""Learned aliasing correction: the hand-written BF16/FP32 MLP kernels against the
float64 oracle (oracle.mlp_forward_backward), and what the trained network gains
over the uncorrected coarse, non-interlaced estimator on held-out fields."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def L():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import learned
    return learned


def test_mlp_forward_and_gradient_match_oracle(L):
    """Same BF16-rounded weights in both; FP32 accumulation on the GPU vs float64:
    outputs within 1e-5, gradients within 1e-3 of the largest component."""
    rng = np.random.default_rng(2)
    flat = np.concatenate([np.concatenate([rng.normal(0.0, np.sqrt(1.0 / fi), fo * fi), rng.normal(0.0, 0.1, fo)])
                           for fo, fi in ((64, 4), (64, 64), (64, 64), (1, 64))]).astype(np.float32)
    net = L.MLP(flat=flat)
    x = rng.normal(size=(300, 4)).astype(np.float32)
    t = rng.normal(size=300).astype(np.float32)
    w = rng.uniform(0.5, 2.0, size=300).astype(np.float32)
    flat = net.bf16.float().cpu().numpy().astype(np.float64)
    loss_ref, g_ref, y_ref = O.mlp_forward_backward(flat, x, t, w)
    y = net.forward(x).cpu().numpy()
    np.testing.assert_allclose(y, y_ref, rtol=1e-5, atol=1e-5)
    loss = net.gradient(x, t, w)
    g = net.grad.cpu().numpy()
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert np.abs(g - g_ref).max() <= 1e-3 * np.abs(g_ref).max()


def test_adam_step_decreases_loss(L):
    net = L.MLP(seed=1)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, size=(512, 4)).astype(np.float32)
    t = np.sin(2 * x[:, 0]) * 0.1 + 0.05 * x[:, 2]
    first = net.gradient(x, t)
    for _ in range(200):
        net.gradient(x, t)
        net.adam(3e-3)
    assert net.gradient(x, t) < 0.2 * first


def test_learned_correction_gains_over_plain(L):
    """Train on pairs made by this library (coarse 32^3 plain vs 128^3 interlaced,
    features estimated from the coarse spectrum),
    then on held-out fields the corrected coarse monopole is closer to the
    interlaced fine one than the plain coarse estimate, bin by bin up to 0.8 k_Nyq."""
    train = L.training_set(64, seed=11, coarse=(32,))
    held = L.training_set(8, seed=97, coarse=(32,))
    net, losses = L.train(train, steps=5000)
    assert losses[-1] < 0.5 * losses[0]
    corr = L.Correction(net)
    plain, fixed = [], []
    for p in held:
        kN = np.pi * p['N'] / p['L']
        pc = corr.apply(p['k'], p['Pc'], kN, p['MAS'], p['slope_est'], p['shot_est'])
        plain.append(np.abs(np.log(p['Pc'] / p['Pf'])))
        fixed.append(np.abs(np.log(pc / p['Pf'])))
    plain, fixed = np.concatenate(plain), np.concatenate(fixed)
    print('held-out mean |log ratio|: plain %.4f corrected %.4f' % (plain.mean(), fixed.mean()))
    assert fixed.mean() < 0.7 * plain.mean()


def test_shipped_weights_evaluation_small(L):
    """The shipped weights on a held-out 128^3-particle field: corrected 64^3 plain
    estimate against the interlaced 128^3 one, with features estimated from the coarse
    spectrum itself; the correction must reduce the mean error up to 0.8 k_Nyq."""
    r = L.evaluate(N=64, side=128, seed=1234, reps=1)
    print('eval 64^3: plain max %.4f mean %.4f, learned max %.4f mean %.4f, slope est %.3f'
          % (r['max_err_plain'], r['mean_err_plain'], r['max_err_learned'], r['mean_err_learned'],
             r['slope_est']))
    assert r['bins'] > 20
    assert r['mean_err_learned'] < r['mean_err_plain']
