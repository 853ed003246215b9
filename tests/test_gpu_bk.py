"""GPU parity of the bispectrum (shell fill + batched C2R + triple-product
reduction) against the reference's golden outputs and the oracle.

Tolerances: P(k_i) rtol 1e-4; B and Q within 1e-3 of max|B| / max|Q| over the
triangle set (B sums products of both signs, so its error is measured against
the largest bispectrum of the set, not bin by bin).
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def PKL():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.Pk_library as P
    return P


@pytest.fixture(scope='module')
def bk():
    return np.load(os.path.join(GOLDEN, 'bk_golden.npz'))


def check(r, B, Q, k, Pk):
    np.testing.assert_allclose(r.k, k, rtol=1e-14)
    np.testing.assert_allclose(r.Pk, Pk, rtol=1e-4)
    assert np.abs(r.B - B).max() <= 1e-3 * np.abs(B).max()
    assert np.abs(r.Q - Q).max() <= 1e-3 * np.abs(Q).max()


def test_bk_golden(PKL, bk):
    N, L, k1, k2 = bk['meta']
    r = PKL.Bk(bk['delta'], L, k1, k2, bk['theta'], 'CIC')
    check(r, bk['Bk_B'], bk['Bk_Q'], bk['Bk_k'], bk['Bk_Pk'])
    e = PKL.Bk(bk['delta'], L, 0.1, 0.1, np.array([2 * np.pi / 3]), 'CIC')
    check(e, bk['Bkeq_B'], bk['Bkeq_Q'], bk['Bkeq_k'], bk['Bkeq_Pk'])


@pytest.mark.parametrize('N,mas', [(64, 'CIC'), (33, 'PCS')])
def test_bk_vs_oracle(PKL, N, mas):
    rng = np.random.default_rng(N)
    L = 1000.0
    pos = (rng.random((N ** 3 * 2, 3)) * L).astype(np.float32)
    d = np.zeros((N, N, N), np.float32)
    O.MA(pos, d, L, mas)
    d = (d / np.float32(d.mean(dtype=np.float64)) - np.float32(1)).astype(np.float32)
    d = (d + 0.3 * d * d).astype(np.float32)    # some non-Gaussianity
    theta = np.linspace(0, np.pi, 7)
    r = PKL.Bk(d, L, 0.05, 0.09, theta, mas)
    o = O.Bk(d, L, 0.05, 0.09, theta, mas, 1)
    check(r, o.B, o.Q, o.k, o.Pk)


def test_bk_triangles_batch_equals_single_calls(PKL, bk):
    N, L, k1, k2 = bk['meta']
    d = bk['delta']
    # shells inside the grid's sphere |k| < kN (k/kF < 16): beyond it almost no
    # triangle closes and B = num/den is round-off in any implementation
    ks = np.linspace(0.03, 0.09, 5)
    tri = [(k, k, k) for k in ks]
    B, Q, P1, P2, P3 = PKL.Bk_triangles(d, L, tri, 'CIC')
    for j, k in enumerate(ks):
        o = O.Bk(d, L, k, k, np.array([2 * np.pi / 3]), 'CIC', 1)
        # k3 of the equilateral triangle rounds to k within 1 ulp: same shell
        assert abs(B[j] - o.B[0]) <= 1e-3 * abs(o.B[0]) + 1e-3 * np.abs(B).max()
        assert abs(P1[j] - o.Pk[0]) <= 1e-4 * o.Pk[0]


def test_reduced_side_equals_full_grid(PKL):
    """The shell fields are band-limited: reduced on the M^3 grid the plan picks (M > 3K)
    they give the same B as on the full grid (float32 sums over fewer cells: within
    1e-5 of the largest |B|) and the same shell powers (Parseval on the input grid)."""
    rng = np.random.default_rng(17)
    N, L = 96, 1000.0
    d = rng.standard_normal((N, N, N)).astype(np.float32)
    d = (d + 0.4 * d * d).astype(np.float32)
    tris = [(0.05, 0.08, 0.1), (0.05, 0.08, 0.12), (0.1, 0.1, 0.1), (0.06, 0.09, 0.07)]
    plan = PKL.BkPlan(N, L, tris, 'CIC')
    assert plan.side < N
    plan.run(d)
    B, Q, P1, P2, P3 = plan.result()
    full = PKL.BkPlan(N, L, tris, 'CIC', side=N)
    full.run(d)
    Bf, Qf, P1f, P2f, P3f = full.result()
    assert np.abs(B - Bf).max() <= 1e-5 * np.abs(Bf).max()
    np.testing.assert_allclose(P3, P3f, rtol=1e-12)
    o = O.Bk(d, L, 0.05, 0.08, np.array([np.arccos((0.1 ** 2 - 0.05 ** 2 - 0.08 ** 2) / (2 * 0.05 * 0.08))]),
             'CIC', 1)
    assert abs(B[0] - o.B[0]) <= 1e-3 * abs(o.B[0])


def test_bk_plan_graph_replay(PKL):
    """The whole bispectrum chain (R2C, deconvolution, shell fill, C2R, grouped sums)
    captured as one CUDA graph and replayed gives the eager result."""
    rng = np.random.default_rng(19)
    N, L = 64, 1000.0
    d = torch.from_numpy(rng.standard_normal((N, N, N)).astype(np.float32)).cuda()
    tris = [(0.05, 0.1, float(k)) for k in np.linspace(0.06, 0.14, 6)] + [(0.08, 0.08, 0.08)]
    plan = PKL.BkPlan(N, L, tris, 'PCS')
    plan.run(d)
    ref = plan.result()
    plan.capture(d)
    for _ in range(2):
        plan.replay()
    got = plan.result()
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


def test_fourier_groups_equal_real_space(PKL):
    """Triangles sharing (k1, k2) summed in Fourier space (the R2C of d_1 d_2 against each
    third shell's modes, Parseval) give the real-space triple sums: every group both
    ways, and the default mix, agree within float32 rounding (1e-5 of the largest |B|),
    numerators and the plan's indicator sums alike; the oracle pins one sweep."""
    rng = np.random.default_rng(23)
    N, L = 96, 1000.0
    d = rng.standard_normal((N, N, N)).astype(np.float32)
    d = (d + 0.4 * d * d).astype(np.float32)
    theta = np.linspace(0.2, 3.0, 9)
    k1, k2 = 0.05, 0.08
    k3 = np.sqrt((k2 * np.sin(theta)) ** 2 + (k2 * np.cos(theta) + k1) ** 2)
    tris = [(k1, k2, float(x)) for x in k3] + [(0.1, 0.1, 0.1), (0.06, 0.09, 0.07)]
    out = {}
    for method in ('real', 'fourier', 'auto'):
        plan = PKL.BkPlan(N, L, tris, 'CIC', method=method)
        plan.run(d)
        out[method] = plan.result()
    assert PKL.BkPlan(N, L, tris, 'CIC').n_fourier_groups == 1      # the sweep, in Fourier space
    Br = out['real'][0]
    for method in ('fourier', 'auto'):
        assert np.abs(out[method][0] - Br).max() <= 1e-5 * np.abs(Br).max(), method
        np.testing.assert_allclose(out[method][2], out['real'][2], rtol=1e-12)
    o = O.Bk(d, L, k1, k2, theta, 'CIC', 1)
    assert np.all(np.abs(out['auto'][0][:9] - o.B) <= 1e-3 * np.abs(o.B).max())
