"""GPU parity of the bispectrum (shell fill + batched C2R + triple-product
reduction) against the reference's golden outputs and the oracle.

Tolerances: P(k_i) rtol 1e-4; B and Q within 1e-3 of max|B| / max|Q| over the
triangle set (B sums products of both signs, so its error is measured against
the largest bispectrum of the set, not bin by bin).
"""
import os

import numpy as np
import pytest

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
