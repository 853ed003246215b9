"""Correlation function (Pk_library.Xi) and correct_MAS on the GPU against the
reference's outputs (tests/golden/xi_golden.npz) and the oracle."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def PKL():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.Pk_library as PKL
    return PKL


@pytest.fixture(scope='module')
def xg():
    return np.load(os.path.join(GOLDEN, 'xi_golden.npz'))


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('axis', [0, 2])
def test_xi_golden(PKL, xg, N, axis):
    """Mode counts and mean separations exact; xi l=0,2,4 within 1e-5 of the largest
    |xi_0| (float32 FFTs and sums against the reference's float64 loop)."""
    r = PKL.Xi(xg['delta_%d' % N], 1000.0, 'CIC', axis)
    np.testing.assert_array_equal(r.Nmodes3D, xg['Xi_%d_axis%d_Nmodes3D' % (N, axis)])
    np.testing.assert_allclose(r.r3D, xg['Xi_%d_axis%d_r3D' % (N, axis)], rtol=1e-12)
    ref = xg['Xi_%d_axis%d_xi' % (N, axis)]
    assert np.abs(r.xi - ref).max() <= 1e-5 * np.abs(ref[:, 0]).max()


def test_xi_larger_grid_vs_oracle(PKL):
    rng = np.random.default_rng(12)
    N = 96
    d = rng.standard_normal((N, N, N)).astype(np.float32)
    r = PKL.Xi(torch.from_numpy(d).cuda(), 500.0, 'TSC', 1)
    o = O.Xi(d, 500.0, 'TSC', 1)
    np.testing.assert_array_equal(r.Nmodes3D, o.Nmodes3D)
    assert np.abs(r.xi - o.xi).max() <= 1e-5 * np.abs(o.xi[:, 0]).max()


@pytest.mark.parametrize('N', [32, 15])
def test_correct_mas_golden(PKL, xg, N):
    """The reference's half-corrected kz = 0, N/2 planes included: within 1e-5 of the
    field's largest value (cuFFT against scipy float32 transforms)."""
    d = xg['delta_%d' % N]
    out = PKL.correct_MAS(d, 1000.0, 'CIC')
    ref = xg['correct_MAS_%d' % N]
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()
