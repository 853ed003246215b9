"""2D maps: Pk_plane and XPk_plane on the GPU against the reference's outputs
(tests/golden/plane_golden.npz) and the oracle."""
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
def pg():
    return np.load(os.path.join(GOLDEN, 'plane_golden.npz'))


@pytest.mark.parametrize('N', [64, 45])
def test_pk_plane_golden(PKL, pg, N):
    """Mode counts exact, k rtol 1e-12, spectra rtol 1e-5 (cuFFT vs float32 FFTs)."""
    a, b = pg['map1_%d' % N], pg['map2_%d' % N]
    r = PKL.Pk_plane(a, 1000.0, 'CIC')
    np.testing.assert_array_equal(r.Nmodes, pg['Pkplane_%d_Nmodes' % N])
    np.testing.assert_allclose(r.k, pg['Pkplane_%d_k' % N], rtol=1e-12)
    np.testing.assert_allclose(r.Pk, pg['Pkplane_%d_Pk' % N], rtol=1e-5)
    x = PKL.XPk_plane(a, b, 1000.0, 'CIC', 'TSC')
    np.testing.assert_array_equal(x.Nmodes, pg['XPkplane_%d_Nmodes' % N])
    np.testing.assert_allclose(x.Pk, pg['XPkplane_%d_Pk' % N], rtol=1e-5)
    sc = np.sqrt(np.abs(pg['XPkplane_%d_Pk' % N][:, 0] * pg['XPkplane_%d_Pk' % N][:, 1]))
    assert np.all(np.abs(x.XPk - pg['XPkplane_%d_XPk' % N]) <= 1e-5 * sc)


def test_pk_plane_large_vs_oracle(PKL):
    rng = np.random.default_rng(6)
    N = 1024
    a = rng.standard_normal((N, N)).astype(np.float32)
    r = PKL.Pk_plane(torch.from_numpy(a).cuda(), 500.0, 'PCS')
    o = O.Pk_plane(a, 500.0, 'PCS')
    np.testing.assert_array_equal(r.Nmodes, o.Nmodes)
    np.testing.assert_allclose(r.Pk, o.Pk, rtol=1e-5)


def test_plane_mode_check_and_size_check(PKL):
    with pytest.raises(ValueError):
        PKL.XPk_plane(np.zeros((16, 16), np.float32), np.zeros((8, 8), np.float32), 1.0)
