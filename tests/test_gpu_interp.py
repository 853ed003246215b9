"""CIC interpolation (MAS_library.CIC_interp) and redshift-space positions
(redshift_space_library.pos_redshift_space) on the GPU against the reference's
outputs (tests/golden/interp_golden.npz) and the oracle."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mods():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.redshift_space_library as RSL
    return MASL, RSL


@pytest.fixture(scope='module')
def ig():
    return np.load(os.path.join(GOLDEN, 'interp_golden.npz'))


def test_cic_interp_matches_oracle_and_reference(mods, ig):
    """Same float operations in the same order as the oracle: bit-exact; the reference
    (built with -ffast-math) within 1e-6 of the field scale."""
    MASL, _ = mods
    pos, field = ig['interp_pos'], ig['interp_field']
    den = np.zeros(pos.shape[0], np.float32)
    MASL.CIC_interp(field, float(ig['interp_meta'][1]), pos, den)
    o = np.zeros_like(den)
    O.CIC_interp(field, float(ig['interp_meta'][1]), pos, o)
    np.testing.assert_array_equal(den, o)
    np.testing.assert_allclose(den, ig['interp_den'], rtol=0, atol=1e-6 * np.abs(field).max())


def test_cic_interp_large_tensor(mods):
    MASL, _ = mods
    rng = np.random.default_rng(3)
    N, L, n = 96, 500.0, 2_000_000
    field = rng.normal(size=(N, N, N)).astype(np.float32)
    pos = (rng.random((n, 3)) * L).astype(np.float32)
    den = torch.empty(n, device='cuda')
    MASL.CIC_interp(torch.from_numpy(field).cuda(), L, torch.from_numpy(pos).cuda(), den)
    o = np.zeros(n, np.float32)
    O.CIC_interp(field, L, pos, o)
    np.testing.assert_array_equal(den.cpu().numpy(), o)


@pytest.mark.parametrize('axis', [0, 1, 2])
def test_pos_redshift_space_bit_exact(mods, ig, axis):
    _, RSL = mods
    L, H, z = (float(x) for x in ig['rsd_meta'])
    p = ig['rsd_pos'].copy()
    RSL.pos_redshift_space(p, ig['rsd_vel'], L, H, z, axis)
    np.testing.assert_array_equal(p, ig['rsd_out_axis%d' % axis])
    t = torch.from_numpy(ig['rsd_pos'].copy()).cuda()
    RSL.pos_redshift_space(t, torch.from_numpy(ig['rsd_vel']).cuda(), L, H, z, axis)
    np.testing.assert_array_equal(t.cpu().numpy(), ig['rsd_out_axis%d' % axis])


def test_pos_redshift_space_far_outside(mods):
    """Displacements of several box lengths: the C remainder keeps the sign of
    pos + BoxSize, exactly like the oracle (and the reference)."""
    _, RSL = mods
    rng = np.random.default_rng(9)
    L = 100.0
    pos = (rng.random((10000, 3)) * L).astype(np.float32)
    vel = (rng.normal(size=(10000, 3)) * 2e4).astype(np.float32)
    a = pos.copy()
    RSL.pos_redshift_space(a, vel, L, 100.0, 0.0, 1)
    b = pos.copy()
    O.pos_redshift_space(b, vel, L, 100.0, 0.0, 1)
    np.testing.assert_array_equal(a, b)
