"""smoothing_library.FT_filter / field_smoothing on the GPU against the reference's
outputs (tests/golden/smoothing_golden.npz)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def SL():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.smoothing_library as SL
    return SL


@pytest.fixture(scope='module')
def sg():
    return np.load(os.path.join(GOLDEN, 'smoothing_golden.npz'))


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('filt,R', [('Top-Hat', 100.0), ('Gaussian', 60.0)])
def test_smoothing_golden(SL, sg, N, filt, R):
    """Filter and smoothed field within 1e-5 of their largest values (cuFFT against
    the reference's float32 transforms, float64 sums in another order)."""
    t = filt.replace('-', '')
    fk = SL.FT_filter(1000.0, R, N, filt)
    gf = sg['filter_%s_%d' % (t, N)]
    assert np.abs(fk - gf).max() <= 1e-5 * np.abs(gf).max()
    sm = SL.field_smoothing(sg['field_%d' % N], gf)
    ref = sg['smoothed_%s_%d' % (t, N)]
    assert np.abs(sm - ref).max() <= 1e-5 * np.abs(ref).max()


def test_unknown_filter_raises(SL):
    with pytest.raises(ValueError):
        SL.FT_filter(1000.0, 10.0, 16, 'Box')
