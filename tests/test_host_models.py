"""Host-side numerics of the learned correction and the batch workload, no GPU:
the network's feature layout, the (slope, shot level) estimate from a coarse
monopole (exact on a noise-free power law plus shot noise), and the seeded
uneven-realization specs of the batch benchmark."""
import math

import numpy as np
import pytest

from pylians_gb300 import batch, learned


def test_feature_layout():
    x = learned.features([0.1, 0.5], 'TSC', -2.0, 0.6)
    assert x.dtype == np.float32 and x.shape == (2, 4)
    np.testing.assert_allclose(x[:, 0], [0.1, 0.5], rtol=1e-7)
    assert (x[:, 1] == 0).all()                          # MAS index - 3
    assert (x[:, 2] == np.float32(-0.5)).all()           # slope + 1.5
    assert (x[:, 3] == np.float32(0.2)).all()            # shot level / 3
    assert learned.features([0.2], 'CIC', -1.5, 0.0)[0, 1] == -1


@pytest.mark.parametrize('slope,nbar', [(-1.5, 1e-3), (-2.5, 1e-1), (-0.5, 1.0)])
def test_feature_estimate_recovers_a_power_law(slope, nbar):
    kN = 0.8
    k = np.linspace(0.006, 0.99 * kN, 140)
    amp = 50.0
    Pk0 = amp * k ** slope + 1.0 / nbar
    b, level = learned.estimate_features(k, Pk0, kN, nbar)
    assert b == pytest.approx(slope, abs=1e-9)
    assert level == pytest.approx(math.log10((1.0 / nbar) / (amp * kN ** slope)), abs=1e-9)


def test_feature_estimate_needs_power_above_shot_noise():
    k = np.linspace(0.01, 0.8, 50)
    with pytest.raises(ValueError):
        learned.estimate_features(k, np.full_like(k, 10.0), 0.8, 0.1)   # P == 1/nbar everywhere


def test_random_specs_are_seeded_and_in_range():
    a = batch.random_specs(64, seed=3)
    assert a == batch.random_specs(64, seed=3)
    assert a != batch.random_specs(64, seed=4)
    for s in a:
        assert s['dims'] in (64, 128, 192, 256)
        assert 100000 <= s['n'] <= 17000000
        assert s['MAS'] in ('CIC', 'TSC', 'PCS')
        assert isinstance(s['interlaced'], bool)
    assert len({s['dims'] for s in a}) > 1 and len({s['interlaced'] for s in a}) == 2
