"""Batched realizations (one persistent deposit launch for many uneven particle sets)
must reproduce the one-at-a-time path (pipeline.ParticlePk) realization by
realization: Nmodes bit-exact, P(k) l=0,2,4 within rtol 1e-4 on the scale of
(2l+1) P0 (the paths accumulate the deposits differently: float32 atomics, or
10.22 fixed point per bin)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mods(tmp_path_factory):
    import pylians_gb300.build as b
    b.build()
    os.environ['PYL_AUTOTUNE_CACHE'] = str(tmp_path_factory.mktemp('tune') / 'autotune.json')
    from pylians_gb300 import batch, pipeline
    return batch, pipeline


def _check(a, b):
    np.testing.assert_array_equal(a.Nmodes3D, b.Nmodes3D)
    np.testing.assert_array_equal(a.Nmodes2D, b.Nmodes2D)
    # l = 0, 2, 4 sums are finalised with factors 1, 5, 9 (Pk_library.pyx:416-418), so
    # the noise scale of column l is (2l+1) P0
    p0 = np.abs(b.Pk[:, 0:1]) * np.array([[1.0, 5.0, 9.0]])
    assert np.all(np.abs(a.Pk - b.Pk) <= 1e-4 * p0 + 1e-12 * p0.max())
    np.testing.assert_allclose(a.Pk1D, b.Pk1D, rtol=1e-4, atol=1e-6 * np.abs(b.Pk1D).max())


@pytest.mark.parametrize('method', ['tiled', 'atomic'])
def test_batch_matches_one_at_a_time(mods, method):
    batch, pipeline = mods
    specs = batch.random_specs(10, seed=3, dims_choices=(32, 48, 64), n_range=(20000, 300000))
    specs[0]['MAS'] = 'NGP'
    gen = torch.Generator(device='cuda')
    gen.manual_seed(7)
    L = 1000.0
    pos = [torch.rand((s['n'], 3), generator=gen, device='cuda') * L for s in specs]
    B = batch.RealizationBatch(specs, L, axis=2, method=method)
    B.step(pos)
    res = B.results()
    for s, p, r in zip(specs, pos, res):
        one = pipeline.ParticlePk(s['dims'], L, s['MAS'], axis=2, interlaced=s['interlaced'],
                                  max_particles=s['n'])
        one.step(p)
        _check(r, one.result())
    # the whole batch as one CUDA graph
    B.capture(pos)
    B.replay()
    for a, b in zip(B.results(), res):
        _check(a, b)


def test_autotune_cache_written(mods):
    batch, _ = mods
    from pylians_gb300 import autotune
    k = autotune.item_size(48, 50000, 'TSC', True)
    assert k in autotune.ITEM_CANDIDATES
    assert os.path.exists(os.environ['PYL_AUTOTUNE_CACHE'])
    assert autotune.item_size(48, 50000, 'TSC', True, tune=False) == k
