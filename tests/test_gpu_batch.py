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


@pytest.mark.parametrize('axis', [0, 1, 2])
@pytest.mark.parametrize('inter', [False, True])
def test_pk_bin_batch_equals_one_field_calls(mods, axis, inter):
    """pyl_pk_bin_batch bins each item with the one-field call's CTA partition and
    float32 partial sums: item by item the sums agree with pyl_pk_bin to float32
    rounding (the partial sums' float atomics run in no fixed order in either)."""
    import ctypes
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr
    from pylians_gb300.batch import PK_ITEM_DT
    L = _lib.load()
    dims, n = 48, 5
    gen = torch.Generator(device='cuda')
    gen.manual_seed(11 + axis + 3 * inter)
    shape = (n, dims, dims, dims // 2 + 1)
    dk = torch.complex(torch.randn(shape, generator=gen, device='cuda'), torch.randn(shape, generator=gen, device='cuda'))
    dk2 = torch.complex(torch.randn(shape, generator=gen, device='cuda'), torch.randn(shape, generator=gen, device='cuda'))
    mas = [1, 2, 3, 4, 2]
    slen = L.pyl_pk_sums_len(dims, 1)
    one = torch.zeros((n, slen), dtype=torch.float64, device='cuda')
    ws = torch.empty(max(L.pyl_pk_workspace_size(dims, 1, axis), 1), dtype=torch.uint8, device='cuda')
    for i in range(n):
        mp = (ctypes.c_int * 1)(mas[i])
        _lib.call('pyl_pk_bin', ptr(dk[i]), ptr(dk2[i]) if inter else None, 1, dk[0].numel(), dims, axis, mp,
                  ptr(one[i]), ptr(ws), ws.numel(), None)
    many = torch.full((n, slen), 7.0, dtype=torch.float64, device='cuda')    # zeroed by the call
    rec = np.zeros(n, dtype=PK_ITEM_DT)
    for i in range(n):
        rec[i] = (dk[i].data_ptr(), dk2[i].data_ptr() if inter else 0, many[i].data_ptr(), mas[i], 0)
    table = torch.from_numpy(rec.view(np.uint8)).cuda()
    nb = L.pyl_pk_bin_batch_workspace_size(dims, n, axis, int(inter))
    wsb = torch.empty(nb, dtype=torch.uint8, device='cuda')
    _lib.call('pyl_pk_bin_batch', ptr(table), n, dims, axis, int(inter), ptr(wsb), nb, None)
    a, b = many.cpu().numpy(), one.cpu().numpy()
    for i in range(n):
        np.testing.assert_allclose(a[i], b[i], rtol=1e-5, atol=1e-6 * np.abs(b[i]).max(), err_msg='item %d' % i)


@pytest.mark.parametrize('axis', [0, 2])
def test_pk_bin_batch_coarsened_partition(mods, axis):
    """With many items the batched launch gives each CTA more rows than a one-field call
    (200 interlaced 128^3 fields: 512 representatives a CTA along axis 2, one row chunk
    per plane along axis 0); the sums still agree with pyl_pk_bin item by item to
    float32 rounding."""
    import ctypes
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr
    from pylians_gb300.batch import PK_ITEM_DT
    L = _lib.load()
    dims, n = 128, 200
    gen = torch.Generator(device='cuda')
    gen.manual_seed(31 + axis)
    shape = (n, dims, dims, dims // 2 + 1)
    dk = torch.complex(torch.randn(shape, generator=gen, device='cuda'), torch.randn(shape, generator=gen, device='cuda'))
    dk2 = torch.complex(torch.randn(shape, generator=gen, device='cuda'), torch.randn(shape, generator=gen, device='cuda'))
    slen = L.pyl_pk_sums_len(dims, 1)
    many = torch.zeros((n, slen), dtype=torch.float64, device='cuda')
    rec = np.zeros(n, dtype=PK_ITEM_DT)
    for i in range(n):
        rec[i] = (dk[i].data_ptr(), dk2[i].data_ptr(), many[i].data_ptr(), 1 + i % 4, 0)
    table = torch.from_numpy(rec.view(np.uint8)).cuda()
    nb = L.pyl_pk_bin_batch_workspace_size(dims, n, axis, 1)
    wsb = torch.empty(nb, dtype=torch.uint8, device='cuda')
    _lib.call('pyl_pk_bin_batch', ptr(table), n, dims, axis, 1, ptr(wsb), nb, None)
    one = torch.zeros(slen, dtype=torch.float64, device='cuda')
    ws = torch.empty(max(L.pyl_pk_workspace_size(dims, 1, axis), 1), dtype=torch.uint8, device='cuda')
    a = many.cpu().numpy()
    for i in range(0, n, 37):
        mp = (ctypes.c_int * 1)(1 + i % 4)
        _lib.call('pyl_pk_bin', ptr(dk[i]), ptr(dk2[i]), 1, dk[0].numel(), dims, axis, mp, ptr(one), ptr(ws),
                  ws.numel(), None)
        b = one.cpu().numpy()
        np.testing.assert_allclose(a[i], b, rtol=1e-5, atol=1e-6 * np.abs(b).max(), err_msg='item %d' % i)
