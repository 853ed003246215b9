"""Calls with more particles than the tiled pass limit (pyl_ma_set_pass_limit, by default
2^32 - 4096, so 2048^3 particles take two passes) run the tiled deposit over consecutive
slices.  The limit is lowered here so that 700,000 particles take four passes; each
result must equal the one-pass result: NGP counts into an integer-valued grid exactly,
the rest within float32 rounding of the per-pass sums (each pass adds its bin sums,
rounded to float32, to the grid; the overdensity adds scaled counts to -1).  Covered: pyl_ma (accumulating into a non-zero grid), the overdensity with the
fill pass and with the owned-cell write-out (first pass stores -1 + value, the rest
accumulate), weights, interlacing, and the redshift-space shift fused into each pass."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TILED = 2
N_PART, LIMIT, DIMS, L = 700_000, 196 * 1024, 64, 1000.0


@pytest.fixture(scope='module')
def lib():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import _lib
    yield _lib
    _lib.call('pyl_ma_set_pass_limit', -1)
    _lib.call('pyl_ma_set_thresholds', -1, -1.0)


def _data(seed, weighted):
    g = torch.Generator(device='cuda')
    g.manual_seed(seed)
    pos = torch.rand((N_PART, 3), generator=g, device='cuda') * L
    w = torch.rand(N_PART, generator=g, device='cuda') + 0.5 if weighted else None
    vel = (torch.rand((N_PART, 3), generator=g, device='cuda') - 0.5) * 600.0
    return pos, w, vel


def _call(_lib, kind, pos, w, mas, inter, limit, base=None, vel=None):
    from pylians_gb300._device import ptr
    L_ = _lib.load()
    _lib.call('pyl_ma_set_pass_limit', limit)
    try:
        nbytes = L_.pyl_ma_workspace_size(N_PART, 3, DIMS, mas, TILED, int(inter))
        ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
        grids = torch.zeros((2, DIMS, DIMS, DIMS), device='cuda')
        if base is not None:
            grids.copy_(base)
        g2 = ptr(grids[1]) if inter else None
        if kind == 'ma':
            _lib.call('pyl_ma', ptr(pos), ptr(w), N_PART, 3, ptr(grids[0]), g2, DIMS, L, mas, TILED, 0,
                      ptr(ws), nbytes, None)
        elif kind == 'od':
            _lib.call('pyl_ma_overdensity', ptr(pos), ptr(w), N_PART, ptr(grids[0]), g2, DIMS, L, mas, TILED,
                      ptr(ws), nbytes, None)
        else:
            _lib.call('pyl_ma_overdensity_rsd', ptr(pos), ptr(vel), ptr(w), N_PART, ptr(grids[0]), g2, DIMS, L,
                      mas, TILED, 100.0, 0.5, 1, ptr(ws), nbytes, None)
        torch.cuda.synchronize()
    finally:
        _lib.call('pyl_ma_set_pass_limit', -1)
    return grids.cpu().numpy()


def _close(a, b, exact):
    if exact:
        np.testing.assert_array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= 4e-6 * np.abs(b).max(), np.abs(a - b).max()


@pytest.mark.parametrize('owned', [False, True])
@pytest.mark.parametrize('mas', [1, 2, 3])
@pytest.mark.parametrize('kind', ['ma', 'od'])
def test_passes_equal_one_pass(lib, kind, mas, owned):
    lib.call('pyl_ma_set_thresholds', DIMS if owned else -1, -1.0)
    try:
        pos, w, _ = _data(3 + mas, weighted=(mas == 3))
        # MA accumulates: an integer-valued starting grid keeps NGP sums exact
        base = torch.floor(torch.rand((2, DIMS, DIMS, DIMS), device='cuda') * 5) if kind == 'ma' else None
        one = _call(lib, kind, pos, w, mas, True, -1, base)
        many = _call(lib, kind, pos, w, mas, True, LIMIT, base)
    finally:
        lib.call('pyl_ma_set_thresholds', -1, -1.0)
    _close(many, one, mas == 1 and kind == 'ma')
    if kind == 'od' and mas != 3:
        # each grid of the overdensity sums to ~0 (mean N / dims^3 from the whole call)
        assert abs(float(many[0].sum(dtype=np.float64))) < 1e-3 * DIMS ** 3


def test_passes_rsd_fused(lib):
    lib.call('pyl_ma_set_thresholds', DIMS, -1.0)
    try:
        pos, _, vel = _data(11, weighted=False)
        p1, p2 = pos.clone(), pos.clone()
        one = _call(lib, 'rsd', p1, None, 2, True, -1, vel=vel)
        many = _call(lib, 'rsd', p2, None, 2, True, LIMIT, vel=vel)
    finally:
        lib.call('pyl_ma_set_thresholds', -1, -1.0)
    # every pass shifts its own slice in place, as the one-pass call shifts all
    assert torch.equal(p1, p2)
    _close(many, one, False)
