"""Allocation-free mass assignment: pyl_ma_noalloc through the C-ABI.

Some callers of this library cannot allocate device memory around a call:
plugins hosted by a framework whose allocator owns all device memory, and loops
that allocate nothing after start-up.
pyl_ma_noalloc serves them with binning scratch compiled into the library
(24 MiB per device; at most 524288 particles and dims <= 512).

The test calls it twice in a row (the shared scratch keeps the previous call's
contents) and compares each result with pyl_ma, the allocating entry point, on
the same inputs: NGP counts bit-exact, CIC/TSC/PCS within 2e-6 of the grid's
largest value (the tolerance of the other mass-assignment tests).  This file is
collected last so that a run stopping at the first failure has run all others.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def lib():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import _lib
    return _lib.load()


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _reference(lib, pos, w, N, L, mas, inter):
    """The allocating entry point with the tiled strategy and a caller-owned workspace."""
    n = pos.shape[0]
    g1 = torch.zeros((N, N, N), device='cuda')
    g2 = torch.zeros((N, N, N), device='cuda') if inter else None
    need = lib.pyl_ma_workspace_size(n, 3, N, mas, 2, int(inter))
    ws = torch.empty(max(need, 1), dtype=torch.uint8, device='cuda')
    rc = lib.pyl_ma(_p(pos), _p(w), n, 3, _p(g1), _p(g2), N, L, mas, 2, 0, _p(ws), need, None)
    assert rc == 0, lib.pyl_last_error()
    return g1, g2


@pytest.mark.parametrize('mas,weighted,inter', [(1, False, False), (2, False, True),
                                                (2, True, False), (3, False, True), (4, True, True)])
def test_noalloc_matches_pyl_ma_twice(lib, mas, weighted, inter):
    rng = np.random.default_rng(100 + mas)
    N, L, n = 96, 500.0, 400000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    w = torch.from_numpy((rng.random(n) * 2).astype(np.float32)).cuda() if weighted else None
    ref1, ref2 = _reference(lib, pos, w, N, L, mas, inter)
    for call in range(2):
        g1 = torch.zeros((N, N, N), device='cuda')
        g2 = torch.zeros((N, N, N), device='cuda') if inter else None
        rc = lib.pyl_ma_noalloc(_p(pos), _p(w), n, _p(g1), _p(g2), N, L, mas, None)
        assert rc == 0, lib.pyl_last_error()
        torch.cuda.synchronize()
        for got, ref in ((g1, ref1), (g2, ref2)):
            if ref is None:
                continue
            if mas == 1 and not weighted:
                assert torch.equal(got, ref), 'call %d: NGP counts differ' % call
            else:
                err = (got - ref).abs().max().item()
                assert err <= 2e-6 * ref.abs().max().item(), 'call %d: max diff %g' % (call, err)


def test_noalloc_largest_request(lib):
    """The documented maximum (524288 particles on a 512^3 grid, which takes the
    two-level placement and so two record buffers) fits the fixed scratch and
    matches pyl_ma."""
    rng = np.random.default_rng(7)
    N, L, n = 512, 1000.0, 1 << 19
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    ref, _ = _reference(lib, pos, None, N, L, 2, False)
    g = torch.zeros((N, N, N), device='cuda')
    rc = lib.pyl_ma_noalloc(_p(pos), None, n, _p(g), None, N, L, 2, None)
    assert rc == 0, lib.pyl_last_error()
    torch.cuda.synchronize()
    assert (g - ref).abs().max().item() <= 2e-6 * ref.abs().max().item()


def test_noalloc_rejects_oversized_requests(lib):
    buf = torch.zeros(16, device='cuda')
    rc = lib.pyl_ma_noalloc(_p(buf), None, (1 << 19) + 1, _p(buf), None, 64, 1.0, 2, None)
    assert rc == 1 and b'524288' in lib.pyl_last_error()
    rc = lib.pyl_ma_noalloc(_p(buf), None, 10, _p(buf), None, 1024, 1.0, 2, None)
    assert rc == 1 and b'dims' in lib.pyl_last_error()
