"""The tiled deposit with every particle of the call in one 32^3 bin: 12M particles
inside one bin of a 768^3 grid (79,000 per histogram chunk in that bin, 366 per cell
on average, clumped input taking the coherent one-pass placement).  The tiled grid
must equal the atomic strategy's, and both must hold every particle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_clumped_bin_matches_atomic():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr
    L_ = _lib.load()
    N, box, n = 768, 768.0, 12_000_000
    g = torch.Generator(device='cuda')
    g.manual_seed(21)
    # cells 100..127 on each axis: one bin (96..127) holds every particle
    pos = (100.0 + 27.0 * torch.rand((n, 3), generator=g, device='cuda')).contiguous()
    out = {}
    for strategy in (1, 2):                       # ATOMIC, TILED
        grid = torch.zeros((N, N, N), device='cuda')
        nbytes = L_.pyl_ma_workspace_size(n, 3, N, 2, strategy, 0)
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device='cuda')
        _lib.call('pyl_ma', ptr(pos), None, n, 3, ptr(grid), None, N, box, 2, strategy, 0, ptr(ws), nbytes, None)
        torch.cuda.synchronize()
        out[strategy] = grid[96:129, 96:129, 96:129].cpu().numpy()
        assert abs(float(grid.sum(dtype=torch.float64)) - n) < 1e-4 * n
        del grid, ws
        torch.cuda.empty_cache()
    ref = out[1]
    assert np.abs(out[2] - ref).max() <= 1e-5 * np.abs(ref).max()
