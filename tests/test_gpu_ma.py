"""GPU parity of mass assignment (pyl_ma through the C-ABI) against the reference's
golden grids and the oracle.

Tolerances: NGP without weights bit-exact (integer counts, any order);
NGP with weights and CIC/TSC/PCS: |gpu - ref| <= 2e-6 * max|ref| per cell (the
reference and the GPU add the same float32 terms in different orders).
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
import oracle as O

pytestmark = pytest.mark.gpu
MAS_LIST = ['NGP', 'CIC', 'TSC', 'PCS']
STRATS = ['atomic', 'tiled', 'sorted']


@pytest.fixture(scope='module')
def MASL():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.MAS_library as M
    return M


@pytest.fixture(scope='module')
def ma():
    return np.load(os.path.join(GOLDEN, 'ma_golden.npz'))


def close(a, b, exact, tol=2e-6):
    if exact:
        np.testing.assert_array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-30), np.abs(a - b).max()


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('tag', ['', 'W'])
@pytest.mark.parametrize('strategy', STRATS)
def test_ma_golden_3d(MASL, ma, mas, tag, strategy):
    pos, W = ma['grid_pos'], ma['grid_W']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    d = np.zeros((N, N, N), np.float32)
    MASL.MA(pos, d, L, mas, W if tag else None, strategy=strategy)
    close(d, ma['MA3D_%s%s' % (mas, tag)], exact=(mas == 'NGP' and not tag))


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('tag', ['', 'W'])
def test_ma_golden_2d(MASL, ma, mas, tag):
    """2D grids take S^3 adds per particle into dims^2 cells (about 330 float adds per
    cell here), so two summation orders differ by tens of ulps: tolerance 1e-5."""
    pos, W = ma['grid_pos'], ma['grid_W']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    d2 = np.zeros((N, N), np.float32)
    MASL.MA(np.ascontiguousarray(pos[:, :2]), d2, L, mas, W if tag else None)
    close(d2, ma['MA2D_%s%s' % (mas, tag)], exact=(mas == 'NGP' and not tag), tol=1e-5)


@pytest.mark.parametrize('mas', MAS_LIST)
def test_ma_c_path_golden(MASL, ma, mas):
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    c = np.zeros((N, N, N), np.float32)
    getattr(MASL, mas + 'c3D')(pos, c, L, 4)
    close(c, ma['MASc3D_%s' % mas], exact=(mas == 'NGP'))


@pytest.mark.parametrize('mas', MAS_LIST)
def test_ma_conservation(MASL, ma, mas):
    """Test/test_MAS.py:10-84 on the GPU: sum(grid)/N == 1."""
    pos = ma['conservation_pos']
    for W in (None, np.full(pos.shape[0], 3.0, np.float32)):
        d = np.zeros((64, 64, 64), np.float32)
        MASL.MA(pos, d, 1.0, mas, W=W)
        norm = pos.shape[0] * (3.0 if W is not None else 1.0)
        s = np.sum(d, dtype=np.float64) / norm
        assert round(s - 1.0, 20 if mas == 'NGP' else 8) == 0


def test_ma_accumulates(MASL, ma):
    """MA adds into the grid it is given.  The atomic path adds 1.0 per particle, so it is
    bit-exact on any base grid; the tiled path adds each tile's integer count at once, so it
    is bit-exact on integer-valued grids (zeros, or counts from earlier files, the reference's
    multi-file pattern) and within one ulp per cell otherwise."""
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    d = ma['accum_base'].copy()
    MASL.MA(pos, d, L, 'NGP', strategy='atomic')
    np.testing.assert_array_equal(d, ma['accum_NGP'])
    t = torch.from_numpy(ma['accum_base'].copy()).cuda()
    MASL.MA(torch.from_numpy(pos).cuda(), t, L, 'NGP', strategy='tiled')
    close(t.cpu().numpy(), ma['accum_NGP'], False, 2e-7)
    base = np.floor(ma['accum_base'] * 3).astype(np.float32)
    o = base.copy()
    O.MA(pos, o, L, 'NGP')
    t = torch.from_numpy(base.copy()).cuda()
    MASL.MA(torch.from_numpy(pos).cuda(), t, L, 'NGP', strategy='tiled')
    np.testing.assert_array_equal(t.cpu().numpy(), o)


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('strategy', STRATS)
def test_ma_interlaced_vs_oracle(MASL, mas, strategy):
    rng = np.random.default_rng(42)
    N, L, n = 48, 500.0, 300000
    pos = (rng.random((n, 3)) * L).astype(np.float32)
    W = (rng.random(n) * 2).astype(np.float32)
    g1 = torch.zeros((N, N, N), device='cuda')
    g2 = torch.zeros((N, N, N), device='cuda')
    MASL.MA(torch.from_numpy(pos).cuda(), g1, L, mas, torch.from_numpy(W).cuda(),
            interlaced=g2, strategy=strategy)
    o1 = np.zeros((N, N, N), np.float32)
    o2 = np.zeros((N, N, N), np.float32)
    O.MA(pos, o1, L, mas, W)
    O.MA((pos + np.float32(0.5 * L / N)).astype(np.float32), o2, L, mas, W)
    close(g1.cpu().numpy(), o1, False, 5e-6)
    close(g2.cpu().numpy(), o2, False, 5e-6)


@pytest.mark.parametrize('mas', MAS_LIST)
def test_tiled_matches_atomic_large(MASL, mas):
    """A grid larger than the tile with ragged tiles (dims not a multiple of 16/32)."""
    rng = np.random.default_rng(7)
    N, L, n = 200, 1000.0, 2_000_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    a = torch.zeros((N, N, N), device='cuda')
    b = torch.zeros((N, N, N), device='cuda')
    MASL.MA(pos, a, L, mas, strategy='atomic')
    MASL.MA(pos, b, L, mas, strategy='tiled')
    if mas == 'NGP':
        assert torch.equal(a, b)
    else:
        assert (a - b).abs().max().item() <= 2e-6 * a.abs().max().item()
    assert abs(b.double().sum().item() - n) <= 1e-6 * n


def test_ngp_bit_exact_config1(MASL):
    """128^3 particles on a 128^3 grid (the small CPU-runnable configuration): NGP
    counts equal the oracle's bit for bit."""
    rng = np.random.default_rng(1)
    N, L = 128, 1000.0
    pos = (rng.random((N ** 3, 3)) * L).astype(np.float32)
    o = np.zeros((N, N, N), np.float32)
    O.MA(pos, o, L, 'NGP', threads=os.cpu_count() or 1)
    for strategy in STRATS:
        g = torch.zeros((N, N, N), device='cuda')
        MASL.MA(torch.from_numpy(pos).cuda(), g, L, 'NGP', strategy=strategy)
        np.testing.assert_array_equal(g.cpu().numpy(), o)


def test_edge_positions(MASL):
    """Empty input, positions on cell edges, at 0, at L, slightly negative and beyond L:
    every index wraps periodically, like the oracle (the reference writes out of bounds
    for the negative ones)."""
    N, L = 16, 1.0
    h = np.float32(L / N)
    pts = np.array([[0, 0, 0], [h, 2 * h, 3 * h], [0.5 * h, 1.5 * h, 2.5 * h], [L, L, L],
                    [np.nextafter(np.float32(L), np.float32(0))] * 3, [-1e-3, -0.2 * h, -0.7 * h],
                    [L + 0.3 * h, 2 * L, 3.3 * L]], np.float32)
    for mas in MAS_LIST:
        for strategy in STRATS:
            g = np.zeros((N, N, N), np.float32)
            MASL.MA(np.zeros((0, 3), np.float32), g, L, mas, strategy=strategy)
            assert not g.any()
            MASL.MA(pts, g, L, mas, strategy=strategy)
            o = np.zeros((N, N, N), np.float32)
            O.MA(pts, o, L, mas)
            close(g, o, mas == 'NGP', 1e-6)


def test_bad_input_raises(MASL):
    with pytest.raises(ValueError):
        MASL.MA(np.zeros((4, 3), np.float64), np.zeros((8, 8, 8), np.float32), 1.0, 'CIC')
    with pytest.raises(ValueError):
        MASL.MA(np.zeros((4, 2), np.float32), np.zeros((8, 8, 8), np.float32), 1.0, 'CIC')
    with pytest.raises(ValueError):
        MASL.MA(np.zeros((4, 3), np.float32), np.zeros((8, 8, 8), np.float32), 1.0, 'XYZ')


@pytest.mark.parametrize('mas', ['NGP', 'CIC'])
def test_two_level_placement_matches_atomic(MASL, mas):
    """Grids with more than 1024 tiles place randomly ordered particles in two levels
    (coarse blocks, then tiles); 544^3 has 17^3 tiles in ragged 4^3 coarse blocks.  Weighted and
    unweighted, plain and interlaced grids must equal the atomic strategy's."""
    rng = np.random.default_rng(11)
    N, L, n = 544, 1000.0, 3_000_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    w = torch.from_numpy((rng.random(n) * 2).astype(np.float32)).cuda()
    for W in (None, w):
        a1 = torch.zeros((N, N, N), device='cuda'); a2 = torch.zeros((N, N, N), device='cuda')
        b1 = torch.zeros((N, N, N), device='cuda'); b2 = torch.zeros((N, N, N), device='cuda')
        MASL.MA(pos, a1, L, mas, W, interlaced=a2, strategy='atomic')
        MASL.MA(pos, b1, L, mas, W, interlaced=b2, strategy='tiled')
        for a, b in ((a1, b1), (a2, b2)):
            if mas == 'NGP' and W is None:
                assert torch.equal(a, b)
            else:
                assert (a - b).abs().max().item() <= 2e-6 * a.abs().max().item()
        del a1, a2, b1, b2


@pytest.mark.parametrize('N', [384, 544, 1024])
def test_coherent_placement_matches_atomic(MASL, N):
    """Particles in spatial order (a jittered lattice, z fastest) share their
    predecessor's bin, so on grids of more than 1024 bins the tiled strategy places
    them straight to their bins in one pass (384^3, 544^3; 1024^3 also stores its
    own cells and passes halos on).  Half-shuffled input (coherence near 1/2) takes
    the two-level sorts.  All must equal the atomic strategy."""
    rng = np.random.default_rng(13)
    L, M = 1000.0, 160
    g = (np.arange(M, dtype=np.float32) + 0.5) * np.float32(L / M)
    q = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    q = (q + (rng.random(q.shape) - 0.5).astype(np.float32) * np.float32(L / M)) % np.float32(L)
    q = q.astype(np.float32)
    half = q.copy()
    idx = rng.permutation(len(q))[: len(q) // 2]
    half[np.sort(idx)] = half[idx]
    w = torch.from_numpy((rng.random(len(q)) * 2).astype(np.float32)).cuda()
    for arr in (q, half):
        pos = torch.from_numpy(arr).cuda()
        for mas, W in (('NGP', None), ('CIC', None), ('TSC', w)):
            a1 = torch.zeros((N, N, N), device='cuda'); a2 = torch.zeros((N, N, N), device='cuda')
            b1 = torch.zeros((N, N, N), device='cuda'); b2 = torch.zeros((N, N, N), device='cuda')
            MASL.MA(pos, a1, L, mas, W, interlaced=a2, strategy='atomic')
            MASL.MA(pos, b1, L, mas, W, interlaced=b2, strategy='tiled')
            for a, b in ((a1, b1), (a2, b2)):
                if mas == 'NGP':
                    assert torch.equal(a, b)
                else:
                    assert (a - b).abs().max().item() <= 2e-6 * a.abs().max().item()
            del a1, a2, b1, b2


def test_owned_cell_write_out_ragged_groups(MASL):
    """1056^3 = 33 bins of 32 per side: owned-cell write-out on a grid that is not a
    power of two (cells wrap by the general rule) whose last group of bins along z
    holds a single bin; plain and interlaced CIC and weighted TSC against the atomic
    strategy."""
    rng = np.random.default_rng(57)
    N, L, n = 1056, 1000.0, 3_000_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    w = torch.from_numpy((rng.random(n) + 0.5).astype(np.float32)).cuda()
    for mas, W in (('CIC', None), ('TSC', w)):
        a1 = torch.zeros((N, N, N), device='cuda'); a2 = torch.zeros((N, N, N), device='cuda')
        MASL.MA(pos, a1, L, mas, W, interlaced=a2, strategy='atomic')
        b1 = torch.zeros((N, N, N), device='cuda'); b2 = torch.zeros((N, N, N), device='cuda')
        MASL.MA(pos, b1, L, mas, W, interlaced=b2, strategy='tiled')
        for a, b in ((a1, b1), (a2, b2)):
            assert (a - b).abs().max().item() <= 2e-6 * a.abs().max().item()
        del a1, a2, b1, b2
        torch.cuda.empty_cache()


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('inter', [False, True])
def test_owned_cell_write_out_accumulates(MASL, mas, inter):
    """On 1024^3 grids (a whole number of 32-cell bins) the tiled deposit stores each
    bin's own cells (old value + bin sum), carries its + z layers to the next bin of
    its CTA and passes its other halo layers to the next bins through a buffer.  It
    must add onto a non-zero grid exactly like the atomic strategy, wrap the halos
    of the last bins onto the first, and give identical bits on a second run (the
    halo sums are added in a fixed order)."""
    rng = np.random.default_rng(31)
    N, L, n = 1024, 1000.0, 4_000_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    # 100 particles in the last cells of the grid along x and z, the first along y:
    # their halos wrap onto bins at the other faces
    corner = rng.random((100, 3)).astype(np.float32) * np.float32(2 * L / N)
    corner[:, 0] = np.float32(L) - corner[:, 0] * np.float32(0.999)
    corner[:, 2] = np.float32(L) - corner[:, 2] * np.float32(0.999)
    pos[:100] = torch.from_numpy(corner % np.float32(L)).cuda()
    gen = torch.Generator(device='cuda')
    gen.manual_seed(31)
    base = torch.rand((N, N, N), generator=gen, device='cuda') * 5
    if mas == 'NGP':
        base = torch.floor(base)        # integer sums: any order gives the same bits
    runs = []
    for strategy in ('atomic', 'tiled', 'tiled'):
        a = base.clone()
        b = base.clone() if inter else None
        MASL.MA(pos, a, L, mas, interlaced=b, strategy=strategy)
        runs.append((a, b))
    for i in range(2 if inter else 1):
        ref, got, again = runs[0][i], runs[1][i], runs[2][i]
        if mas == 'NGP':
            assert torch.equal(ref, got)
        else:
            assert (ref - got).abs().max().item() <= 2e-6 * ref.abs().max().item()
        assert torch.equal(got, again)


@pytest.mark.parametrize('mas', MAS_LIST)
def test_weighted_fixed_point_edge_weights(MASL, mas):
    """Weighted tiled deposits accumulate weight / max|weight| in fixed point: weights
    spanning six decades, a negative weight (the bin is redone in float32) and all
    zero weights must all match the oracle (tolerance 2e-6 of the grid maximum)."""
    rng = np.random.default_rng(41)
    N, L, n = 96, 1000.0, 1_500_000
    pos = (rng.random((n, 3)) * L).astype(np.float32)
    wide = (10.0 ** rng.uniform(-3, 3, n)).astype(np.float32)
    neg = (rng.random(n) + 0.5).astype(np.float32)
    neg[12345] = -2.0
    zero = np.zeros(n, np.float32)
    for W in (wide, neg, zero):
        g = torch.zeros((N, N, N), device='cuda')
        g2 = torch.zeros((N, N, N), device='cuda')
        MASL.MA(torch.from_numpy(pos).cuda(), g, L, mas, torch.from_numpy(W).cuda(), interlaced=g2,
                strategy='tiled')
        o = np.zeros((N, N, N), np.float32)
        O.MA(pos, o, L, mas, W, threads=os.cpu_count() or 1)
        got = g.cpu().numpy()
        assert np.abs(got - o).max() <= 2e-6 * max(np.abs(o).max(), 1e-30), (mas, np.abs(got - o).max())
        if not W.any():
            assert not got.any() and not g2.cpu().numpy().any()


@pytest.mark.parametrize('mas', ['CIC', 'TSC', 'PCS'])
def test_fixed_point_overflow_falls_back(MASL, mas):
    """The tiled deposit accumulates a bin in 10.22 fixed point (cell sums below 1024).
    30000 particles at one position push cells past that: the bin must be redone in
    float32 (float sums of 30000 equal terms round by up to ~1e-3 relative in any
    order), not wrapped values (off by 1024)."""
    N, L = 64, 1000.0
    rng = np.random.default_rng(5)
    pos = np.concatenate([np.full((30000, 3), 123.4, np.float32),
                          (rng.random((20000, 3)) * L).astype(np.float32)])
    g = torch.zeros((N, N, N), device='cuda')
    MASL.MA(torch.from_numpy(pos).cuda(), g, L, mas, strategy='tiled')
    o = np.zeros((N, N, N), np.float32)
    O.MA(pos, o, L, mas)
    assert o.max() > 1024
    assert np.abs(g.cpu().numpy() - o).max() <= 5e-3 * o.max()


@pytest.mark.parametrize('mas', ['CIC', 'TSC', 'PCS'])
@pytest.mark.parametrize('inter', [False, True])
@pytest.mark.parametrize('clump', [0, 60000])
def test_dense_bins_find_wraps_from_the_total(MASL, mas, inter, clump):
    """From two particles per bin cell on average (here 1.1M particles in the eight
    32^3 bins of a 64^3 grid) the deposit skips reading back the old cell values and
    finds fixed-point wraps from the bin's total instead.  Uniform particles must
    match the oracle like every other fixed-point deposit; a clump of 60000
    particles at one position pushes cells past 1024 and its bin must be redone in
    float32, on both grids."""
    N, L = 64, 1000.0
    rng = np.random.default_rng(17)
    pos = np.concatenate([np.full((clump, 3), 123.4, np.float32),
                          (rng.random((1_100_000 - clump, 3)) * L).astype(np.float32)])
    g1 = torch.zeros((N, N, N), device='cuda')
    g2 = torch.zeros((N, N, N), device='cuda') if inter else None
    MASL.MA(torch.from_numpy(pos).cuda(), g1, L, mas, interlaced=g2, strategy='tiled')
    grids = [(g1, pos)]
    if inter:
        grids.append((g2, (pos + np.float32(0.5 * L / N)).astype(np.float32)))
    for g, p in grids:
        o = np.zeros((N, N, N), np.float32)
        O.MA(p, o, L, mas, threads=os.cpu_count() or 1)
        got = g.cpu().numpy()
        if clump:
            assert o.max() > 1024
            assert np.abs(got - o).max() <= 5e-3 * o.max()
        else:
            close(got, o, False, 5e-6)


def test_sorted_is_reproducible(MASL):
    """The sorted strategy sums every cell in one fixed order (neighbouring base cells,
    then particle index), with no atomics: two runs give identical bits, weighted and
    interlaced included."""
    rng = np.random.default_rng(21)
    N, L, n = 96, 1000.0, 1_500_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    W = torch.from_numpy((rng.random(n) * 2).astype(np.float32)).cuda()
    for mas in ('CIC', 'TSC', 'PCS'):
        out = []
        for _ in range(2):
            a = torch.zeros((N, N, N), device='cuda')
            b = torch.zeros((N, N, N), device='cuda')
            MASL.MA(pos, a, L, mas, W, interlaced=b, strategy='sorted')
            out.append((a, b))
        assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])


@pytest.mark.parametrize('mas', ['NGP', 'CIC', 'TSC', 'PCS'])
def test_sorted_staged_gather_equals_straight_sums(MASL, mas):
    """The sorted gather stages each CTA's base-cell particles in shared memory with
    their weights computed once; a window of more than the stage limit is summed
    straight from the sorted runs.  Both give the same products in the same order:
    with every window summed straight (limit 0) the grids are the same bits,
    weighted and interlaced, and a clump of 20000 particles (windows past the
    default limit beside staged ones) still matches the oracle."""
    from pylians_gb300 import _lib
    rng = np.random.default_rng(23)
    N, L, n = 80, 1000.0, 700_000
    pos = np.concatenate([(rng.random((n, 3)) * L).astype(np.float32),
                          (np.float32(400.0) + rng.random((20000, 3)).astype(np.float32) * np.float32(30.0))])
    W = (rng.random(pos.shape[0]) * 2).astype(np.float32)
    tp, tw = torch.from_numpy(pos).cuda(), torch.from_numpy(W).cuda()
    res = []
    try:
        for limit in (-1, 0):
            _lib.call('pyl_sorted_set_stage_limit', limit)
            a = torch.zeros((N, N, N), device='cuda')
            b = torch.zeros((N, N, N), device='cuda')
            MASL.MA(tp, a, L, mas, tw, interlaced=b, strategy='sorted')
            res.append((a, b))
    finally:
        _lib.call('pyl_sorted_set_stage_limit', -1)
    assert torch.equal(res[0][0], res[1][0]) and torch.equal(res[0][1], res[1][1])
    # against float64 sums of the reference's float32 weights: the clump's cells
    # (values ~1250) sum up to ~10^5 float32 terms (PCS: 64 base cells of ~1400
    # particles), rounding measured at 1.2e-5 of the largest cell; one particle lost
    # or doubled would move a cell by ~0.1 or more (3e-5 of it is 0.04)
    o = np.zeros((N, N, N), np.float64)
    O.ma_acc64(pos, o, L, mas, W, threads=os.cpu_count() or 1)
    got = res[0][0].cpu().numpy().astype(np.float64)
    assert np.abs(got - o).max() <= 3e-5 * np.abs(o).max()


def test_sorted_ngp_is_the_serial_loop(MASL, ma):
    """NGP under the sorted strategy adds each cell's particles in index order onto the
    grid it is given: bit-identical to the reference's serial loop for weighted
    deposits onto a non-integer base grid, where any other order differs in the last bits."""
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    rng = np.random.default_rng(4)
    W = (rng.random(pos.shape[0]) * 3).astype(np.float32)
    base = (rng.random((N, N, N)) * 7).astype(np.float32)
    o = base.copy()
    O.MA(pos, o, L, 'NGP', W, threads=1)
    t = torch.from_numpy(base.copy()).cuda()
    MASL.MA(torch.from_numpy(pos).cuda(), t, L, 'NGP', torch.from_numpy(W).cuda(), strategy='sorted')
    np.testing.assert_array_equal(t.cpu().numpy(), o)


def test_sorted_overdensity_matches_tiled(MASL):
    """Fused overdensity through the sorted strategy against the tiled one (grids
    filled with -1, deposits scaled by cells / N)."""
    rng = np.random.default_rng(8)
    N, L, n = 128, 1000.0, 3_000_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    res = {}
    for s in ('tiled', 'sorted'):
        a = torch.empty((N, N, N), device='cuda')
        b = torch.empty((N, N, N), device='cuda')
        MASL.overdensity_device(pos, a, L, "CIC", grid_interlaced=b, strategy=s)
        res[s] = (a, b)
    for i in range(2):
        assert (res['tiled'][i] - res['sorted'][i]).abs().max().item() <= 2e-6 * res['tiled'][i].abs().max().item() + 1e-6


def test_staged_placement_reports_no_device_error(MASL):
    """The TMA-staged histogram and placement kernels (bulk copies + bounded mbarrier
    waits) finish without a failed wait on a two-level grid, and an offset particle
    array (not 16-byte aligned) takes the direct-load kernels with the same result."""
    import ctypes
    from pylians_gb300 import _lib
    rng = np.random.default_rng(17)
    N, L, n = 544, 1000.0, 2_000_001
    pos = torch.from_numpy((rng.random((n + 1, 3)) * L).astype(np.float32)).cuda()
    word = ctypes.c_uint(0)
    _lib.call('pyl_device_error', 1, ctypes.byref(word))
    a = torch.zeros((N, N, N), device='cuda')
    b = torch.zeros((N, N, N), device='cuda')
    MASL.MA(pos[1:].contiguous(), a, L, 'CIC', strategy='tiled')
    MASL.MA(pos[1:], b, L, 'CIC', strategy='tiled')        # 12-byte offset view
    torch.cuda.synchronize()
    _lib.call('pyl_device_error', 0, ctypes.byref(word))
    assert word.value == 0
    assert (a - b).abs().max().item() <= 2e-6 * a.abs().max().item()


@pytest.mark.parametrize('name', ['CICW_d', 'NGPW_d'])
def test_ma_f64_golden(MASL, name):
    """CICW_d / NGPW_d into float64 grids against the compiled reference: NGPW_d bit-exact
    (float32 weights summed in float64 are exact here, whatever the order); CICW_d within
    1e-6 of the grid maximum (the reference's -ffast-math build multiplies the four float32
    factors in another association, an ulp apart).  3D onto zeros and onto a non-zero base
    (+=), 2D positions into a (N, N, 1) grid, numpy in and a CUDA tensor in place."""
    g = np.load(os.path.join(GOLDEN, 'ma_d_golden.npz'))
    pos, W = g['pos'], g['W']
    N, L = int(g['meta'][0]), float(g['meta'][1])
    fn = getattr(MASL, name)
    exact = name == 'NGPW_d'
    tol = 1e-6
    d = np.zeros((N, N, N))
    fn(pos, d, L, W)
    close(d, g['%s_3D' % name], exact, tol)
    d = g['base'].copy()
    fn(pos, d, L, W)
    close(d, g['%s_3D_accum' % name], exact, tol)
    d = np.zeros((N, N, 1))
    fn(np.ascontiguousarray(pos[:, :2]), d, L, W)
    close(d, g['%s_2D' % name], exact, tol)
    t = torch.zeros((N, N, N), dtype=torch.float64, device='cuda')
    fn(torch.from_numpy(pos).cuda(), t, L, torch.from_numpy(W).cuda())
    close(t.cpu().numpy(), g['%s_3D' % name], exact, tol)
