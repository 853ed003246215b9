"""Parity at the benchmark configurations' own shapes, against the oracle.

The other GPU tests shrink the inputs; these run each configuration at its
full size through the product path and compare with the oracle (the C/numpy
restatement of the reference, on all host cores):

  * headline grid: CIC + interlaced P(k) (axis 0, l = 0,2,4, Pk2D) on the
    1024^3 grid with 2^26 particles: the owned-cell write-out, the halo kernel
    and the barrier-free staged deposit of that grid; Nmodes1D/2D/3D, kpar,
    kper bit-exact against the oracle's integer mode loop;
  * headline particle count: 1024^3 particles on the 1024^3 grids (the bench
    step, two-level placement included), every cell of an x slab of both grids
    against the oracle's deposit of the particles that reach it, and the mass
    of the whole grid;
  * the wrap-from-total deposit together with the owned-cell write-out (it
    runs from two particles per cell on 1024^3 grids and up), reached on a
    128^3 grid by moving the two thresholds, with clumped particles whose
    cells wrap the fixed-point sums;
  * Zel'dovich + redshift space: 512^3 lattice particles on 512^3 grids, TSC
    and PCS with and without interlacing, and XPk against the NGP field;
  * bispectrum: the 256^3 field, k1 = 0.1, k2 = 0.2 h/Mpc with 32 theta bins
    and 20 equilateral triangles k = 0.02..0.4 h/Mpc in one batched call;
  * batched realizations: a sample of the 512 seeded realizations spanning all
    four grid sizes and the 1e5..1.7e7 particle range, per realization
    against the oracle (not against the one-at-a-time GPU path).

Tolerances are those of the smaller tests: integer quantities bit-exact, grids
|gpu - oracle| <= 1e-5 max|oracle| for the overdensity (the GPU writes
-1 + n/mean in one pass, the oracle n/mean - 1 after the deposit), P(k) rtol
1e-4 (check_pk), B within 1e-3 of the largest |B| of the set.
"""
import os

import numpy as np
import pytest
import torch

import oracle as O
from test_gpu_pk import PK_NAMES, XPK_NAMES, check_pk

pytestmark = pytest.mark.gpu
T = os.cpu_count() or 1


@pytest.fixture(scope='module', autouse=True)
def built():
    import pylians_gb300.build as b
    b.build()


def oracle_overdensity(pos, N, L, mas, shift=False, n_total=None, acc64=False):
    """The callers' convention (Pk_snapshot.py:80-88): MA, then delta = n/mean - 1 in float32.
    acc64: the reference's float32 weights summed in float64, then the overdensity rounded
    to float32 (the oracle without its own float32 accumulation noise)."""
    p = (pos + np.float32(0.5 * L / N)).astype(np.float32) if shift else pos
    n = pos.shape[0] if n_total is None else n_total
    if acc64:
        g64 = np.zeros((N, N, N), np.float64)
        O.ma_acc64(p, g64, L, mas, threads=T)
        return (g64 / (n / N ** 3) - 1.0).astype(np.float32)
    g = np.zeros((N, N, N), np.float32)
    O.MA(p, g, L, mas, threads=T)
    g /= np.float32(n / N ** 3)
    g -= np.float32(1.0)
    return g


def grid_close(gpu, ref, tol=1e-5):
    err = np.abs(gpu - ref).max()
    assert err <= tol * np.abs(ref).max(), (err, np.abs(ref).max())


def test_headline_grid_pk_vs_oracle():
    from pylians_gb300.pipeline import ParticlePk
    N, L, n = 1024, 1000.0, 1 << 26
    gen = torch.Generator(device='cuda')
    gen.manual_seed(11)
    pos = torch.rand((n, 3), generator=gen, device='cuda') * L
    pp = ParticlePk(N, L, 'CIC', axis=0, interlaced=True, max_particles=n)
    pp.step(pos)
    r = pp.result()
    host = pos.cpu().numpy()
    del pos
    a = oracle_overdensity(host, N, L, 'CIC')
    grid_close(pp.grids[0].cpu().numpy(), a)
    b = oracle_overdensity(host, N, L, 'CIC', shift=True)
    grid_close(pp.grids[1].cpu().numpy(), b)
    del pp
    torch.cuda.empty_cache()
    o = O.Pk(a, L, 0, 'CIC', T, interlaced=b)
    check_pk(r, lambda k: getattr(o, k), PK_NAMES)
    assert r.Nmodes3D.sum() + 1 == (N ** 3 - 8) // 2 + 8


def test_headline_particles_slab_vs_oracle():
    """1024^3 particles on the 1024^3 grids.  Cells with x in [2, 63] of both grids
    receive mass only from particles whose plain base cell x lies in [0, 63], so the
    oracle deposits exactly those particles and the slab must match cell by cell."""
    from pylians_gb300.pipeline import ParticlePk
    N, L, n = 1024, 1000.0, 1 << 30
    gen = torch.Generator(device='cuda')
    gen.manual_seed(1)
    pos = torch.rand((n, 3), generator=gen, device='cuda') * L
    pp = ParticlePk(N, L, 'CIC', axis=0, interlaced=True, max_particles=n)
    pp.step(pos)
    # the mass of the whole grid: sum of delta = 0 up to the float32 rounding of each cell
    for g in pp.grids:
        s = g.double().sum().item()
        assert abs(s) <= 1e-6 * N ** 3, s
    slabs = [g[2:64].cpu().numpy() for g in pp.grids]
    r = pp.result()
    assert r.Nmodes3D.sum() + 1 == (N ** 3 - 8) // 2 + 8
    del pp
    torch.cuda.empty_cache()
    inv = np.float32(N) / np.float32(L)
    sel = (pos[:, 0] * inv < 64.0)
    part = pos[sel].cpu().numpy()
    del pos, sel
    torch.cuda.empty_cache()
    for gi, shift in ((0, False), (1, True)):
        ref = oracle_overdensity(part, N, L, 'CIC', shift=shift, n_total=n)[2:64]
        grid_close(slabs[gi], ref)


def test_wrap_from_total_with_owned_cells():
    """The bin-total wrap check and the owned-cell write-out together, on a 128^3
    grid: thresholds moved so that both apply, particles clumped into a few cells
    so that fixed-point cell sums pass 1024 and the bins redo in float32.  Those
    cells hold about 4000 float32 terms summed in different orders on the two sides
    (a few 1e-5 of the cell apart), so grids agree within 1e-4 of their largest
    value; a wrap missed by the check would be off by 1024 counts (about 600 in
    the overdensity, a quarter of the largest value)."""
    import pylians_gb300.MAS_library as MASL
    from pylians_gb300 import _lib
    N, L = 128, 1000.0
    rng = np.random.default_rng(41)
    uni = (rng.random((3_000_000, 3)) * L).astype(np.float32)
    clump = (np.float32(500.0) + rng.random((100_000, 3)).astype(np.float32) * np.float32(3 * L / N))
    pos = np.concatenate([uni, clump.astype(np.float32)])
    _lib.call('pyl_ma_set_thresholds', 128, 0.5)
    try:
        for mas in ('CIC', 'TSC'):
            for inter in (False, True):
                d = torch.empty((N, N, N), device='cuda')
                d2 = torch.empty((N, N, N), device='cuda') if inter else None
                MASL.overdensity_device(torch.from_numpy(pos).cuda(), d, L, mas, grid_interlaced=d2,
                                        strategy='tiled')
                grid_close(d.cpu().numpy(), oracle_overdensity(pos, N, L, mas), tol=1e-4)
                if inter:
                    grid_close(d2.cpu().numpy(), oracle_overdensity(pos, N, L, mas, shift=True), tol=1e-4)
                g = np.zeros((N, N, N), np.float32)
                MASL.MA(pos, g, L, mas, strategy='tiled')
                o = np.zeros((N, N, N), np.float32)
                O.MA(pos, o, L, mas, threads=T)
                assert o.max() > 1024.0                     # cells past the fixed-point range
                assert np.abs(g - o).max() <= 1e-4 * np.abs(o).max()
    finally:
        _lib.call('pyl_ma_set_thresholds', -1, -1.0)


@pytest.fixture(scope='module')
def zeldovich512():
    from pylians_gb300 import synthetic
    pos = synthetic.zeldovich(N_field=256, N_lattice=512, BoxSize=1000.0, sigma=0.5, f=0.5, rsd_axis=2, seed=1)
    return pos, pos.cpu().numpy()


@pytest.mark.parametrize('mas', ['TSC', 'PCS'])
def test_zeldovich512_vs_oracle(zeldovich512, mas):
    from pylians_gb300.pipeline import ParticlePk
    pos, host = zeldovich512
    N, L = 512, 1000.0
    a = oracle_overdensity(host, N, L, mas)
    b = oracle_overdensity(host, N, L, mas, shift=True)
    for inter in (False, True):
        pp = ParticlePk(N, L, mas, axis=2, interlaced=inter, max_particles=pos.shape[0])
        pp.step(pos)
        grid_close(pp.grids[0].cpu().numpy(), a)
        if inter:
            grid_close(pp.grids[1].cpu().numpy(), b)
        r = pp.result()
        o = O.Pk(a, L, 2, mas, T, interlaced=b if inter else None)
        check_pk(r, lambda k: getattr(o, k), [k for k in PK_NAMES if k != 'Pkphase'], floor=1e-6)
        del pp
        torch.cuda.empty_cache()


def test_zeldovich512_xpk_against_ngp(zeldovich512):
    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.Pk_library as PKL
    pos, host = zeldovich512
    N, L = 512, 1000.0
    d = [torch.empty((N, N, N), device='cuda') for _ in range(2)]
    MASL.overdensity_device(pos, d[0], L, 'TSC')
    MASL.overdensity_device(pos, d[1], L, 'NGP')
    a = oracle_overdensity(host, N, L, 'TSC')
    b = oracle_overdensity(host, N, L, 'NGP')
    grid_close(d[0].cpu().numpy(), a)
    grid_close(d[1].cpu().numpy(), b)
    r = PKL.XPk(d, L, 2, ['TSC', 'NGP'])
    o = O.XPk([a, b], L, 2, ['TSC', 'NGP'], T)
    check_pk(r, lambda k: getattr(o, k), XPK_NAMES, cross=True, floor=1e-6)


def test_bispectrum256_vs_oracle():
    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.Pk_library as PKL
    N, L = 256, 1000.0
    gen = torch.Generator(device='cuda')
    gen.manual_seed(3)
    pos = torch.rand((N ** 3, 3), generator=gen, device='cuda') * L
    d = torch.empty((N, N, N), device='cuda')
    MASL.overdensity_device(pos, d, L, 'CIC')
    delta = d.cpu().numpy()
    grid_close(delta, oracle_overdensity(pos.cpu().numpy(), N, L, 'CIC'))
    theta = np.linspace(0, np.pi, 32)
    k3 = np.sqrt((0.2 * np.sin(theta)) ** 2 + (0.2 * np.cos(theta) + 0.1) ** 2)
    ks = np.linspace(0.02, 0.4, 20)
    tris = [(0.1, 0.2, float(x)) for x in k3] + [(float(k), float(k), float(k)) for k in ks]
    B, Q, P1, P2, P3 = PKL.Bk_triangles(d, L, tris, 'CIC')
    o = O.Bk(delta, L, 0.1, 0.2, theta, 'CIC', T)
    ob = [o.B] + [O.Bk(delta, L, k, k, np.array([2 * np.pi / 3]), 'CIC', T).B for k in ks]
    ob = np.concatenate(ob)
    assert np.abs(B - ob).max() <= 1e-3 * np.abs(ob).max()
    # the sweep's shell powers P(k1), P(k2), P(k3) against the oracle's
    np.testing.assert_allclose(P1[:32], o.Pk[0], rtol=1e-4)
    np.testing.assert_allclose(P2[:32], o.Pk[1], rtol=1e-4)
    np.testing.assert_allclose(P3[:32], o.Pk[2:], rtol=1e-4)
    # the same call through Bk (the reference's entry point)
    r = PKL.Bk(d, L, 0.1, 0.2, theta, 'CIC')
    assert np.abs(r.B - o.B).max() <= 1e-3 * np.abs(o.B).max()
    assert np.abs(r.Q - o.Q).max() <= 1e-3 * np.abs(o.Q).max()


def _sample(specs):
    """Realizations spanning the four grid sizes, the smallest and largest particle
    counts, every MAS and both interlacing choices."""
    pick = set()
    for dims in (64, 128, 192, 256):
        idx = [i for i, s in enumerate(specs) if s['dims'] == dims]
        pick.add(min(idx, key=lambda i: specs[i]['n']))
        pick.add(max(idx, key=lambda i: specs[i]['n']))
    for mas in ('CIC', 'TSC', 'PCS'):
        for inter in (False, True):
            pick.add(next(i for i, s in enumerate(specs) if s['MAS'] == mas and s['interlaced'] == inter))
    return sorted(pick)


def test_batch_sample_vs_oracle(tmp_path):
    os.environ['PYL_AUTOTUNE_CACHE'] = str(tmp_path / 'autotune.json')
    from pylians_gb300 import batch
    L = 1000.0
    full = batch.random_specs(512, seed=0)
    specs = [full[i] for i in _sample(full)]
    ns = [s['n'] for s in specs]
    assert min(ns) < 200_000 and max(ns) > 10_000_000
    assert {s['dims'] for s in specs} == {64, 128, 192, 256}
    gen = torch.Generator(device='cuda')
    gen.manual_seed(5)
    pos = [torch.rand((s['n'], 3), generator=gen, device='cuda') * L for s in specs]
    B = batch.RealizationBatch(specs, L, axis=0)
    B.step(pos)
    res = B.results()
    for s, p, r in zip(specs, pos, res):
        host = p.cpu().numpy()
        N, mas = s['dims'], s['MAS']
        # the oracle sums the reference's float32 weights in float64: its float32 serial
        # sums (one rounding of the cell value per add; 59 particles per cell with PCS on
        # 64^3 are 3776 adds a cell) carry rounding noise that the deconvolution lifts to
        # 4e-4 of the Pk2D bins near the corner, 16x that of this path's 10.22 fixed-point
        # sums, so the comparison would measure the oracle's error
        a = oracle_overdensity(host, N, L, mas, acc64=True)
        b = oracle_overdensity(host, N, L, mas, shift=True, acc64=True) if s['interlaced'] else None
        o = O.Pk(a, L, 0, mas, T, interlaced=b)
        # 1e5 particles on 256^3 cells are pure shot noise, and near the grid's corner the
        # TSC/PCS window leaves (2/pi)^(6p) of that power, so after deconvolution the
        # float32 rounding of either grid (white in k) is a 1e-4 effect in those Pk2D
        # bins, and one-mode bins can hold 1e-4 of the typical power: a floor of 5e-4
        # of the median bin for Pk2D and of the peak monopole for the 3D multipoles
        check_pk(r, lambda k: getattr(o, k), [k for k in PK_NAMES if k != 'Pkphase'], floor=5e-4,
                 floor2d=5e-4)
