"""GPU parity of P(k) / XPk (cuFFT R2C + the fused deconvolve/bin kernel) against
the reference's golden outputs and the oracle.

Tolerances: Nmodes1D/2D/3D, kpar, kper bit-exact; k1D, k3D rtol 1e-12;
P(k) sums: |gpu - ref| <= 1e-4 * |ref| for l=0, 1D, 2D and phase, and
|gpu - ref| <= 1e-4 * |P0| for the l=2,4 multipoles (they cross zero).
The GPU and the reference use different float32 FFTs (cuFFT vs FFTW/pocketfft).
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-4


@pytest.fixture(scope='module')
def PKL():
    import pylians_gb300.build as b
    b.build()
    import pylians_gb300.Pk_library as P
    return P


@pytest.fixture(scope='module')
def pk():
    return np.load(os.path.join(GOLDEN, 'pk_golden.npz'))


EXACT = ('Nmodes1D', 'Nmodes2D', 'Nmodes3D', 'kpar', 'kper')


def cross_scale(auto, nfields):
    """sqrt(|P_ii P_jj|) for the pairs i<j in the reference's order: cross spectra of
    weakly correlated fields sit near zero, so their error is measured on this scale."""
    cols = [np.sqrt(np.abs(auto[..., i] * auto[..., j]))
            for i in range(nfields) for j in range(i + 1, nfields)]
    return np.stack(cols, axis=-1)


def check_pk(r, get, names, cross=False, floor=1e-8, floor2d=0.0):
    for n in names:
        x, y = np.asarray(getattr(r, n)), np.asarray(get(n))
        assert x.shape == y.shape, (n, x.shape, y.shape)
        if n in ('XPk', 'PkX1D', 'PkX2D'):
            auto = np.asarray(get({'XPk': 'Pk', 'PkX1D': 'Pk1D', 'PkX2D': 'Pk2D'}[n]))
            F = auto.shape[-1]
            sc = cross_scale(auto[:, 0] if n == 'XPk' else auto, F)
            if n == 'XPk':
                sc = sc[:, None, :]
            sc = np.broadcast_to(sc, y.shape)
            ok = np.isfinite(y)
            err = np.abs(x - y)[ok]
            assert np.all(err <= RTOL * sc[ok] + 1e-6 * np.abs(y[ok]).max()), (n, np.max(err / (sc[ok] + 1e-30)))
        elif n in EXACT:
            np.testing.assert_array_equal(x, y, err_msg=n)
        elif n in ('k1D', 'k3D'):
            np.testing.assert_allclose(x, y, rtol=1e-12, err_msg=n)
        elif n in ('Pk', 'XPk'):
            # absolute floor `floor` of the largest monopole: bins whose power sits many
            # decades below the peak are float32 round-off on both sides
            p0 = np.abs(y[:, 0:1])
            atol = floor * p0.max()
            assert np.all(np.abs(x - y) <= RTOL * p0 + atol + 1e-30), (n, np.max(np.abs(x - y) / (p0 + atol + 1e-30)))
        else:
            ok = np.isfinite(y)
            assert np.array_equal(ok, np.isfinite(x)), n
            if n in ('Pk2D', 'PkX2D'):
                # the DC bin (k_par = k_per = 0) holds |delta(k=0)|^2, pure float round-off of
                # a zero-mean field whatever its size: compared on the array's scale
                big = np.abs(y[ok]).max()
                assert np.all(np.abs(x[0] - y[0]) <= 1e-4 * big), (n, 'DC', x[0], y[0])
                ok = ok.copy()
                ok[0] = False
            # floor: cross spectra pass through zero, so the absolute floor is 1e-6 of
            # the array's largest value; floor2d adds floor2d x the median |bin| for 2D
            # spectra of shot-noise fields (see the batched-realization test)
            atol = 1e-6 * np.abs(y[ok]).max()
            if floor2d and n in ('Pk2D', 'PkX2D'):
                atol = max(atol, floor2d * np.median(np.abs(y[ok])))
            err = np.abs(x[ok] - y[ok])
            assert np.all(err <= RTOL * np.abs(y[ok]) + atol), (n, np.max(err / (np.abs(y[ok]) + atol / RTOL)))


PK_NAMES = ['k1D', 'Pk1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'Nmodes2D', 'k3D', 'Pk',
            'Nmodes3D', 'Pkphase']
XPK_NAMES = ['k1D', 'Pk1D', 'PkX1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'PkX2D', 'Nmodes2D',
             'k3D', 'Pk', 'XPk', 'Nmodes3D']


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('axis', [0, 1, 2])
def test_pk_golden(PKL, pk, N, axis):
    r = PKL.Pk(pk['delta_%d' % N], 1000.0, axis, 'CIC', 1)
    check_pk(r, lambda n: pk['Pk_%d_axis%d_%s' % (N, axis, n)], PK_NAMES)


@pytest.mark.parametrize('N', [32, 15])
def test_xpk_golden(PKL, pk, N):
    fields = [pk['delta_%d' % N], pk['delta2_%d' % N], pk['delta3_%d' % N]]
    r = PKL.XPk(fields, 1000.0, 1, ['CIC', 'PCS', 'NGP'], 1)
    check_pk(r, lambda n: pk['XPk_%d_%s' % (N, n)], XPK_NAMES)


def test_xpk_many_fields_pairwise(PKL, pk):
    """Five fields exceed one launch; the pairwise path must equal the oracle."""
    d = pk['delta_32']
    fields = [d, (0.5 * d).astype(np.float32), np.roll(d, 1, 0), np.roll(d, 2, 1), (d * d).astype(np.float32)]
    mas = ['CIC', 'CIC', 'TSC', 'NGP', 'PCS']
    r = PKL.XPk(fields, 1000.0, 2, mas)
    o = O.XPk(fields, 1000.0, 2, mas)
    check_pk(r, lambda n: getattr(o, n), XPK_NAMES)


@pytest.mark.parametrize('axis', [0, 2])
def test_pk_config1_vs_oracle(PKL, axis):
    """128^3 particles, CIC on 128^3, overdensity, P(k) with l=0,2,4 and Pk2D."""
    rng = np.random.default_rng(1)
    N, L = 128, 1000.0
    pos = (rng.random((N ** 3, 3)) * L).astype(np.float32)
    g = np.zeros((N, N, N), np.float32)
    O.MA(pos, g, L, 'CIC', threads=os.cpu_count() or 1)
    g /= np.float32(N ** 3 / N ** 3)
    g -= np.float32(1.0)
    r = PKL.Pk(g, L, axis, 'CIC')
    o = O.Pk(g, L, axis, 'CIC', os.cpu_count() or 1)
    check_pk(r, lambda n: getattr(o, n), PK_NAMES)
    assert r.Nmodes3D.sum() + 1 == (N ** 3 - 8) // 2 + 8


@pytest.mark.parametrize('mas', ['CIC', 'PCS'])
def test_pk_interlaced_vs_oracle(PKL, mas):
    rng = np.random.default_rng(3)
    N, L = 64, 1000.0
    a = rng.standard_normal((N, N, N)).astype(np.float32)
    b = (a + 0.1 * rng.standard_normal((N, N, N))).astype(np.float32)
    r = PKL.Pk(a, L, 1, mas, interlaced=b)
    o = O.Pk(a, L, 1, mas, 1, interlaced=b)
    check_pk(r, lambda n: getattr(o, n), PK_NAMES)


def test_keep_deltak(PKL, pk):
    d = pk['delta_32']
    r = PKL.Pk(d, 1000.0, 0, 'TSC', keep_deltak=True)
    o = O.Pk(d, 1000.0, 0, 'TSC', 1, keep_deltak=True)
    # the reference corrects only the modes it visits; the GPU corrects every stored mode
    vis = o.delta_k != O.fft_r2c(d)
    np.testing.assert_allclose(r.delta_k[vis], o.delta_k[vis], rtol=2e-5, atol=2e-5 * np.abs(o.delta_k).max())


def test_fft_roundtrip(PKL):
    """R2C (unnormalised) then the normalised C2R of IFFT3Dr_f returns the input."""
    rng = np.random.default_rng(5)
    for N in (16, 15, 64):
        a = rng.standard_normal((N, N, N)).astype(np.float32)
        k = PKL.FFT3Dr_f(a)
        np.testing.assert_allclose(k, O.fft_r2c(a), rtol=1e-4, atol=1e-4 * np.abs(k).max())
        b = PKL.IFFT3Dr_f(k)
        np.testing.assert_allclose(b, a, atol=1e-5)


def test_pipeline_matches_stepwise(PKL):
    """The resident ParticlePk chain (and its CUDA-graph replay) equals MA + normalise + Pk."""
    from pylians_gb300.pipeline import ParticlePk
    import pylians_gb300.MAS_library as MASL
    rng = np.random.default_rng(9)
    N, L, n = 64, 1000.0, 400000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    pp = ParticlePk(N, L, 'CIC', axis=0, interlaced=True, max_particles=n)
    pp.step(pos)
    r = pp.result()
    g1 = torch.zeros((N, N, N), device='cuda')
    g2 = torch.zeros((N, N, N), device='cuda')
    MASL.MA(pos, g1, L, 'CIC', interlaced=g2)
    m = np.float32(n / N ** 3)
    a = (g1.cpu().numpy() / m - np.float32(1)).astype(np.float32)
    b = (g2.cpu().numpy() / m - np.float32(1)).astype(np.float32)
    o = O.Pk(a, L, 0, 'CIC', 1, interlaced=b)
    check_pk(r, lambda k: getattr(o, k), PK_NAMES)
    pp.capture(pos)
    for _ in range(2):
        pp.replay()
    r2 = pp.result()
    np.testing.assert_array_equal(r2.Nmodes3D, r.Nmodes3D)
    np.testing.assert_allclose(r2.Pk, r.Pk, rtol=1e-6, atol=1e-6 * np.abs(r.Pk[:, 0]).max())


@pytest.mark.parametrize('weighted', [False, True])
def test_overdensity_deposit_matches_two_pass(weighted):
    """pyl_ma_overdensity (fill -1, deposits scaled by 1/mean) equals MA followed by
    delta = n/mean - 1 (Pk_snapshot.py:70-88) within a few float32 ulps of delta."""
    import pylians_gb300.MAS_library as MASL
    rng = np.random.default_rng(21)
    N, L, n = 96, 1000.0, 1_500_000
    pos = torch.from_numpy((rng.random((n, 3)) * L).astype(np.float32)).cuda()
    W = torch.from_numpy((rng.random(n) * 3).astype(np.float32)).cuda() if weighted else None
    for strategy in ('atomic', 'tiled'):
        d1 = torch.empty((N, N, N), device='cuda'); d2 = torch.empty((N, N, N), device='cuda')
        MASL.overdensity_device(pos, d1, L, 'CIC', W, grid_interlaced=d2, strategy=strategy)
        g1 = torch.zeros((N, N, N), device='cuda'); g2 = torch.zeros((N, N, N), device='cuda')
        MASL.MA(pos, g1, L, 'CIC', W, interlaced=g2, strategy=strategy)
        mean = (W.double().sum().item() if weighted else float(n)) / N ** 3
        for d, g in ((d1, g1), (d2, g2)):
            ref = g.double() / mean - 1.0
            assert (d.double() - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()


@pytest.mark.parametrize('mas', ['NGP', 'CIC', 'TSC', 'PCS'])
@pytest.mark.parametrize('N', [200, 1024])
def test_overdensity_owned_cells_with_empty_bins(mas, N):
    """Particles packed into one corner leave most bins empty, which must still read
    -1, and every cell must equal the two-pass MA + delta = n/mean - 1, plain and
    interlaced.  1024^3 takes the owned-cell write-out: every bin, empty or not,
    stores -1 + its sum into its own cells and its halo into a buffer that a second
    kernel adds to the next bins; the ragged 200^3 grid fills with -1 and adds every
    bin with its halo atomically."""
    import pylians_gb300.MAS_library as MASL
    rng = np.random.default_rng(23)
    L, n = 1000.0, 1_500_000
    pos = torch.from_numpy((rng.random((n, 3)) * 260.0 + 30.0).astype(np.float32)).cuda()
    d1 = torch.full((N, N, N), 7.0, device='cuda'); d2 = torch.full((N, N, N), 7.0, device='cuda')
    MASL.overdensity_device(pos, d1, L, mas, grid_interlaced=d2, strategy='tiled')
    g1 = torch.zeros((N, N, N), device='cuda'); g2 = torch.zeros((N, N, N), device='cuda')
    MASL.MA(pos, g1, L, mas, interlaced=g2, strategy='atomic')
    mean = float(n) / N ** 3
    for d, g in ((d1, g1), (d2, g2)):
        ref = g.double() / mean - 1.0
        assert (d.double() - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
        assert torch.equal(d[g == 0], torch.full_like(d[g == 0], -1.0))


@pytest.mark.parametrize('axis', [0, 2])
def test_pk_bin_partials_match_shared_sums(PKL, axis):
    """One-field binning flushes into per-CTA global partial sums when the caller's
    workspace holds them (pyl_pk_workspace_size) and into shared memory otherwise
    (axis 0 without a workspace; axis 2 with only the ring table): both must give the
    same sums (float32 partials added in different orders: rtol 1e-5 of each bin's
    monopole scale)."""
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr, stream_ptr
    L = _lib.load()
    rng = np.random.default_rng(12)
    N = 96
    a = torch.from_numpy(rng.standard_normal((N, N, N)).astype(np.float32)).cuda()
    b = torch.from_numpy(rng.standard_normal((N, N, N)).astype(np.float32)).cuda()
    dk = torch.empty((2, N, N, N // 2 + 1), dtype=torch.complex64, device='cuda')
    _lib.call('pyl_fft_r2c', ptr(torch.stack([a, b])), ptr(dk), N, 2, stream_ptr())
    n = L.pyl_pk_sums_len(N, 1)
    mp, keep = PKL.ctypes_int_array([2])
    full = L.pyl_pk_workspace_size(N, 1, axis)
    ring = L.pyl_pk_workspace_size(N, 2, 2) if axis == 2 else 0    # ring table only (two fields: no partials)
    ws = torch.empty(full, dtype=torch.uint8, device='cuda')
    out = []
    for nbytes in (full, ring):
        s = torch.empty(n, dtype=torch.float64, device='cuda')
        _lib.call('pyl_pk_bin', ptr(dk[0]), ptr(dk[1]), 1, 0, N, axis, mp, ptr(s),
                  ptr(ws) if nbytes else None, nbytes, stream_ptr())
        out.append(s.cpu().numpy())
    scale = np.abs(out[1]).max()
    np.testing.assert_allclose(out[0], out[1], rtol=1e-5, atol=1e-6 * scale)
