"""Pins the oracle (oracle/pyl_oracle.c + oracle/oracle.py) to the reference's own outputs.

The fixtures in tests/golden were produced by the compiled reference
(tests/golden/make_golden.py).  Tolerances:
  * NGP / NGPW grids, Nmodes*, kpar/kper: bit-exact;
  * CIC/TSC/PCS grids: |diff| <= 2e-6 * max|grid| (the reference is built with
    -ffast-math -march=native, so its compiler may fuse a multiply into the grid
    update; the oracle never does);
  * P(k)/XPk/B(k) from the same float32 input: relative 1e-9 (only the FFT
    library differs: scipy.fft float32 here, FFTW float32 in the reference).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import oracle as O

MAS_LIST = ['NGP', 'CIC', 'TSC', 'PCS']


@pytest.fixture(scope='module')
def ma():
    return np.load(os.path.join(GOLDEN, 'ma_golden.npz'))


@pytest.fixture(scope='module')
def pk():
    return np.load(os.path.join(GOLDEN, 'pk_golden.npz'))


@pytest.fixture(scope='module')
def bk():
    return np.load(os.path.join(GOLDEN, 'bk_golden.npz'))


def _grid_close(a, b, mas):
    if mas == 'NGP':
        np.testing.assert_array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= 2e-6 * np.abs(b).max()


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('weighted', [False, True])
def test_ma_conservation(ma, mas, weighted):
    """Test/test_MAS.py:10-84: sum(grid)/N == 1 (NGP to 20 places, others to 8)."""
    pos = ma['conservation_pos']
    W = np.full(pos.shape[0], 3.0, np.float32) if weighted else None
    d = np.zeros((64, 64, 64), np.float32)
    O.MA(pos, d, 1.0, mas, W=W)
    s = np.sum(d, dtype=np.float64)
    ref = float(ma['conservation_sum_%s%s' % (mas, 'W' if weighted else '')])
    norm = 3.0 * pos.shape[0] if weighted else pos.shape[0]
    assert round(s / norm - 1.0, 20 if mas == 'NGP' else 8) == 0
    if mas == 'NGP':
        assert s == ref
    else:
        assert abs(s - ref) <= 1e-8 * norm


@pytest.mark.parametrize('mas', MAS_LIST)
@pytest.mark.parametrize('tag', ['', 'W'])
def test_ma_grids(ma, mas, tag):
    pos, W = ma['grid_pos'], ma['grid_W']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    w = W if tag else None
    d = np.zeros((N, N, N), np.float32)
    O.MA(pos, d, L, mas, W=w)
    _grid_close(d, ma['MA3D_%s%s' % (mas, tag)], mas)
    d2 = np.zeros((N, N), np.float32)
    O.MA(np.ascontiguousarray(pos[:, :2]), d2, L, mas, W=w)
    _grid_close(d2, ma['MA2D_%s%s' % (mas, tag)], mas)
    c = np.zeros((N, N, N), np.float32)
    O.ma_kernel(pos, c, L, mas, w, threads=1, flavor=1)
    _grid_close(c, ma['MASc3D_%s%s' % (mas, tag)], mas)


def test_ma_accumulates(ma):
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    d = ma['accum_base'].copy()
    O.MA(pos, d, L, 'NGP')
    np.testing.assert_array_equal(d, ma['accum_NGP'])


def test_ma_openmp_matches_serial(ma):
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    a = np.zeros((N, N, N), np.float32)
    b = np.zeros((N, N, N), np.float32)
    O.ma_kernel(pos, a, L, 'NGP', None, threads=1, flavor=1)
    O.ma_kernel(pos, b, L, 'NGP', None, threads=4, flavor=1)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize('mas', ['NGP', 'CIC', 'TSC', 'PCS'])
def test_ma_acc64_matches_golden(ma, mas):
    """The float64-sum oracle keeps the reference's weights: its grid, rounded to
    float32, matches the compiled reference's within float32 accumulation rounding
    (NGP counts exactly)."""
    pos = ma['grid_pos']
    N, L = int(ma['grid_meta'][0]), float(ma['grid_meta'][1])
    g = np.zeros((N, N, N), np.float64)
    O.ma_acc64(pos, g, L, mas, threads=4)
    ref = ma['MA3D_%s' % mas]
    if mas == 'NGP':
        np.testing.assert_array_equal(g.astype(np.float32), ref)
    else:
        assert np.abs(g - ref).max() <= 2e-6 * np.abs(ref).max()


def _cmp_attr(x, y, name):
    x = np.asarray(x); y = np.asarray(y)
    assert x.shape == y.shape, name
    if name.startswith('Nmodes') or name in ('kpar', 'kper'):
        np.testing.assert_array_equal(x, y, err_msg=name)
    else:
        scale = np.abs(y).max() if y.size else 1.0
        np.testing.assert_allclose(x, y, rtol=1e-9, atol=1e-9 * scale, err_msg=name)


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('axis', [0, 1, 2])
def test_pk(pk, N, axis):
    r = O.Pk(pk['delta_%d' % N], 1000.0, axis, 'CIC', 1)
    for name in ['k1D', 'Pk1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'Nmodes2D',
                 'k3D', 'Pk', 'Nmodes3D', 'Pkphase']:
        _cmp_attr(getattr(r, name), pk['Pk_%d_axis%d_%s' % (N, axis, name)], name)


@pytest.mark.parametrize('N', [32, 15])
def test_xpk(pk, N):
    fields = [pk['delta_%d' % N], pk['delta2_%d' % N], pk['delta3_%d' % N]]
    r = O.XPk(fields, 1000.0, 1, ['CIC', 'PCS', 'NGP'], 1)
    for name in ['k1D', 'Pk1D', 'PkX1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'PkX2D',
                 'Nmodes2D', 'k3D', 'Pk', 'XPk', 'Nmodes3D']:
        _cmp_attr(getattr(r, name), pk['XPk_%d_%s' % (N, name)], name)


def test_pk_threads_match(pk):
    d = pk['delta_32']
    a = O.Pk(d, 1000.0, 2, 'CIC', 1)
    b = O.Pk(d, 1000.0, 2, 'CIC', 4)
    np.testing.assert_array_equal(a.Nmodes3D, b.Nmodes3D)
    np.testing.assert_allclose(a.Pk, b.Pk, rtol=1e-12)


def test_bk(bk):
    N, L, k1, k2 = bk['meta']
    r = O.Bk(bk['delta'], L, k1, k2, bk['theta'], 'CIC', 1)
    for n in ('B', 'Q', 'k', 'Pk'):
        np.testing.assert_allclose(getattr(r, n), bk['Bk_' + n], rtol=1e-9, err_msg=n)
    e = O.Bk(bk['delta'], L, 0.1, 0.1, np.array([2 * np.pi / 3]), 'CIC', 1)
    for n in ('B', 'Q', 'k', 'Pk'):
        np.testing.assert_allclose(getattr(e, n), bk['Bkeq_' + n], rtol=1e-9, err_msg=n)


def test_interlace_phase_reduces_aliasing():
    """Interlacing (no reference counterpart): the combined field's NGP/CIC P(k) of a
    uniform random catalogue approaches the shot noise 1/nbar near the Nyquist frequency,
    while the non-interlaced one overshoots it (aliasing of the shot noise)."""
    rng = np.random.default_rng(3)
    N, L = 32, 1000.0
    pos = (rng.random((N ** 3, 3)) * L).astype(np.float32)
    h = L / N
    pos2 = np.mod(pos + np.float32(0.5 * h), np.float32(L)).astype(np.float32)
    a = np.zeros((N, N, N), np.float32); O.MA(pos, a, L, 'CIC')
    b = np.zeros((N, N, N), np.float32); O.MA(pos2, b, L, 'CIC')
    m = np.mean(a, dtype=np.float64)
    a = (a / m - 1).astype(np.float32); b = (b / m - 1).astype(np.float32)
    plain = O.Pk(a, L, 0, 'CIC', 1)
    inter = O.Pk(a, L, 0, 'CIC', 1, interlaced=b)
    shot = L ** 3 / pos.shape[0]
    sel = (plain.k3D > 0.6 * np.pi / h) & (plain.k3D < 0.9 * np.pi / h)
    err_plain = np.abs(np.mean(plain.Pk[sel, 0]) / shot - 1)
    err_inter = np.abs(np.mean(inter.Pk[sel, 0]) / shot - 1)
    assert err_inter < err_plain


@pytest.fixture(scope='module')
def ig():
    return np.load(os.path.join(GOLDEN, 'interp_golden.npz'))


def test_oracle_cic_interp_golden(ig):
    """CIC_interp restatement against the reference's output.  MAS_library.pyx is built with
    -O3 -ffast-math -march=native (library/setup.py:8-11), which contracts and reorders the
    eight-term sum, so the two agree to a few ulps: within 1e-6 of the field scale."""
    pos = ig['interp_pos']
    den = np.zeros(pos.shape[0], np.float32)
    O.CIC_interp(ig['interp_field'], float(ig['interp_meta'][1]), pos, den)
    np.testing.assert_allclose(den, ig['interp_den'], rtol=0, atol=1e-6 * np.abs(ig['interp_field']).max())


@pytest.mark.parametrize('axis', [0, 1, 2])
def test_oracle_rsd_golden(ig, axis):
    """pos_redshift_space is built without extra flags (library/setup.py:23): bit-exact."""
    L, H, z = (float(x) for x in ig['rsd_meta'])
    p = ig['rsd_pos'].copy()
    O.pos_redshift_space(p, ig['rsd_vel'], L, H, z, axis)
    np.testing.assert_array_equal(p, ig['rsd_out_axis%d' % axis])


@pytest.fixture(scope='module')
def xg():
    return np.load(os.path.join(GOLDEN, 'xi_golden.npz'))


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('axis', [0, 2])
def test_oracle_xi_golden(xg, N, axis):
    r = O.Xi(xg['delta_%d' % N], 1000.0, 'CIC', axis)
    np.testing.assert_array_equal(r.Nmodes3D, xg['Xi_%d_axis%d_Nmodes3D' % (N, axis)])
    np.testing.assert_allclose(r.r3D, xg['Xi_%d_axis%d_r3D' % (N, axis)], rtol=1e-12)
    ref = xg['Xi_%d_axis%d_xi' % (N, axis)]
    assert np.abs(r.xi - ref).max() <= 1e-6 * np.abs(ref[:, 0]).max()


@pytest.mark.parametrize('N', [32, 15])
def test_oracle_correct_mas_golden(xg, N):
    """The same float operations and the same (scipy) inverse transform as the
    reference run under the pyFFTW stand-in: bit-exact."""
    np.testing.assert_array_equal(O.correct_MAS(xg['delta_%d' % N], 1000.0, 'CIC'), xg['correct_MAS_%d' % N])


@pytest.fixture(scope='module')
def pg():
    return np.load(os.path.join(GOLDEN, 'plane_golden.npz'))


@pytest.mark.parametrize('N', [64, 45])
def test_oracle_plane_golden(pg, N):
    a, b = pg['map1_%d' % N], pg['map2_%d' % N]
    r = O.Pk_plane(a, 1000.0, 'CIC')
    np.testing.assert_array_equal(r.Nmodes, pg['Pkplane_%d_Nmodes' % N])
    np.testing.assert_allclose(r.Pk, pg['Pkplane_%d_Pk' % N], rtol=1e-12)
    x = O.XPk_plane(a, b, 1000.0, 'CIC', 'TSC')
    for n in ('k', 'Pk', 'XPk', 'r'):
        np.testing.assert_allclose(getattr(x, n), pg['XPkplane_%d_%s' % (N, n)], rtol=1e-12)


@pytest.fixture(scope='module')
def sg():
    return np.load(os.path.join(GOLDEN, 'smoothing_golden.npz'))


@pytest.mark.parametrize('N', [32, 15])
@pytest.mark.parametrize('filt,R', [('Top-Hat', 100.0), ('Gaussian', 60.0)])
def test_oracle_smoothing_golden(sg, N, filt, R):
    t = filt.replace('-', '')
    gf = sg['filter_%s_%d' % (t, N)]
    np.testing.assert_array_equal(O.FT_filter(1000.0, R, N, filt), gf)
    sm = O.field_smoothing(sg['field_%d' % N], gf)
    ref = sg['smoothed_%s_%d' % (t, N)]
    assert np.abs(sm - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize('name,mas', [('CICW_d', 'CIC'), ('NGPW_d', 'NGP')])
def test_ma_f64_golden(name, mas):
    """CICW_d / NGPW_d (MAS_library.pyx:229-266, :338-358): float64 grids.  The oracle adds the
    same float32 products in the reference's serial order, so every case is bit-exact: 3D onto
    zeros and onto a non-zero base, and 2D positions into a (N, N, 1) grid."""
    g = np.load(os.path.join(GOLDEN, 'ma_d_golden.npz'))
    pos, W = g['pos'], g['W']
    N, L = int(g['meta'][0]), float(g['meta'][1])
    d = np.zeros((N, N, N))
    O.ma_f64(pos, d, L, mas, W)
    np.testing.assert_array_equal(d, g['%s_3D' % name])
    d = g['base'].copy()
    O.ma_f64(pos, d, L, mas, W)
    np.testing.assert_array_equal(d, g['%s_3D_accum' % name])
    d = np.zeros((N, N, 1))
    O.ma_f64(np.ascontiguousarray(pos[:, :2]), d, L, mas, W)
    np.testing.assert_array_equal(d, g['%s_2D' % name])
