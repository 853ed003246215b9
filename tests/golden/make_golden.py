"""Generate the golden fixtures in tests/golden from the compiled reference.

Run in a container where the reference sources exist (they do not travel to
the GPU machine):

    python oracle/build_ref.py          # compiles the reference into oracle/_ref
    python tests/golden/make_golden.py  # writes tests/golden/*.npz

Every array in the fixtures is an OUTPUT of the reference's own code
(MAS_library.MA / *c3D, Pk_library.Pk / XPk, bispectrum_library.Bk) on
seeded synthetic inputs that are stored beside it.  The inputs follow the
reference's unit tests (Test/test_MAS.py:10-84: seed 1, uniform particles in a
unit box, W = 3.0) and the benchmark workloads (1000 Mpc/h box, uniform
particles, CIC overdensity), shrunk so the fixtures stay small.
"""
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
import build_ref  # noqa: E402

MAS_LIST = ['NGP', 'CIC', 'TSC', 'PCS']


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


def edge_positions(L, N):
    """Positions on cell edges, half cells, the box origin and just below L."""
    h = np.float32(L / N)
    pts = [[0, 0, 0], [h * 0.5, h * 1.5, h * 2.5], [h, 2 * h, 3 * h],
           [L * 0.5, L * 0.25, L * 0.75], [np.nextafter(np.float32(L), np.float32(0))] * 3,
           [h * (N - 0.5), h * 0.4999, h * 0.5001]]
    return np.array(pts, dtype=np.float32)


def make_ma(MASL):
    out = {}
    # Test/test_MAS.py protocol: seed 1, 1000 particles, BoxSize 1, 64^3, W = 3
    np.random.seed(1)
    pos = np.random.random((1000, 3)).astype(np.float32)
    W = np.ones(1000, dtype=np.float32) * 3.0
    out['conservation_pos'] = pos
    for mas in MAS_LIST:
        for tag, w in (('', None), ('W', W)):
            d = np.zeros((64, 64, 64), np.float32)
            MASL.MA(pos, d, 1.0, mas, W=w)
            out['conservation_sum_%s%s' % (mas, tag)] = np.sum(d, dtype=np.float64)
    # per-cell grids on a small mesh, 3D and 2D, with and without weights
    rng = np.random.default_rng(20240601)
    N, L = 24, 1000.0
    pos = np.concatenate([(rng.random((3000, 3)) * L).astype(np.float32), edge_positions(L, N)])
    W = (rng.random(pos.shape[0]) * 3.0).astype(np.float32)
    out['grid_pos'] = pos
    out['grid_W'] = W
    out['grid_meta'] = np.array([N, L])
    for mas in MAS_LIST:
        for tag, w in (('', None), ('W', W)):
            d = np.zeros((N, N, N), np.float32)
            MASL.MA(pos, d, L, mas, W=w)
            out['MA3D_%s%s' % (mas, tag)] = d
            d2 = np.zeros((N, N), np.float32)
            MASL.MA(np.ascontiguousarray(pos[:, :2]), d2, L, mas, W=w)
            out['MA2D_%s%s' % (mas, tag)] = d2
            c = np.zeros((N, N, N), np.float32)
            fn = getattr(MASL, mas + ('Wc3D' if w is not None else 'c3D'))
            if w is None:
                fn(pos, c, L, 1)
            else:
                fn(pos, c, w, L, 1)
            out['MASc3D_%s%s' % (mas, tag)] = c
    # accumulation semantics: MA adds into a non-zero grid
    base = (rng.random((N, N, N)) * 2.0).astype(np.float32)
    out['accum_base'] = base
    d = base.copy()
    MASL.MA(pos, d, L, 'NGP')
    out['accum_NGP'] = d
    return out


def make_ma_d(MASL):
    """CICW_d / NGPW_d (float64 grids): 3D on the per-cell mesh of make_ma, 2D
    positions into a (N, N, 1) grid, and accumulation onto a non-zero base."""
    out = {}
    rng = np.random.default_rng(20240602)
    N, L = 24, 1000.0
    pos = np.concatenate([(rng.random((3000, 3)) * L).astype(np.float32), edge_positions(L, N)])
    W = (rng.random(pos.shape[0]) * 3.0).astype(np.float32)
    out['pos'] = pos
    out['W'] = W
    out['meta'] = np.array([N, L])
    base = rng.random((N, N, N))
    out['base'] = base
    for name in ('CICW_d', 'NGPW_d'):
        fn = getattr(MASL, name)
        d = np.zeros((N, N, N), np.float64)
        fn(pos, d, L, W)
        out['%s_3D' % name] = d
        d = base.copy()
        fn(pos, d, L, W)
        out['%s_3D_accum' % name] = d
        d = np.zeros((N, N, 1), np.float64)
        fn(np.ascontiguousarray(pos[:, :2]), d, L, W)
        out['%s_2D' % name] = d
    return out


def cic_overdensity(MASL, pos, N, L):
    d = np.zeros((N, N, N), np.float32)
    MASL.MA(pos, d, L, 'CIC')
    d /= np.mean(d, dtype=np.float64)
    d -= 1.0
    return d


def attrs(obj, names):
    return {n: np.asarray(getattr(obj, n)) for n in names}


PK_ATTRS = ['k1D', 'Pk1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'Nmodes2D',
            'k3D', 'Pk', 'Nmodes3D', 'Pkphase']
XPK_ATTRS = ['k1D', 'Pk1D', 'PkX1D', 'Nmodes1D', 'kpar', 'kper', 'Pk2D', 'PkX2D', 'Nmodes2D',
             'k3D', 'Pk', 'XPk', 'Nmodes3D']


def make_pk(MASL, PKL):
    out = {}
    rng = np.random.default_rng(7)
    L = 1000.0
    for N in (32, 15):
        pos = (rng.random((N ** 3 * 2, 3)) * L).astype(np.float32)
        d = cic_overdensity(MASL, pos, N, L)
        out['delta_%d' % N] = d
        for axis in (0, 1, 2):
            with quiet():
                P = PKL.Pk(d, L, axis, 'CIC', 1)
            for k, v in attrs(P, PK_ATTRS).items():
                out['Pk_%d_axis%d_%s' % (N, axis, k)] = v
        d2 = (0.5 * d + 0.2 * d * d).astype(np.float32)
        d3 = np.roll(d, 3, axis=1).astype(np.float32)
        out['delta2_%d' % N] = d2
        out['delta3_%d' % N] = d3
        with quiet():
            X = PKL.XPk([d, d2, d3], L, 1, ['CIC', 'PCS', 'NGP'], 1)
        for k, v in attrs(X, XPK_ATTRS).items():
            out['XPk_%d_%s' % (N, k)] = v
    return out


def make_bk(MASL, BKL):
    out = {}
    rng = np.random.default_rng(11)
    N, L = 32, 1000.0
    pos = (rng.random((N ** 3 * 2, 3)) * L).astype(np.float32)
    d = cic_overdensity(MASL, pos, N, L)
    out['delta'] = d
    theta = np.linspace(0, np.pi, 6)
    out['theta'] = theta
    out['meta'] = np.array([N, L, 0.05, 0.08])
    with quiet():
        B = BKL.Bk(d, L, 0.05, 0.08, theta, 'CIC', 1)
    for n in ('B', 'Q', 'k', 'Pk'):
        out['Bk_' + n] = np.asarray(getattr(B, n))
    with quiet():
        E = BKL.Bk(d, L, 0.1, 0.1, np.array([2 * np.pi / 3]), 'CIC', 1)
    for n in ('B', 'Q', 'k', 'Pk'):
        out['Bkeq_' + n] = np.asarray(getattr(E, n))
    return out


def make_interp_rsd(MASL, RSL):
    """MAS_library.CIC_interp (MAS_library.pyx:558-599) on a random 24^3 field, and
    redshift_space_library.pos_redshift_space (redshift_space_library.pyx:29-43) with
    displacements that push particles below 0 and beyond BoxSize along each axis."""
    out = {}
    rng = np.random.default_rng(31)
    N, L = 24, 1000.0
    field = rng.normal(size=(N, N, N)).astype(np.float32)
    pos = np.concatenate([(rng.random((4000, 3)) * L).astype(np.float32), edge_positions(L, N)])
    den = np.zeros(pos.shape[0], np.float32)
    MASL.CIC_interp(field, L, pos, den)
    out['interp_field'] = field
    out['interp_pos'] = pos
    out['interp_den'] = den
    out['interp_meta'] = np.array([N, L])
    vel = (rng.normal(size=(4000, 3)) * 400.0).astype(np.float32)
    rpos = (rng.random((4000, 3)) * L).astype(np.float32)
    out['rsd_pos'] = rpos
    out['rsd_vel'] = vel
    out['rsd_meta'] = np.array([L, 100.0, 0.5])
    for axis in (0, 1, 2):
        p = rpos.copy()
        RSL.pos_redshift_space(p, vel, L, 100.0, 0.5, axis)
        out['rsd_out_axis%d' % axis] = p
    return out


def make_xi(MASL, PKL):
    """Pk_library.Xi and correct_MAS (Pk_library.pyx:1749-1806, 2035-2150) on a 32^3
    CIC overdensity of 1000 Mpc/h, and on a 15^3 one (odd grid)."""
    out = {}
    rng = np.random.default_rng(41)
    L = 1000.0
    for N in (32, 15):
        pos = (rng.random((N ** 3 * 2, 3)) * L).astype(np.float32)
        d = cic_overdensity(MASL, pos, N, L)
        out['delta_%d' % N] = d
        for axis in (0, 2):
            with quiet():
                X = PKL.Xi(d, L, 'CIC', axis, 1)
            out['Xi_%d_axis%d_r3D' % (N, axis)] = np.asarray(X.r3D)
            out['Xi_%d_axis%d_xi' % (N, axis)] = np.asarray(X.xi)
            out['Xi_%d_axis%d_Nmodes3D' % (N, axis)] = np.asarray(X.Nmodes3D)
        with quiet():
            out['correct_MAS_%d' % N] = np.asarray(PKL.correct_MAS(d, L, 'CIC', 1))
    return out


def make_plane(MASL, PKL):
    """Pk_library.Pk_plane / XPk_plane (Pk_library.pyx:440-516, 814-941) on 2D CIC
    maps of 64^2 and 45^2 cells (1000 Mpc/h)."""
    out = {}
    rng = np.random.default_rng(51)
    L = 1000.0
    for N in (64, 45):
        pos = (rng.random((N * N * 4, 2)) * L).astype(np.float32)
        a = np.zeros((N, N), np.float32)
        MASL.MA(pos, a, L, 'CIC')
        a /= np.mean(a, dtype=np.float64); a -= 1.0
        b = (0.7 * a + 0.3 * np.roll(a, 2, axis=0)).astype(np.float32)
        out['map1_%d' % N], out['map2_%d' % N] = a, b
        with quiet():
            P = PKL.Pk_plane(a, L, 'CIC', 1)
            X = PKL.XPk_plane(a, b, L, 'CIC', 'TSC', 1)
        for n in ('k', 'Nmodes', 'Pk'):
            out['Pkplane_%d_%s' % (N, n)] = np.asarray(getattr(P, n))
        for n in ('k', 'Nmodes', 'Pk', 'XPk', 'r'):
            out['XPkplane_%d_%s' % (N, n)] = np.asarray(getattr(X, n))
    return out


def make_smoothing(MASL):
    """smoothing_library.FT_filter and field_smoothing (smoothing_library.pyx:20-114):
    Top-Hat and Gaussian filters on 32^3 and 15^3 grids, applied to a CIC field."""
    SL = build_ref.load_smoothing()
    out = {}
    rng = np.random.default_rng(61)
    L = 1000.0
    for N in (32, 15):
        pos = (rng.random((N ** 3 * 2, 3)) * L).astype(np.float32)
        d = cic_overdensity(MASL, pos, N, L)
        out['field_%d' % N] = d
        for filt, R in (('Top-Hat', 100.0), ('Gaussian', 60.0)):
            with quiet():
                fk = np.asarray(SL.FT_filter(L, R, N, filt, 1))
                sm = np.asarray(SL.field_smoothing(d, fk, 1))
            tag = filt.replace('-', '')
            out['filter_%s_%d' % (tag, N)] = fk
            out['smoothed_%s_%d' % (tag, N)] = sm
    return out


def main(which=('ma', 'ma_d', 'pk', 'bk', 'interp', 'xi', 'plane', 'smoothing')):
    if not build_ref.built():
        build_ref.build()
    MASL, PKL, BKL = build_ref.load_reference()
    if 'ma' in which:
        np.savez_compressed(os.path.join(HERE, 'ma_golden.npz'), **make_ma(MASL))
    if 'ma_d' in which:
        np.savez_compressed(os.path.join(HERE, 'ma_d_golden.npz'), **make_ma_d(MASL))
    if 'pk' in which:
        np.savez_compressed(os.path.join(HERE, 'pk_golden.npz'), **make_pk(MASL, PKL))
    if 'bk' in which:
        np.savez_compressed(os.path.join(HERE, 'bk_golden.npz'), **make_bk(MASL, BKL))
    if 'smoothing' in which:
        np.savez_compressed(os.path.join(HERE, 'smoothing_golden.npz'), **make_smoothing(MASL))
    if 'plane' in which:
        np.savez_compressed(os.path.join(HERE, 'plane_golden.npz'), **make_plane(MASL, PKL))
    if 'xi' in which:
        np.savez_compressed(os.path.join(HERE, 'xi_golden.npz'), **make_xi(MASL, PKL))
    if 'interp' in which:
        RSL = build_ref.load_redshift_space()
        np.savez_compressed(os.path.join(HERE, 'interp_golden.npz'), **make_interp_rsd(MASL, RSL))
    for f in sorted(os.listdir(HERE)):
        if f.endswith('.npz'):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == '__main__':
    main(tuple(sys.argv[1:]) or ('ma', 'ma_d', 'pk', 'bk', 'interp', 'xi', 'plane', 'smoothing'))
