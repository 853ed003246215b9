"""The Zel'dovich + redshift-space workload (a 256^3 Gaussian field with
P ~ k^-1.5 exp(-(k/0.5)^2), sigma 0.5, 512^3 lattice particles, f = 0.5 along
axis 2), shrunk to a 32^3 field and 64^3 particles: TSC and PCS with and
without interlacing, P(k) l=0,2,4 and Pk2D along the distortion axis, and XPk
against the NGP field, each against the oracle on the same particles."""
import numpy as np
import pytest
import torch

import oracle as O
from test_gpu_pk import PK_NAMES, XPK_NAMES, check_pk

pytestmark = pytest.mark.gpu

L = 300.0
N = 64


@pytest.fixture(scope='module')
def parts():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import synthetic
    pos = synthetic.zeldovich(N_field=32, N_lattice=64, BoxSize=L, sigma=0.5, f=0.5, rsd_axis=2, seed=3)
    return pos, pos.cpu().numpy()


def oracle_delta(pos, mas, shift=False):
    p = (pos + np.float32(0.5 * L / N)).astype(np.float32) if shift else pos
    g = np.zeros((N, N, N), np.float32)
    O.MA(p, g, L, mas)
    g /= np.float32(pos.shape[0] / N ** 3)
    g -= np.float32(1.0)
    return g


def test_displaced_particles_are_in_the_box(parts):
    pos, host = parts
    assert host.shape == (64 ** 3, 3)
    assert host.min() >= 0.0 and host.max() < L
    # the lattice is displaced (not a uniform grid any more) by a few Mpc/h
    lattice = (np.indices((64, 64, 64)).reshape(3, -1).T + 0.5) * (L / 64)
    d = np.abs(host - lattice)
    d = np.minimum(d, L - d)
    assert 0.1 < np.sqrt((d ** 2).sum(1).mean()) < 30.0


@pytest.mark.parametrize('mas', ['TSC', 'PCS'])
@pytest.mark.parametrize('inter', [False, True])
def test_zeldovich_pk_vs_oracle(parts, mas, inter):
    from pylians_gb300.pipeline import ParticlePk
    pos, host = parts
    pp = ParticlePk(N, L, mas, axis=2, interlaced=inter, max_particles=pos.shape[0])
    pp.step(pos)
    r = pp.result()
    a = oracle_delta(host, mas)
    o = O.Pk(a, L, 2, mas, 1, interlaced=oracle_delta(host, mas, True) if inter else None)
    # A displaced lattice has almost no power past its 32^3 field's Nyquist frequency:
    # there the bins hold 1e-5..1e-6 of the peak, near-cancellations (interlacing, the
    # PCS window) of float32 round-off that differs between the two deposits, and the
    # phases of such modes are noise.  Floor 1e-6 of the peak; Pkphase left out.
    check_pk(r, lambda n: getattr(o, n), [n for n in PK_NAMES if n != 'Pkphase'], floor=1e-6)
    # redshift-space distortion: a positive quadrupole on large scales
    assert np.mean(r.Pk[:8, 1]) > 0


def test_zeldovich_xpk_against_ngp(parts):
    import pylians_gb300.Pk_library as PKL
    _, host = parts
    a = oracle_delta(host, 'TSC')
    b = oracle_delta(host, 'NGP')
    r = PKL.XPk([torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()], L, 2, ['TSC', 'NGP'])
    o = O.XPk([a, b], L, 2, ['TSC', 'NGP'], 1)
    check_pk(r, lambda n: getattr(o, n), XPK_NAMES, cross=True, floor=1e-6)


@pytest.mark.parametrize('strategy', ['auto', 'atomic'])
def test_rsd_fused_into_deposit(strategy):
    """ParticlePk.step(pos, rsd=...) shifts the positions in place exactly like
    pos_redshift_space (fused into the histogram pass on the tiled path, a pass of
    its own otherwise) and deposits the shifted particles."""
    from pylians_gb300.pipeline import ParticlePk
    import pylians_gb300.redshift_space_library as RSL
    rng = np.random.default_rng(33)
    n, N, Lb = 1_200_000, 96, 500.0
    pos = torch.from_numpy((rng.random((n, 3)) * Lb).astype(np.float32)).cuda()
    vel = torch.from_numpy((rng.normal(size=(n, 3)) * 500.0).astype(np.float32)).cuda()
    a, b = pos.clone(), pos.clone()
    p1 = ParticlePk(N, Lb, 'CIC', axis=2, interlaced=True, strategy=strategy, max_particles=n)
    p1.step(a, rsd=(vel, 100.0, 0.5, 2))
    RSL.pos_redshift_space(b, vel, Lb, 100.0, 0.5, 2)
    p2 = ParticlePk(N, Lb, 'CIC', axis=2, interlaced=True, strategy=strategy, max_particles=n)
    p2.step(b)
    assert torch.equal(a, b)
    r1, r2 = p1.result(), p2.result()
    np.testing.assert_array_equal(r1.Nmodes3D, r2.Nmodes3D)
    np.testing.assert_allclose(r1.Pk, r2.Pk, rtol=1e-5, atol=1e-6 * np.abs(r2.Pk[:, 0]).max())
