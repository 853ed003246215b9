"""Oracle for Pylians' density-field and clustering path: MA, Pk, XPk, Bk on the CPU.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference legs of ``bench.py`` use this module, as the reference
results the GPU path is compared with and as the timed CPU baseline.  The product (``pylians_gb300``) never imports it.

The hot loops are the plain-C restatement in ``pyl_oracle.c`` (mass assignment,
P(k) mode loop); this file restates the rest in numpy, each part citing the
reference lines it follows:

  MA()                MAS_library.pyx:57-112 (dispatch, 2D renormalisation)
  ma_acc64()          the same weights summed in float64 (no accumulation rounding)
  ma_f64()            CICW_d MAS_library.pyx:229-266, NGPW_d :338-358 (float64 grids)
  frequencies()       Pk_library.pyx:59-64
  MAS_function()      Pk_library.pyx:75-81
  check_number_modes  Pk_library.pyx:90-102
  FFT3Dr_f/IFFT3Dr_f  Pk_library.pyx:120-133,152-165 (unnormalised, float32)
  Pk                  Pk_library.pyx:266-425
  XPk                 Pk_library.pyx:534-798
  Bk                  bispectrum_library.pyx:32-196

The FFT is ``scipy.fft`` in float32.  The reference's FFT is pyFFTW/FFTW3,
which is not vendored and is pinned to no version; FFT parity is therefore
pinned only against scipy.fft (float32) and numpy's float64 FFT, within the
tolerance each test states.

Interlacing has no counterpart in the reference.  Its oracle is this file's
``interlace_combine``: the reference mass assignment run on positions shifted
by half a cell, combined in Fourier space as
    delta(k) = 1/2 [delta_1(k) + delta_2(k) exp(i pi (kx+ky+kz)/N)]
(Sefusatti, Crocce, Scoccimarro & Couchman 2016, MNRAS 460, 3624).
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, 'liboracle_pyl.so')
_lib = None

MAS_INDEX = {'NGP': 1, 'CIC': 2, 'TSC': 3, 'PCS': 4}


def build(force=False):
    """Compile pyl_oracle.c into oracle/liboracle_pyl.so (gcc, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, 'pyl_oracle.c')
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    cmd = ['gcc', '-O2', '-fopenmp', '-ffp-contract=off', '-fPIC', '-shared',
           src, '-o', _LIB_PATH + '.tmp', '-lm']
    subprocess.check_call(cmd)
    os.replace(_LIB_PATH + '.tmp', _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.oracle_ma.argtypes = [P, ctypes.c_int64, ctypes.c_int, P, ctypes.c_int, ctypes.c_float,
                                ctypes.c_int, P, ctypes.c_int, ctypes.c_int]
        L.oracle_ma.restype = ctypes.c_int
        L.oracle_ma_acc64.argtypes = L.oracle_ma.argtypes
        L.oracle_ma_acc64.restype = ctypes.c_int
        L.oracle_pk_modes.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int] + [P] * 12
        L.oracle_pk_modes.restype = ctypes.c_int
        L.oracle_cic_interp.argtypes = [P, ctypes.c_int, ctypes.c_float, P, ctypes.c_int64, P]
        L.oracle_cic_interp.restype = None
        L.oracle_rsd.argtypes = [P, P, ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_int]
        L.oracle_rsd.restype = None
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# --------------------------------------------------------------------------- MA
def ma_kernel(pos, number, BoxSize, MAS, W=None, threads=1, flavor=0):
    """One deposit pass (no 2D renormalisation).  flavor 0: MAS_library.pyx kernels;
    flavor 1: MAS_c.c kernels (threads>1 uses OpenMP atomics as MAS_c.c does)."""
    assert pos.dtype == np.float32 and pos.flags.c_contiguous
    assert number.dtype == np.float32 and number.flags.c_contiguous
    ndim = pos.shape[1]
    assert number.ndim == ndim
    w = None
    if W is not None:
        w = np.ascontiguousarray(W, dtype=np.float32)
        assert w.shape[0] == pos.shape[0]
    rc = lib().oracle_ma(_ptr(pos), pos.shape[0], ndim, _ptr(number), number.shape[0],
                         float(BoxSize), MAS_INDEX[MAS], _ptr(w), int(threads), int(flavor))
    if rc:
        raise ValueError('oracle_ma failed (%d)' % rc)


def ma_acc64(pos, number, BoxSize, MAS, W=None, threads=1):
    """ma_kernel (flavor 0, 3D) with the reference's float32 weights and products added
    to the float64 grid ``number``: no float32 accumulation rounding."""
    assert pos.dtype == np.float32 and pos.flags.c_contiguous and pos.shape[1] == 3
    assert number.dtype == np.float64 and number.flags.c_contiguous and number.ndim == 3
    w = None if W is None else np.ascontiguousarray(W, dtype=np.float32)
    rc = lib().oracle_ma_acc64(_ptr(pos), pos.shape[0], 3, _ptr(number), number.shape[0], float(BoxSize),
                               MAS_INDEX[MAS], _ptr(w), int(threads), 0)
    if rc:
        raise ValueError('oracle_ma_acc64 failed (%d)' % rc)


def ma_f64(pos, number, BoxSize, MAS, W):
    """CICW_d / NGPW_d (MAS_library.pyx:229-266, :338-358) in numpy: float32 weights and
    products as the compiled reference evaluates them, added to the float64 grid number[dims][dims][depth]
    in the reference's serial order (particle by particle, corners in its order).  2D positions
    keep the third index at 0 with weight 1.0 on both CIC sides."""
    assert pos.dtype == np.float32 and number.dtype == np.float64 and number.ndim == 3
    n, coord = pos.shape
    dims, depth = number.shape[0], number.shape[2]
    inv = np.float32(dims) / np.float32(BoxSize)
    W = np.asarray(W, dtype=np.float32)
    flat = number.reshape(-1)
    if MAS == 'NGP':
        idx = np.zeros((n, 3), np.int64)
        for a in range(coord):
            k = np.trunc((pos[:, a] * inv).astype(np.float64) + 0.5).astype(np.int64)
            idx[:, a] = np.mod(k, dims)
        np.add.at(flat, (idx[:, 0] * dims + idx[:, 1]) * depth + idx[:, 2], W.astype(np.float64))
        return
    if MAS != 'CIC':
        raise ValueError('the reference has CICW_d and NGPW_d only')
    lo = np.zeros((n, 3), np.int64)
    hi = np.zeros((n, 3), np.int64)
    d = np.ones((n, 3), np.float32)
    u = np.ones((n, 3), np.float32)
    for a in range(coord):
        dist = (pos[:, a] * inv).astype(np.float32)
        k = np.trunc(dist).astype(np.int64)
        u[:, a] = (dist - k.astype(np.float32)).astype(np.float32)
        d[:, a] = (np.float32(1.0) - u[:, a]).astype(np.float32)
        lo[:, a] = np.mod(k, dims)
        hi[:, a] = np.mod(lo[:, a] + 1, dims)
    idxs, vals = [], []
    for cx, ix in ((d[:, 0], lo[:, 0]), (u[:, 0], hi[:, 0])):
        for cy, iy in ((d[:, 1], lo[:, 1]), (u[:, 1], hi[:, 1])):
            for cz, iz in ((d[:, 2], lo[:, 2]), (u[:, 2], hi[:, 2])):
                idxs.append((ix * dims + iy) * depth + iz)
                # (d0 d1)(d2 W): the association the reference's -ffast-math build evaluates
                # (its source reads left to right; the compiled golden grids pin this order)
                vals.append(((cx * cy).astype(np.float32) * (cz * W).astype(np.float32)).astype(np.float32))
    order = np.stack(idxs, axis=1).reshape(-1)       # particle-major, corners in the reference's order
    np.add.at(flat, order, np.stack(vals, axis=1).reshape(-1).astype(np.float64))


def MA(pos, number, BoxSize, MAS='CIC', W=None, renormalize_2D=True, threads=1):
    """MAS_library.MA (MAS_library.pyx:57-112): accumulate into ``number`` in place."""
    if pos.shape[1] != number.ndim:
        raise ValueError('pos have %d dimensions and the density %d' % (pos.shape[1], number.ndim))
    if MAS not in MAS_INDEX:
        raise ValueError('option not valid: MAS=%r' % (MAS,))
    ma_kernel(pos, number, BoxSize, MAS, W, threads=threads, flavor=0)
    if number.ndim == 2 and renormalize_2D and MAS != 'NGP':
        number /= {'CIC': 2.0, 'TSC': 3.0, 'PCS': 4.0}[MAS]


def CIC_interp(density, BoxSize, pos, den):
    """MAS_library.CIC_interp (MAS_library.pyx:558-599): den[i] <- CIC value at pos[i]."""
    assert density.dtype == np.float32 and density.flags.c_contiguous and density.ndim == 3
    assert pos.dtype == np.float32 and pos.flags.c_contiguous and den.dtype == np.float32
    lib().oracle_cic_interp(_ptr(density), density.shape[0], float(BoxSize), _ptr(pos), pos.shape[0], _ptr(den))


def pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis):
    """redshift_space_library.pos_redshift_space (redshift_space_library.pyx:29-43), in place."""
    assert pos.dtype == np.float32 and pos.flags.c_contiguous and vel.dtype == np.float32
    assert vel.flags.c_contiguous and vel.shape == pos.shape
    lib().oracle_rsd(_ptr(pos), _ptr(vel), pos.shape[0], float(BoxSize), float(Hubble), float(redshift), int(axis))


# ------------------------------------------------------------------ P(k) pieces
def frequencies(BoxSize, dims):
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    kmax_par = middle
    kmax_per = int(np.sqrt(middle ** 2 + middle ** 2))
    kmax = int(np.sqrt(middle ** 2 + middle ** 2 + middle ** 2))
    return kF, kN, kmax_par, kmax_per, kmax


def MAS_function(MAS):
    return MAS_INDEX.get(MAS, 0)


def check_number_modes(Nmodes, dims):
    own = 1 if dims % 2 == 1 else 8
    indep = (dims ** 3 - own) // 2 + own
    if int(np.sum(Nmodes)) != indep:
        raise RuntimeError('Not all modes counted: %d vs %d' % (int(np.sum(Nmodes)), indep))


def fft_r2c(delta, threads=1):
    import scipy.fft
    return scipy.fft.rfftn(np.asarray(delta, dtype=np.float32), workers=max(1, threads))


def fft_c2r(dk, dims, threads=1):
    import scipy.fft
    return scipy.fft.irfftn(np.asarray(dk, dtype=np.complex64), s=(dims,) * 3, norm='forward',
                            workers=max(1, threads))


def interlace_combine(dk1, dk2):
    """1/2 [dk1 + dk2 exp(i pi (kx+ky+kz)/N)] on the half-complex grid, phase in float64.
    The frequencies are the reference's: index i > N/2 means i - N, so the Nyquist
    index N/2 of an even grid is +N/2."""
    dims = dk1.shape[0]
    middle = dims // 2
    k = np.arange(dims)
    k = np.where(k > middle, k - dims, k)      # the reference's signed frequency (Pk_library.pyx:315)
    kz = np.arange(dims // 2 + 1)
    out = np.empty(dk1.shape, np.complex64)
    step = max(1, (1 << 24) // (dims * (dims // 2 + 1)))      # x slabs of ~16M modes (bounded memory)
    for x0 in range(0, dims, step):
        x1 = min(dims, x0 + step)
        ph = np.pi / dims * (k[x0:x1, None, None] + k[None, :, None] + kz[None, None, :])
        out[x0:x1] = 0.5 * (dk1[x0:x1].astype(np.complex128) + dk2[x0:x1].astype(np.complex128) * np.exp(1j * ph))
    return out


def pk_mode_sums(dk_fields, axis, mas_p, threads=1):
    """Raw per-bin sums of the Pk/XPk mode loop.  ``dk_fields`` is modified (MAS-corrected)."""
    F = len(dk_fields)
    dims = dk_fields[0].shape[0]
    kF, kN, kmax_par, kmax_per, kmax = frequencies(1.0, dims)
    nb1, nb2, nb3 = kmax_par + 1, (kmax_par + 1) * (kmax_per + 1), kmax + 1
    X = F * (F - 1) // 2
    if F == 1 and dk_fields[0].dtype == np.complex64 and dk_fields[0].flags.c_contiguous:
        dk = dk_fields[0][None]                        # no copy of a large single field
    else:
        dk = np.ascontiguousarray(np.stack(dk_fields).astype(np.complex64))
    z = lambda *s: np.zeros(s, np.float64)
    out = dict(k1D=z(nb1), Nmodes1D=z(nb1), Pk1D=z(nb1, F), PkX1D=z(nb1, max(X, 1)),
               Nmodes2D=z(nb2), Pk2D=z(nb2, F), PkX2D=z(nb2, max(X, 1)),
               k3D=z(nb3), Nmodes3D=z(nb3), Pk3D=z(nb3, 3, F), PkX3D=z(nb3, 3, max(X, 1)),
               Pkphase=z(nb3, F))
    mp = np.asarray(mas_p, dtype=np.int32)
    names = ['k1D', 'Nmodes1D', 'Pk1D', 'PkX1D', 'Nmodes2D', 'Pk2D', 'PkX2D',
             'k3D', 'Nmodes3D', 'Pk3D', 'PkX3D', 'Pkphase']
    rc = lib().oracle_pk_modes(_ptr(dk), F, dims, int(axis), _ptr(mp), int(threads),
                               *[_ptr(out[n]) for n in names])
    if rc:
        raise RuntimeError('oracle_pk_modes failed (%d)' % rc)
    out['delta_k'] = dk
    return out


class _Result(object):
    pass


def finalize_pk(s, BoxSize, dims, F, cross=False):
    """Finalisation of Pk (Pk_library.pyx:384-421) and XPk (:740-796) in float64."""
    kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
    fact = (BoxSize / dims ** 2) ** 3
    X = F * (F - 1) // 2
    r = _Result()
    with np.errstate(divide='ignore', invalid='ignore'):
        k1D = s['k1D'][1:].copy(); N1 = s['Nmodes1D'][1:].copy()
        k1D = (k1D / N1) * kF
        kmaxper = np.sqrt(kN ** 2 - k1D ** 2)
        area = (np.pi * kmaxper ** 2 / N1) / (2.0 * np.pi) ** 2
        Pk1D = s['Pk1D'][1:] * fact * area[:, None]
        PkX1D = s['PkX1D'][1:, :X] * fact * area[:, None]
        ip = np.arange(kmax_par + 1); iq = np.arange(kmax_per + 1)
        kpar = np.zeros((kmax_par + 1) * (kmax_per + 1)); kper = np.zeros_like(kpar)
        idx = (kmax_par + 1) * iq[None, :] + ip[:, None]
        kpar[idx] = (0.5 * (ip + ip + 1) * kF)[:, None]
        kper[idx] = (0.5 * (iq + iq + 1) * kF)[None, :]
        N2 = s['Nmodes2D']
        Pk2D = s['Pk2D'] * fact / N2[:, None]
        PkX2D = s['PkX2D'][:, :X] * fact / N2[:, None]
        check_number_modes(s['Nmodes3D'], dims)
        N3 = s['Nmodes3D'][1:].copy()
        k3D = (s['k3D'][1:] / N3) * kF
        P3 = s['Pk3D'][1:].copy()
        P3[:, 0] = (P3[:, 0] / N3[:, None]) * fact
        P3[:, 1] = (P3[:, 1] * 5.0 / N3[:, None]) * fact
        P3[:, 2] = (P3[:, 2] * 9.0 / N3[:, None]) * fact
        X3 = s['PkX3D'][1:, :, :X].copy()
        X3[:, 0] = (X3[:, 0] / N3[:, None]) * fact
        X3[:, 1] = (X3[:, 1] * 5.0 / N3[:, None]) * fact
        X3[:, 2] = (X3[:, 2] * 9.0 / N3[:, None]) * fact
        ph = (s['Pkphase'][1:] / N3[:, None]) * fact
    r.k1D, r.Nmodes1D = k1D, N1
    r.kpar, r.kper, r.Nmodes2D = kpar, kper, N2.copy()
    r.k3D, r.Nmodes3D = k3D, N3
    if cross:
        r.Pk1D, r.PkX1D, r.Pk2D, r.PkX2D = Pk1D, PkX1D, Pk2D, PkX2D
        r.Pk, r.XPk = P3, X3
    else:
        r.Pk1D, r.Pk2D, r.Pk, r.Pkphase = Pk1D[:, 0], Pk2D[:, 0], P3[:, :, 0], ph[:, 0]
    return r


def Pk(delta, BoxSize, axis=2, MAS='CIC', threads=1, keep_deltak=False, interlaced=None):
    """Pk_library.Pk (Pk_library.pyx:266-425); ``interlaced`` is the half-cell-shifted grid."""
    dims = delta.shape[0]
    dk = fft_r2c(delta, threads)
    if interlaced is not None:
        dk = interlace_combine(dk, fft_r2c(interlaced, threads))
    s = pk_mode_sums([dk], axis, [MAS_function(MAS)], threads)
    r = finalize_pk(s, BoxSize, dims, 1)
    if keep_deltak:
        r.delta_k = s['delta_k'][0]
    return r


def XPk(delta, BoxSize, axis=2, MAS=None, threads=1, interlaced=None):
    """Pk_library.XPk (Pk_library.pyx:534-798)."""
    F = len(delta)
    dims = delta[0].shape[0]
    for d in delta[1:]:
        if d.shape[0] != dims:
            raise ValueError('Fields have different grid sizes')
    dks = [fft_r2c(d, threads) for d in delta]
    if interlaced is not None:
        dks = [interlace_combine(a, fft_r2c(b, threads)) for a, b in zip(dks, interlaced)]
    s = pk_mode_sums(dks, axis, [MAS_function(m) for m in MAS], threads)
    return finalize_pk(s, BoxSize, dims, F, cross=True)


# -------------------------------------------------------------------- bispectrum
def mas_factor_grid(dims, MAS):
    """float32 MAS factor on the half-complex grid: (float)(C(kx) C(ky) C(kz)), C in float64."""
    p = MAS_function(MAS)
    middle = dims // 2
    k = np.arange(dims); k = np.where(k > middle, k - dims, k)
    x = (np.pi / dims) * k
    with np.errstate(divide='ignore', invalid='ignore'):
        c = np.where(x == 0.0, 1.0, (x / np.sin(x)) ** p)
    cz = c[:middle + 1]
    return ((c[:, None, None] * c[None, :, None]) * cz[None, None, :]).astype(np.float32)


def mode_k2(dims):
    middle = dims // 2
    k = np.arange(dims); k = np.where(k > middle, k - dims, k).astype(np.int64)
    kz = np.arange(middle + 1, dtype=np.int64)
    return k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2


def Bk(delta, BoxSize, k1, k2, theta, MAS='CIC', threads=1):
    """Pk_library.Bk (bispectrum_library.pyx:32-196)."""
    dims = delta.shape[0]
    kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
    theta = np.asarray(theta, dtype=np.float64)
    bins = theta.shape[0]
    k3 = np.sqrt((k2 * np.sin(theta)) ** 2 + (k2 * np.cos(theta) + k1) ** 2)
    k_all = np.zeros(bins + 2); k_all[0] = k1; k_all[1] = k2; k_all[2:] = k3
    k_min = (k_all - kF) / kF
    k_max = (k_all + kF) / kF
    dk = fft_r2c(delta, threads)
    mf = mas_factor_grid(dims, MAS)
    dk = (dk.real * mf + 1j * (dk.imag * mf)).astype(np.complex64)
    kk = np.sqrt(mode_k2(dims).astype(np.float64))

    def shell(i):
        m = (kk >= k_min[i]) & (kk < k_max[i])
        d = np.where(m, dk, 0).astype(np.complex64)
        I = m.astype(np.complex64)
        return fft_c2r(d, dims, threads), fft_c2r(I, dims, threads)

    fact_p = (BoxSize / dims ** 2) ** 3
    fact_b = (BoxSize ** 2 / dims ** 3) ** 3
    Pk = np.zeros(bins + 2)
    B = np.zeros(bins); Q = np.zeros(bins)
    d1, I1 = shell(0)
    Pk[0] = np.sum((d1 * d1).astype(np.float64)) / np.sum((I1 * I1).astype(np.float64)) * fact_p
    d2, I2 = shell(1)
    Pk[1] = np.sum((d2 * d2).astype(np.float64)) / np.sum((I2 * I2).astype(np.float64)) * fact_p
    d12 = d1 * d2
    I12 = I1 * I2
    for j in range(bins):
        d3, I3 = shell(j + 2)
        Pk[j + 2] = (np.sum((d3 * d3).astype(np.float64)) /
                     np.sum((I3 * I3).astype(np.float64))) * fact_p
        B[j] = (np.sum((d12 * d3).astype(np.float64)) / np.sum((I12 * I3).astype(np.float64))) * fact_b
        Q[j] = B[j] / (Pk[0] * Pk[1] + Pk[0] * Pk[j + 2] + Pk[1] * Pk[j + 2])
    r = _Result()
    r.B, r.Q, r.k, r.Pk = B, Q, k_all, Pk
    return r


if __name__ == '__main__':
    print(build(force='--force' in sys.argv))


# ----------------------------------------------------- MLP (learned correction)
# float64 restatement of the 4 -> 64 -> 64 -> 64 -> 1 tanh network of the
# learned aliasing correction (no counterpart in the reference): the values the
# GPU forward/backward kernels' outputs and gradients are compared with.
MLP_SHAPES = [('W1', (64, 4)), ('b1', (64,)), ('W2', (64, 64)), ('b2', (64,)),
              ('W3', (64, 64)), ('b3', (64,)), ('W4', (1, 64)), ('b4', (1,))]


def mlp_unpack(flat):
    out, o = {}, 0
    for name, shp in MLP_SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(flat[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def mlp_forward_backward(flat, x, t, w=None):
    """Loss sum_s w_s (y_s - t_s)^2 / sum_s w_s, its gradient (flat, float64) and y."""
    p = mlp_unpack(flat)
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    w = np.ones_like(t) if w is None else np.asarray(w, np.float64)
    h1 = np.tanh(x @ p['W1'].T + p['b1'])
    h2 = np.tanh(h1 @ p['W2'].T + p['b2'])
    h3 = np.tanh(h2 @ p['W3'].T + p['b3'])
    y = (h3 @ p['W4'].T + p['b4'])[:, 0]
    ws = w.sum()
    loss = np.sum(w * (y - t) ** 2) / ws
    dy = 2.0 * w * (y - t) / ws
    g = {}
    g['W4'] = dy[None, :] @ h3
    g['b4'] = np.array([dy.sum()])
    d3 = (dy[:, None] * p['W4']) * (1 - h3 ** 2)
    g['W3'] = d3.T @ h2
    g['b3'] = d3.sum(0)
    d2 = (d3 @ p['W3']) * (1 - h2 ** 2)
    g['W2'] = d2.T @ h1
    g['b2'] = d2.sum(0)
    d1 = (d2 @ p['W2']) * (1 - h1 ** 2)
    g['W1'] = d1.T @ x
    g['b1'] = d1.sum(0)
    grad = np.concatenate([g[name].ravel() for name, _ in MLP_SHAPES])
    return loss, grad, y


# ------------------------------------------------------------ correct_MAS / Xi
def _freqs(dims):
    """Signed frequency of each index, index dims/2 -> +dims/2 (Pk_library.pyx:1780)."""
    i = np.arange(dims)
    return np.where(i > dims // 2, i - dims, i)


def _mas_factor(dims, p):
    """float32 MAS factor of every stored half-complex mode: the float64 product of
    the three axis factors, rounded once (Pk_library.pyx:1779-1794, 2067-2077)."""
    f = _freqs(dims)
    fz = np.arange(dims // 2 + 1)
    def c(k):
        x = np.pi * k / dims
        with np.errstate(invalid='ignore', divide='ignore'):
            r = np.where(k == 0, 1.0, x / np.sin(np.where(k == 0, 1.0, x)))
        return r ** p if p else np.ones_like(x, dtype=np.float64)
    return (c(f)[:, None, None] * c(f)[None, :, None] * c(fz)[None, None, :]).astype(np.float32)


def correct_MAS(delta, BoxSize, MAS='CIC', threads=1):
    """Pk_library.correct_MAS (Pk_library.pyx:1749-1806): the mode loop skips the
    redundant half of the kz = 0 and kz = N/2 planes (:1789-1792), then a normalised
    C2R."""
    import scipy.fft
    dims = delta.shape[0]
    dk = fft_r2c(delta, threads)
    f, fz = _freqs(dims), np.arange(dims // 2 + 1)
    kx, ky, kz = np.meshgrid(f, f, fz, indexing='ij')
    even = dims % 2 == 0
    plane = (kz == 0) | ((kz == dims // 2) & even)
    skip = plane & ((kx < 0) | (((kx == 0) | ((kx == dims // 2) & even)) & (ky < 0)))
    dk = np.where(skip, dk, dk * _mas_factor(dims, MAS_function(MAS))).astype(np.complex64)
    return scipy.fft.irfftn(dk, s=delta.shape, workers=max(1, threads)).astype(np.float32)


def Xi(delta, BoxSize, MAS='CIC', axis=2, threads=1):
    """Pk_library.Xi (Pk_library.pyx:2035-2150) restated with numpy."""
    import scipy.fft
    dims = delta.shape[0]
    dk = fft_r2c(delta, threads)
    dk = (dk * _mas_factor(dims, MAS_function(MAS))).astype(np.complex64)
    p = (dk.real * dk.real + dk.imag * dk.imag).astype(np.float32)
    xi = scipy.fft.irfftn(p.astype(np.complex64), s=delta.shape, workers=max(1, threads)).astype(np.float32)
    f = _freqs(dims)
    kx, ky, kz = np.meshgrid(f, f, f, indexing='ij')
    k2 = kx * kx + ky * ky + kz * kz
    k = np.sqrt(k2.astype(np.float64))
    idx = np.floor(k + 1e-9).astype(np.int64)
    idx = np.where((idx + 1) ** 2 <= k2, idx + 1, idx)
    idx = np.where(idx ** 2 > k2, idx - 1, idx)
    par = (kx, ky, kz)[axis].astype(np.float64)
    with np.errstate(invalid='ignore', divide='ignore'):
        mu = np.where(k == 0, 0.0, par / np.where(k == 0, 1.0, k))
    mu2 = mu * mu
    nb = int(np.sqrt(3.0 * (dims // 2) ** 2)) + 1
    x = xi.astype(np.float64).ravel()
    i = idx.ravel()
    r3D = np.bincount(i, k.ravel(), nb)
    N = np.bincount(i, None, nb).astype(np.float64)
    X0 = np.bincount(i, x, nb)
    X2 = np.bincount(i, x * (3.0 * mu2.ravel() - 1.0) / 2.0, nb)
    X4 = np.bincount(i, x * (35.0 * mu2.ravel() ** 2 - 30.0 * mu2.ravel() + 3.0) / 8.0, nb)
    r = _Result()
    N1 = N[1:]
    r.r3D = r3D[1:] / N1 * (BoxSize * 1.0 / dims)
    r.Nmodes3D = N1
    r.xi = np.stack([X0[1:] / N1, X2[1:] * 5.0 / N1, X4[1:] * 9.0 / N1], axis=1) / float(dims) ** 3
    return r


# ------------------------------------------------------------------- 2D maps
def _plane(maps, BoxSize, mas_list):
    """Sums of Pk_plane / XPk_plane (Pk_library.pyx:440-516, 814-941) with numpy."""
    import scipy.fft
    dims = maps[0].shape[0]
    middle = dims // 2
    f, fy = _freqs(dims), np.arange(dims // 2 + 1)
    kx, ky = np.meshgrid(f, fy, indexing='ij')
    even = dims % 2 == 0
    keep = ~(((ky == 0) | ((ky == middle) & even)) & (kx < 0))
    n2 = kx * kx + ky * ky
    k = np.sqrt(n2.astype(np.float64))
    idx = np.floor(k + 1e-9).astype(np.int64)
    idx = np.where(idx * idx > n2, idx - 1, idx)
    nb = int(np.sqrt(middle ** 2 + middle ** 2)) + 1
    dks = []
    for m, mas in zip(maps, mas_list):
        dk = scipy.fft.rfftn(np.asarray(m, np.float32))
        p = MAS_function(mas)
        def c(q):
            x = np.pi * q / dims
            with np.errstate(invalid='ignore', divide='ignore'):
                r = np.where(q == 0, 1.0, x / np.sin(np.where(q == 0, 1.0, x)))
            return r ** p if p else np.ones_like(x, dtype=np.float64)
        fac = (c(f)[:, None] * c(fy)[None, :]).astype(np.float32)
        dks.append((dk * fac).astype(np.complex64))
    i = idx[keep]
    K = np.bincount(i, k[keep], nb)
    N = np.bincount(i, None, nb).astype(np.float64)
    P = [np.bincount(i, (d.real.astype(np.float64) ** 2 + d.imag.astype(np.float64) ** 2)[keep], nb) for d in dks]
    X = None
    if len(dks) > 1:
        a, b = dks
        X = np.bincount(i, (a.real.astype(np.float64) * b.real + a.imag.astype(np.float64) * b.imag)[keep], nb)
    return dims, K, N, P, X


def Pk_plane(delta, BoxSize, MAS='CIC', threads=1):
    dims, K, N, P, _ = _plane([delta], BoxSize, [MAS])
    kF = 2.0 * np.pi / BoxSize
    r = _Result()
    r.k = K[1:] / N[1:] * kF
    r.Nmodes = N[1:]
    r.Pk = P[0][1:] / N[1:] * (BoxSize / dims ** 2) ** 2
    return r


def XPk_plane(delta1, delta2, BoxSize, MAS1=None, MAS2=None, threads=1):
    dims, K, N, P, X = _plane([delta1, delta2], BoxSize, [MAS1, MAS2])
    kF = 2.0 * np.pi / BoxSize
    fact = (BoxSize / dims ** 2) ** 3
    r = _Result()
    r.k = K[1:] / N[1:] * kF
    r.Nmodes = N[1:]
    r.Pk = np.stack([P[0][1:] / N[1:] * fact, P[1][1:] / N[1:] * fact], axis=1)
    r.XPk = X[1:] / N[1:] * fact
    r.r = r.XPk / np.sqrt(r.Pk[:, 0] * r.Pk[:, 1])
    return r


# ------------------------------------------------------------------ smoothing
def FT_filter(BoxSize, R, dims, Filter, threads=1):
    """smoothing_library.FT_filter (smoothing_library.pyx:20-87): the filter on the
    grid (Top-Hat: 1 where d^2 <= (R dims/BoxSize)^2; Gaussian: exp(-d^2/(2 R_grid^2))),
    divided by its float64 sum, then R2C."""
    if Filter not in ('Top-Hat', 'Gaussian'):
        raise ValueError('Filter %s not implemented!' % Filter)
    R_grid = np.float32(np.float32(R) * dims / np.float32(BoxSize))
    R2 = np.float32(R_grid * R_grid)
    f = _freqs(dims)
    d2 = (f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2)
    if Filter == 'Top-Hat':
        field = (d2 <= R2).astype(np.float32)
    else:
        field = np.exp(-d2 / (2.0 * np.float64(R2))).astype(np.float32)
    norm = np.sum(field, dtype=np.float64)
    field = (field.astype(np.float64) / norm).astype(np.float32)
    return fft_r2c(field, threads).astype(np.complex64)


def field_smoothing(field, filter_k, threads=1):
    """smoothing_library.field_smoothing (:94-123): normalised C2R of FFT(field) * filter_k."""
    import scipy.fft
    fk = (fft_r2c(field, threads) * filter_k).astype(np.complex64)
    return scipy.fft.irfftn(fk, s=field.shape, workers=max(1, threads)).astype(np.float32)
