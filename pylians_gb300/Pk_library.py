"""Drop-in for Pylians' Pk_library (power spectra and bispectrum) on the GPU.

Mirrors library/Pk_library/Pk_library.pyx and bispectrum_library.pyx:
  frequencies(BoxSize, dims)                          Pk_library.pyx:59-64
  MAS_function(MAS)                                   :75-81
  check_number_modes(Nmodes, dims)                    :90-102
  FFT3Dr_f(a, threads) / IFFT3Dr_f(a, threads)        :120-133, :152-165
  Pk(delta, BoxSize, axis=2, MAS='CIC', threads=1, keep_deltak=False)   :266-425
      -> k1D, Pk1D, Nmodes1D, kpar, kper, Pk2D, Nmodes2D, k3D, Pk, Pkphase, Nmodes3D
  XPk(delta, BoxSize, axis=2, MAS=None, threads=1)    :534-798
      -> k1D, Pk1D, PkX1D, Nmodes1D, kpar, kper, Pk2D, PkX2D, Nmodes2D, k3D, Pk, XPk, Nmodes3D
  Bk(delta, BoxSize, k1, k2, theta, MAS='CIC', threads=1)   bispectrum_library.pyx:32-196
      -> B, Q, k, Pk

The mode loops run in libpylgpu.so (one read of each half-complex field, no
k-grid materialised); only the O(bins) finalisation below runs on the host,
in float64, with the reference's formulas.  `threads` is accepted and ignored.
Differences: check_number_modes(_2D) raise RuntimeError instead of sys.exit();
keyword-only `interlaced=` takes the half-cell-shifted grid(s) produced by
MAS_library.MA(..., interlaced=...).  Inputs may be numpy arrays or CUDA tensors.
"""
import math
import time

import numpy as np
import torch

from . import _lib
from ._device import as_device_c64, as_device_f32, is_torch, ptr, require_cuda, stream_ptr, workspace

__all__ = ['frequencies', 'MAS_function', 'check_number_modes', 'FFT3Dr_f', 'IFFT3Dr_f',
           'Pk', 'XPk', 'Bk', 'Bk_triangles', 'Xi', 'correct_MAS', 'Pk_plane', 'XPk_plane',
           'frequencies_2D', 'check_number_modes_2D', 'FFT2Dr_f', 'pk_sums_device', 'finalize_pk', 'geometry']


def frequencies(BoxSize, dims):
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    kmax_par = middle
    kmax_per = int(np.sqrt(middle ** 2 + middle ** 2))
    kmax = int(np.sqrt(middle ** 2 + middle ** 2 + middle ** 2))
    return kF, kN, kmax_par, kmax_per, kmax


def MAS_function(MAS):
    return _lib.MAS_INDEX.get(MAS, 0)


def check_number_modes(Nmodes, dims):
    own = 1 if dims % 2 == 1 else 8
    indep = (dims ** 3 - own) // 2 + own
    counted = int(np.sum(Nmodes))
    if counted != indep:
        raise RuntimeError('Not all modes counted: counted %d independent modes, expected %d'
                           % (counted, indep))


def _half_shape(dims):
    return (dims, dims, dims // 2 + 1)


def FFT3Dr_f(a, threads=1):
    """Unnormalised float32 R2C of a dims^3 grid -> complex64 (dims, dims, dims//2+1)."""
    require_cuda()
    x = as_device_f32(a, 'a')
    dims = x.shape[0]
    out = torch.empty(_half_shape(dims), dtype=torch.complex64, device=x.device)
    _lib.call('pyl_fft_r2c', ptr(x), ptr(out), dims, 1, stream_ptr())
    return out if is_torch(a) else out.cpu().numpy()


def IFFT3Dr_f(a, threads=1):
    """float32 C2R of a (dims, dims, dims//2+1) complex64 grid, divided by dims^3: the
    reference calls pyFFTW plans through FFTW.__call__, whose normalise_idft defaults to
    True (its Xi scales this transform by 1/dims^3 only, Pk_library.pyx:2144)."""
    require_cuda()
    x = as_device_c64(a, 'a').clone()     # cuFFT C2R overwrites its input
    dims = x.shape[0]
    out = torch.empty((dims,) * 3, dtype=torch.float32, device=x.device)
    _lib.call('pyl_fft_c2r', ptr(x), ptr(out), dims, 1, stream_ptr())
    _lib.call('pyl_scale', ptr(out), out.numel(), float(np.float32(1.0 / float(dims) ** 3)), stream_ptr())
    return out if is_torch(a) else out.cpu().numpy()


# --------------------------------------------------------------- geometry cache
_GEOM = {}


def geometry(dims, axis, device=None):
    """Data-independent per-bin sums (mode counts, sum |k|, sum |k_par|) for a grid and
    line of sight, computed once on the device and cached like an FFT plan."""
    dev = device if device is not None else torch.cuda.current_device()
    key = (str(dev), dims, axis)
    g = _GEOM.get(key)
    if g is None:
        L = _lib.load()
        n = L.pyl_pk_geometry_len(dims)
        t = torch.empty(n, dtype=torch.float64, device=dev)
        nbytes = L.pyl_pk_workspace_size(dims, 1, axis)
        ws = workspace.get(nbytes)
        _lib.call('pyl_pk_geometry', dims, axis, ptr(t), ptr(ws), nbytes, stream_ptr())
        g = t.cpu().numpy()
        _GEOM[key] = g
    return g


def _split_geometry(g, dims):
    _, _, kmax_par, kmax_per, kmax = frequencies(1.0, dims)
    nb1, nb2, nb3 = kmax_par + 1, (kmax_par + 1) * (kmax_per + 1), kmax + 1
    o = np.cumsum([0, nb1, nb1, nb2, nb3, nb3])
    return dict(K1=g[o[0]:o[1]], N1=g[o[1]:o[2]], N2=g[o[2]:o[3]], K3=g[o[3]:o[4]], N3=g[o[4]:o[5]])


def _split_sums(s, dims, F):
    _, _, kmax_par, kmax_per, kmax = frequencies(1.0, dims)
    nb1, nb2, nb3 = kmax_par + 1, (kmax_par + 1) * (kmax_per + 1), kmax + 1
    C = F + F * (F - 1) // 2
    o = np.cumsum([0, nb3 * 3 * C, nb3 * F, nb1 * C, nb2 * C])
    return dict(P3=s[o[0]:o[1]].reshape(nb3, 3, C), PH=s[o[1]:o[2]].reshape(nb3, F),
                P1=s[o[2]:o[3]].reshape(nb1, C), P2=s[o[3]:o[4]].reshape(nb2, C))


def pk_sums_device(dk, dims, axis, mas_list, dk_interlaced=None, out=None, stream=None):
    """Launch the fused deconvolve+bin kernel on F stacked half-complex fields
    (complex64 tensor [F, dims, dims, dims//2+1]); returns the float64 sums tensor."""
    F = dk.shape[0]
    L = _lib.load()
    n = L.pyl_pk_sums_len(dims, F)
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=dk.device)
    mp, keep = ctypes_int_array(mas_list)
    fstride = dims * dims * (dims // 2 + 1)
    nbytes = L.pyl_pk_workspace_size(dims, F, axis)
    ws = workspace.get(nbytes)
    _lib.call('pyl_pk_bin', ptr(dk), ptr(dk_interlaced), F, fstride, dims, axis, mp, ptr(out),
              ptr(ws), nbytes, stream_ptr(stream))
    del keep
    return out


def ctypes_int_array(vals):
    import ctypes
    arr = (ctypes.c_int * len(vals))(*[int(v) for v in vals])
    return ctypes.cast(arr, ctypes.c_void_p), arr


class _Result(object):
    pass


def finalize_pk(sums, geom, BoxSize, dims, F, cross):
    """Host float64 finalisation: Pk_library.pyx:384-421 (Pk) and :740-796 (XPk)."""
    kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
    fact = (BoxSize / dims ** 2) ** 3
    X = F * (F - 1) // 2
    s = _split_sums(sums, dims, F)
    g = _split_geometry(geom, dims)
    r = _Result()
    with np.errstate(divide='ignore', invalid='ignore'):
        N1 = g['N1'][1:].copy()
        k1D = (g['K1'][1:] / N1) * kF
        kmaxper = np.sqrt(kN ** 2 - k1D ** 2)
        area = (np.pi * kmaxper ** 2 / N1) / (2.0 * np.pi) ** 2
        P1 = s['P1'][1:] * fact * area[:, None]
        ip = np.arange(kmax_par + 1)
        iq = np.arange(kmax_per + 1)
        kpar = np.zeros((kmax_par + 1) * (kmax_per + 1))
        kper = np.zeros_like(kpar)
        idx = (kmax_par + 1) * iq[None, :] + ip[:, None]
        kpar[idx] = (0.5 * (ip + ip + 1) * kF)[:, None]
        kper[idx] = (0.5 * (iq + iq + 1) * kF)[None, :]
        N2 = g['N2'].copy()
        P2 = s['P2'] * fact / N2[:, None]
        check_number_modes(g['N3'], dims)
        N3 = g['N3'][1:].copy()
        k3D = (g['K3'][1:] / N3) * kF
        P3 = s['P3'][1:].copy()
        P3[:, 0] = (P3[:, 0] / N3[:, None]) * fact
        P3[:, 1] = (P3[:, 1] * 5.0 / N3[:, None]) * fact
        P3[:, 2] = (P3[:, 2] * 9.0 / N3[:, None]) * fact
        PH = (s['PH'][1:] / N3[:, None]) * fact
    r.k1D, r.Nmodes1D = k1D, N1
    r.kpar, r.kper, r.Nmodes2D = kpar, kper, N2
    r.k3D, r.Nmodes3D = k3D, N3
    if cross:
        r.Pk1D, r.PkX1D = np.ascontiguousarray(P1[:, :F]), np.ascontiguousarray(P1[:, F:F + X])
        r.Pk2D, r.PkX2D = np.ascontiguousarray(P2[:, :F]), np.ascontiguousarray(P2[:, F:F + X])
        r.Pk, r.XPk = np.ascontiguousarray(P3[:, :, :F]), np.ascontiguousarray(P3[:, :, F:F + X])
    else:
        r.Pk1D, r.Pk2D = P1[:, 0].copy(), P2[:, 0].copy()
        r.Pk, r.Pkphase = np.ascontiguousarray(P3[:, :, 0]), PH[:, 0].copy()
    return r


def _fields_to_dk(deltas, device):
    dims = deltas[0].shape[0]
    F = len(deltas)
    dk = torch.empty((F,) + _half_shape(dims), dtype=torch.complex64, device=device)
    for i, d in enumerate(deltas):
        x = as_device_f32(d, 'delta')
        if tuple(x.shape) != (dims,) * 3:
            raise ValueError('Fields have different grid sizes!!!')
        _lib.call('pyl_fft_r2c', ptr(x), ptr(dk[i]), dims, 1, stream_ptr())
    return dk


class Pk(object):
    def __init__(self, delta, BoxSize, axis=2, MAS='CIC', threads=1, keep_deltak=False, *,
                 interlaced=None, verbose=False):
        require_cuda()
        start = time.time()
        if axis not in (0, 1, 2):
            raise ValueError('axis must be 0, 1 or 2')
        dims = delta.shape[0]
        dev = torch.device('cuda', torch.cuda.current_device())
        dk = _fields_to_dk([delta], dev)
        dk2 = _fields_to_dk([interlaced], dev) if interlaced is not None else None
        p = MAS_function(MAS)
        s = pk_sums_device(dk, dims, axis, [p], dk2)
        geom = geometry(dims, axis)
        r = finalize_pk(s.cpu().numpy(), geom, BoxSize, dims, 1, cross=False)
        self.__dict__.update(r.__dict__)
        if keep_deltak:
            _lib.call('pyl_mas_deconvolve', ptr(dk[0]), ptr(dk2), dims, p, stream_ptr())
            self.delta_k = dk[0] if is_torch(delta) else dk[0].cpu().numpy()
        if verbose:
            print('Time taken = %.2f seconds' % (time.time() - start))


# ------------------------------------------------------------------- 2D fields
def frequencies_2D(BoxSize, dims):
    """Pk_library.frequencies_2D (Pk_library.pyx:67-72)."""
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    return kF, kN, middle, middle, int(np.sqrt(middle ** 2 + middle ** 2))


def check_number_modes_2D(Nmodes, dims):
    """Pk_library.check_number_modes_2D (:105-117); raises RuntimeError, like
    check_number_modes, instead of exiting."""
    own = 1 if dims % 2 == 1 else 4
    indep = (dims ** 2 - own) // 2 + own
    if int(np.sum(Nmodes)) != indep:
        raise RuntimeError('Not all modes counted: counted %d independent modes, expected %d'
                         % (int(np.sum(Nmodes)), indep))


def FFT2Dr_f(a, threads=1):
    """Unnormalised float32 R2C of a (dims, dims) map (Pk_library FFT2Dr_f)."""
    require_cuda()
    x = as_device_f32(a, 'a')
    dims = x.shape[0]
    out = torch.empty((dims, dims // 2 + 1), dtype=torch.complex64, device=x.device)
    _lib.call('pyl_fft2_r2c', ptr(x), ptr(out), dims, 1, stream_ptr())
    return out if is_torch(a) else out.cpu().numpy()


def _plane_sums(maps, mas):
    xs = [as_device_f32(m, 'delta') for m in maps]
    dims = xs[0].shape[0]
    for x in xs:
        if x.dim() != 2 or tuple(x.shape) != (dims, dims):
            raise ValueError('maps must be square (dims, dims) float32 arrays of one size')
    dks = []
    for x in xs:
        dk = torch.empty((dims, dims // 2 + 1), dtype=torch.complex64, device=x.device)
        _lib.call('pyl_fft2_r2c', ptr(x), ptr(dk), dims, 1, stream_ptr())
        dks.append(dk)
    nb = _lib.load().pyl_pk_plane_bins(dims)
    sums = torch.empty(5 * nb, dtype=torch.float64, device=xs[0].device)
    _lib.call('pyl_pk_plane_bin', ptr(dks[0]), ptr(dks[1]) if len(dks) > 1 else None, dims,
              MAS_function(mas[0]), MAS_function(mas[1]) if len(mas) > 1 else 0, ptr(sums), stream_ptr())
    s = sums.cpu().numpy().reshape(5, nb)
    return dims, s


class Pk_plane(object):
    """Pk_library.Pk_plane (Pk_library.pyx:440-516): P(k) of a 2D map; attributes k,
    Nmodes, Pk (DC bin dropped)."""

    def __init__(self, delta, BoxSize, MAS='CIC', threads=1):
        require_cuda()
        dims, s = _plane_sums([delta], [MAS])
        kF = frequencies_2D(BoxSize, dims)[0]
        check_number_modes_2D(s[1], dims)
        N = s[1][1:]
        self.k = s[0][1:] / N * kF
        self.Nmodes = N
        self.Pk = s[2][1:] / N * (BoxSize / dims ** 2) ** 2


class XPk_plane(object):
    """Pk_library.XPk_plane (Pk_library.pyx:814-941): auto and cross P(k) of two 2D
    maps; attributes k, Nmodes, Pk [bins, 2], XPk, r = XPk / sqrt(Pk1 Pk2).  As in the
    reference, spectra are scaled by (BoxSize/dims^2)^3 and the size check compares
    delta1.shape[0] with delta2.shape[1]."""

    def __init__(self, delta1, delta2, BoxSize, MAS1=None, MAS2=None, threads=1):
        require_cuda()
        if delta1.shape[0] != delta2.shape[1]:
            raise ValueError('Images have different grid sizes!!!')
        dims, s = _plane_sums([delta1, delta2], [MAS1, MAS2])
        kF = frequencies_2D(BoxSize, dims)[0]
        fact = (BoxSize / dims ** 2) ** 3
        N = s[1][1:]
        self.k = s[0][1:] / N * kF
        self.Nmodes = N
        self.Pk = np.stack([s[2][1:] / N * fact, s[3][1:] / N * fact], axis=1)
        self.XPk = s[4][1:] / N * fact
        self.r = self.XPk / np.sqrt(self.Pk[:, 0] * self.Pk[:, 1])


def correct_MAS(delta, BoxSize, MAS='CIC', threads=1):
    """Pk_library.correct_MAS (Pk_library.pyx:1749-1806): the field with its Fourier
    modes divided by the MAS window, back at the input's scale.  As in the reference,
    the redundant half of the kz = 0 and kz = N/2 planes is left uncorrected
    (:1789-1792) and those planes enter the inverse transform through their
    Hermitian part."""
    require_cuda()
    x = as_device_f32(delta, 'delta')
    dims = x.shape[0]
    dk = torch.empty(_half_shape(dims), dtype=torch.complex64, device=x.device)
    _lib.call('pyl_fft_r2c', ptr(x), ptr(dk), dims, 1, stream_ptr())
    _lib.call('pyl_correct_mas', ptr(dk), dims, MAS_function(MAS), stream_ptr())
    out = torch.empty((dims,) * 3, dtype=torch.float32, device=x.device)
    _lib.call('pyl_fft_c2r', ptr(dk), ptr(out), dims, 1, stream_ptr())
    _lib.call('pyl_scale', ptr(out), out.numel(), float(np.float32(1.0 / float(dims) ** 3)), stream_ptr())
    return out if is_torch(delta) else out.cpu().numpy()


class Xi(object):
    """Pk_library.Xi (Pk_library.pyx:2035-2150): correlation function of a grid from the
    inverse transform of |delta_k W^-1|^2; attributes r3D, xi ([bins, 3]: l = 0, 2, 4)
    and Nmodes3D (bin 0 dropped, as the reference)."""

    def __init__(self, delta, BoxSize, MAS='CIC', axis=2, threads=1):
        require_cuda()
        if axis not in (0, 1, 2):
            raise ValueError('axis must be 0, 1 or 2')
        x = as_device_f32(delta, 'delta')
        dims = x.shape[0]
        dk = torch.empty(_half_shape(dims), dtype=torch.complex64, device=x.device)
        _lib.call('pyl_fft_r2c', ptr(x), ptr(dk), dims, 1, stream_ptr())
        _lib.call('pyl_xi_power', ptr(dk), dims, MAS_function(MAS), stream_ptr())
        g = torch.empty((dims,) * 3, dtype=torch.float32, device=x.device)
        _lib.call('pyl_fft_c2r', ptr(dk), ptr(g), dims, 1, stream_ptr())
        del dk
        nb = _lib.load().pyl_xi_sums_len(dims) // 5
        sums = torch.empty(5 * nb, dtype=torch.float64, device=x.device)
        _lib.call('pyl_xi_bin', ptr(g), dims, axis, ptr(sums), stream_ptr())
        s = sums.cpu().numpy()
        X = s[:3 * nb].reshape(nb, 3)[1:]
        R, N = s[3 * nb:4 * nb][1:], s[4 * nb:][1:]
        # the unnormalised C2R carries dims^3; the reference's normalised one leaves the
        # 1/dims^3 of its finalisation (:2144-2146)
        norm = 1.0 / float(dims) ** 6
        self.r3D = R / N * (BoxSize * 1.0 / dims)
        self.Nmodes3D = N
        self.xi = np.stack([X[:, 0] / N * norm, X[:, 1] * 5.0 / N * norm, X[:, 2] * 9.0 / N * norm], axis=1)


class XPk(object):
    def __init__(self, delta, BoxSize, axis=2, MAS=None, threads=1, *, interlaced=None,
                 verbose=False):
        require_cuda()
        start = time.time()
        if axis not in (0, 1, 2):
            raise ValueError('axis must be 0, 1 or 2')
        F = len(delta)
        if MAS is None or len(MAS) != F:
            raise ValueError('XPk needs one MAS per field')
        dims = delta[0].shape[0]
        dev = torch.device('cuda', torch.cuda.current_device())
        dk = _fields_to_dk(list(delta), dev)
        dk2 = _fields_to_dk(list(interlaced), dev) if interlaced is not None else None
        mas_p = [MAS_function(m) for m in MAS]
        geom = geometry(dims, axis)
        if F <= 4:
            s = pk_sums_device(dk, dims, axis, mas_p, dk2)
            r = finalize_pk(s.cpu().numpy(), geom, BoxSize, dims, F, cross=True)
        else:
            r = self._pairwise(dk, dk2, dims, axis, mas_p, geom, BoxSize)
        self.__dict__.update(r.__dict__)
        if verbose:
            print('Time taken = %.2f seconds' % (time.time() - start))

    @staticmethod
    def _pairwise(dk, dk2, dims, axis, mas_p, geom, BoxSize):
        """More than 4 fields: one 2-field launch per pair (i<j); field i's auto spectra
        come from its first pair."""
        F = dk.shape[0]
        X = F * (F - 1) // 2
        out, x = None, 0
        for i in range(F):
            for j in range(i + 1, F):
                pair = torch.stack([dk[i], dk[j]])
                pair2 = torch.stack([dk2[i], dk2[j]]) if dk2 is not None else None
                s = pk_sums_device(pair, dims, axis, [mas_p[i], mas_p[j]], pair2)
                r = finalize_pk(s.cpu().numpy(), geom, BoxSize, dims, 2, cross=True)
                if out is None:
                    out = _Result()
                    for k in ('k1D', 'Nmodes1D', 'kpar', 'kper', 'Nmodes2D', 'k3D', 'Nmodes3D'):
                        setattr(out, k, getattr(r, k))
                    nb3, nb1, nb2 = r.Pk.shape[0], r.Pk1D.shape[0], r.Pk2D.shape[0]
                    out.Pk, out.XPk = np.zeros((nb3, 3, F)), np.zeros((nb3, 3, X))
                    out.Pk1D, out.PkX1D = np.zeros((nb1, F)), np.zeros((nb1, X))
                    out.Pk2D, out.PkX2D = np.zeros((nb2, F)), np.zeros((nb2, X))
                for f, c in ((i, 0), (j, 1)):
                    if (f == i and j == i + 1) or (f == j and i == 0):
                        out.Pk[:, :, f] = r.Pk[:, :, c]
                        out.Pk1D[:, f] = r.Pk1D[:, c]
                        out.Pk2D[:, f] = r.Pk2D[:, c]
                out.XPk[:, :, x] = r.XPk[:, :, 0]
                out.PkX1D[:, x] = r.PkX1D[:, 0]
                out.PkX2D[:, x] = r.PkX2D[:, 0]
                x += 1
        return out


# ------------------------------------------------------------------ bispectrum
def shell_k2_bounds(k_min, k_max):
    """Exact integer bounds [lo, hi) on kx^2+ky^2+kz^2 for k_min <= sqrt(k2) < k_max, with
    sqrt the correctly rounded float64 square root the reference compares (:115-117)."""
    def first_at_least(x):
        if x <= 0.0:
            return 0
        c = max(0, int(math.floor(x * x)) - 2)
        while np.sqrt(np.float64(c)) < x:
            c += 1
        while c > 0 and np.sqrt(np.float64(c - 1)) >= x:
            c -= 1
        return c
    return first_at_least(k_min), first_at_least(k_max)


def _fast_side(m):
    """Smallest even side >= m whose prime factors are 2, 3, 5 and 7 (fast cuFFT sizes)."""
    m = max(2, int(m))
    while True:
        if m % 2 == 0:
            r = m
            for p in (2, 3, 5, 7):
                while r % p == 0:
                    r //= p
            if r == 1:
                return m
        m += 1


def bk_side(dims, bounds):
    """Side M of the grid the shell fields are transformed and reduced on: the smallest
    fast side above 3 K (K the largest wave number of any shell: k^2 < max hi), or dims
    when that is not smaller.  The shell fields are band-limited, so their triple-product
    sums over M^3 cells are (M/dims)^3 those over dims^3 cells (pyl_bk_shell_fill)."""
    hi = max(b[1] for b in bounds)
    K = 0
    while (K + 1) ** 2 < hi:
        K += 1
    m = _fast_side(3 * K + 1)
    return m if m < dims else dims


class BkPlan(object):
    """Bispectra of a fixed triangle set (k1, k2, k3 in h/Mpc) on dims^3 fields: shells,
    their exact integer bounds, triangle groups, their reduced grids and every device
    buffer are set up once, and so are the indicator fields' triple sums (sum_x I_a I_b
    I_c depends only on the shells; made once per plan by the same kernels).

    Triangles sharing their first two shells (a, b) form a group.  A group of several
    triangles is summed in Fourier space: P_ab = d_a d_b on a reduced grid, its R2C, and
    for each triangle the sum over its third shell's modes of Re(delta conj(P_ab^))
    (Parseval: the real-space triple sum), so only d_a and d_b need real space.  A lone
    triangle is reduced in real space (pyl_bk_triangles) from the C2R of its shells.
    method='real' or 'fourier' forces one way for every group.

    Each group or lone triangle is evaluated on its own reduced grid, the smallest fast
    side above 3 K with K the largest wave number of its shells (bk_side): the shell
    fields are band-limited, so the sums there equal the full grid's up to the factor
    (M/dims)^3 that B, a ratio, cancels.  Groups and triangles of one side share one
    shell fill, one batched C2R and one reduction; `side` forces one side for all.

    run(delta) enqueues the data-dependent chain on one stream (R2C, MAS deconvolution,
    the shell powers, then per side the shell fill, C2R and triangle sums) with no host
    synchronisation, so capture() can record it as a CUDA graph; result() reads the sums
    back and finalises B, Q and the shell powers (bispectrum_library.pyx:132-190)."""

    MAX_SHELLS = 96

    def __init__(self, dims, BoxSize, triangles, MAS='CIC', device=None, side=None, method='auto'):
        require_cuda()
        import ctypes
        if method not in ('auto', 'real', 'fourier'):
            raise ValueError("method must be 'auto', 'real' or 'fourier'")
        self.dims, self.BoxSize, self.MAS = int(dims), float(BoxSize), MAS
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        kF = frequencies(BoxSize, dims)[0]
        keys, index, tri_idx = [], {}, []
        for (a, b, c) in triangles:
            ids = []
            for k in (a, b, c):
                kmin, kmax = (k - kF) / kF, (k + kF) / kF       # bispectrum_library.pyx:73-77
                if (kmin, kmax) not in index:
                    index[(kmin, kmax)] = len(keys)
                    keys.append((kmin, kmax))
                ids.append(index[(kmin, kmax)])
            tri_idx.append(ids)
        self.tri = np.asarray(tri_idx, dtype=np.int64)
        self.bounds = [shell_k2_bounds(lo, hi) for lo, hi in keys]
        S, T = len(self.bounds), len(tri_idx)
        self.method = method

        # units: Fourier groups (several triangles sharing (a, b)) and lone triangles
        groups = {}
        for t, (a, b, c) in enumerate(tri_idx):
            groups.setdefault((a, b), []).append(t)
        units = []
        for (a, b), ts in groups.items():
            if method == 'fourier' or (method == 'auto' and len(ts) >= 2):
                units.append(('fourier', (a, b), ts))
            else:
                units.extend(('real', None, [t]) for t in ts)
        # reduced side of each unit (the smallest valid one), then a ladder of sides at
        # least 3/2 apart that every unit rounds up to: a few sides, each with one
        # shell fill, one batched C2R and one reduction, instead of one per unit
        own = []
        for kind, ab, ts in units:
            sh = [s_ for t in ts for s_ in tri_idx[t]]
            own.append(int(side) if side else bk_side(self.dims, [self.bounds[s_] for s_ in sh]))
        ladder = []
        for m in sorted(set(own), reverse=True):
            if not ladder or 3 * m <= 2 * ladder[-1]:
                ladder.append(m)
        by_side = {}
        for u, m in zip(units, own):
            mm = min(x for x in ladder if x >= m)
            by_side.setdefault(mm, []).append(u)
        self.sides = sorted(by_side)
        self.side = max(self.sides)

        dev = self.device
        I64, I32 = ctypes.c_int64, ctypes.c_int
        self.dk = torch.empty(_half_shape(self.dims), dtype=torch.complex64, device=dev)
        self.power = torch.empty(2 * S, dtype=torch.float64, device=dev)
        self.num = torch.empty(T, dtype=torch.float64, device=dev)       # internal order
        self.den = torch.empty(T, dtype=torch.float64, device=dev)
        # every shell's power: one fill call per 96 shells, no field written
        self._pw = []
        for s0 in range(0, S, self.MAX_SHELLS):
            bs = self.bounds[s0:s0 + self.MAX_SHELLS]
            self._pw.append((s0, len(bs), (I64 * len(bs))(*[b[0] for b in bs]), (I64 * len(bs))(*[b[1] for b in bs]),
                             (I32 * len(bs))(*([-1] * len(bs)))))
        order = []
        self._classes = []
        for m in self.sides:
            us = by_side[m]
            needed = sorted(set(s_ for kind, ab, ts in us for s_ in (ab if kind == 'fourier' else tri_idx[ts[0]])))
            slot = {s_: i for i, s_ in enumerate(needed)}
            half, cells = m * m * (m // 2 + 1), m ** 3
            stride = (cells + 3) // 4 * 4
            c = dict(side=m, R=len(needed), half=half, cells=cells, stride=stride,
                     cd=torch.empty((len(needed), half), dtype=torch.complex64, device=dev),
                     d_real=torch.empty(len(needed) * stride, dtype=torch.float32, device=dev),
                     pw_scratch=torch.empty(2 * len(needed), dtype=torch.float64, device=dev))
            # fill: the needed shells only (their own cube of modes), in chunks of 96
            c['fill'] = []
            for j0 in range(0, len(needed), self.MAX_SHELLS):
                part = needed[j0:j0 + self.MAX_SHELLS]
                c['fill'].append((j0, len(part), (I64 * len(part))(*[self.bounds[s_][0] for s_ in part]),
                                  (I64 * len(part))(*[self.bounds[s_][1] for s_ in part]),
                                  (I32 * len(part))(*range(j0, j0 + len(part)))))
            real_ts = [ts[0] for kind, ab, ts in us if kind == 'real']
            c['real_off'], c['n_real'] = len(order), len(real_ts)
            c['tri'] = (I32 * max(3 * len(real_ts), 1))(*[slot[s_] for t in real_ts for s_ in tri_idx[t]])
            order.extend(real_ts)
            c['dots'] = []
            c['fourier_off'] = len(order)
            for kind, (a, b), ts in [u for u in us if u[0] == 'fourier']:
                for j0 in range(0, len(ts), self.MAX_SHELLS):
                    part = ts[j0:j0 + self.MAX_SHELLS]
                    n = len(part)
                    cb = [self.bounds[tri_idx[t][2]] for t in part]
                    c['dots'].append((slot[a], slot[b], n, (I64 * n)(*[x[0] for x in cb]),
                                      (I64 * n)(*[x[1] for x in cb]), (I32 * n)(*range(len(order), len(order) + n))))
                    order.extend(part)
            c['n_fourier'] = len(order) - c['fourier_off']
            if c['dots']:
                c['prod'] = torch.empty(stride, dtype=torch.float32, device=dev)
                c['prod_hat'] = torch.empty(half, dtype=torch.complex64, device=dev)
            self._classes.append(c)
        self.order = np.array(order, dtype=np.int64)
        self.R = sum(c['R'] for c in self._classes)                   # shell fields in real space
        self.n_fourier_groups = sum(len(c['dots']) for c in self._classes)
        self.mas_p = MAS_function(MAS)
        self.graph = None
        self._indicator_sums()

    def _powers(self, dk, st):
        import ctypes
        for s0, ns, lo, hi, sl in self._pw:
            _lib.call('pyl_bk_shell_fill', dk, self.dims, self.dims, ctypes.cast(lo, ctypes.c_void_p),
                      ctypes.cast(hi, ctypes.c_void_p), ctypes.cast(sl, ctypes.c_void_p), ns, None, None,
                      ptr(self.power[2 * s0:]), st)

    def _fill(self, c, dk, st):
        """The class's needed shells into its half grids: delta fields, or with dk None
        the indicator fields."""
        import ctypes
        for j0, ns, lo, hi, sl in c['fill']:
            _lib.call('pyl_bk_shell_fill', dk, self.dims, c['side'], ctypes.cast(lo, ctypes.c_void_p),
                      ctypes.cast(hi, ctypes.c_void_p), ctypes.cast(sl, ctypes.c_void_p), ns,
                      ptr(c['cd']) if dk is not None else None, None if dk is not None else ptr(c['cd']),
                      ptr(c['pw_scratch'][2 * j0:]), st)

    def _c2r(self, c, st):
        m, R = c['side'], c['R']
        if R == 0:
            return
        if c['stride'] == c['cells']:
            _lib.call('pyl_fft_c2r', ptr(c['cd']), ptr(c['d_real']), m, R, st)
        else:
            for s_ in range(R):
                _lib.call('pyl_fft_c2r', ptr(c['cd'][s_]), ptr(c['d_real'][s_ * c['stride']:]), m, 1, st)

    def _sums(self, c, dk, indicator, out, st):
        """The class's triangle sums (delta fields, or the indicator fields when
        `indicator`) into out (internal order)."""
        import ctypes
        m, stride = c['side'], c['stride']
        if c['n_real']:
            d_f, i_f = (None, ptr(c['d_real'])) if indicator else (ptr(c['d_real']), None)
            o = ptr(out[c['real_off']:])
            _lib.call('pyl_bk_triangles', d_f, i_f, m, stride, max(c['R'], 1), ctypes.cast(c['tri'], ctypes.c_void_p),
                      c['n_real'], None if indicator else o, o if indicator else None, st)
        if c['dots']:
            out[c['fourier_off']:c['fourier_off'] + c['n_fourier']].zero_()
            for sa, sb, n, lo, hi, dst in c['dots']:
                _lib.call('pyl_bk_product', ptr(c['d_real'][sa * stride:]), ptr(c['d_real'][sb * stride:]),
                          ptr(c['prod']), c['cells'], st)
                _lib.call('pyl_fft_r2c', ptr(c['prod']), ptr(c['prod_hat']), m, 1, st)
                _lib.call('pyl_bk_shell_dots', None if indicator else dk, self.dims, ptr(c['prod_hat']), m,
                          ctypes.cast(lo, ctypes.c_void_p), ctypes.cast(hi, ctypes.c_void_p),
                          ctypes.cast(dst, ctypes.c_void_p), n, ptr(out), st)

    def _chain(self, dk, indicator, out, st):
        for c in self._classes:
            self._fill(c, dk, st)
            self._c2r(c, st)
            self._sums(c, dk, indicator, out, st)

    def _indicator_sums(self):
        """den = sum_x I_a I_b I_c on the reduced grids, once: the indicator fields are
        filled into the delta buffers (which every run overwrites), transformed and
        summed, with no delta input."""
        with torch.cuda.device(self.device):
            st = stream_ptr(None)
            self._chain(None, True, self.den, st)

    def run(self, delta, stream=None):
        """Enqueue the chain on `delta` (a dims^3 float32 grid); nothing waits on the host."""
        x = as_device_f32(delta, 'delta')
        if tuple(x.shape) != (self.dims,) * 3:
            raise ValueError('delta must be a %d^3 grid' % self.dims)
        self._x = x
        st = stream_ptr(stream)
        d = self.dims
        _lib.call('pyl_fft_r2c', ptr(x), ptr(self.dk), d, 1, st)
        _lib.call('pyl_mas_deconvolve', ptr(self.dk), None, d, self.mas_p, st)
        self._powers(ptr(self.dk), st)
        self._chain(ptr(self.dk), False, self.num, st)

    def capture(self, delta):
        """Record run(delta) (fixed address) as a CUDA graph; replay() relaunches it."""
        self.run(delta)             # warm-up: plans, function attributes
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(delta)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def result(self):
        """(B, Q, Pk1, Pk2, Pk3) per triangle, in float64 on the host."""
        L, d = self.BoxSize, self.dims
        pw = self.power.cpu().numpy()
        P = (pw[0::2] / pw[1::2]) * (L / d ** 2) ** 3
        ratio = np.empty(len(self.tri))
        ratio[self.order] = self.num.cpu().numpy() / self.den.cpu().numpy()
        B = ratio * (L ** 2 / d ** 3) ** 3
        t = self.tri
        P1, P2, P3 = P[t[:, 0]], P[t[:, 1]], P[t[:, 2]]
        Q = B / (P1 * P2 + P1 * P3 + P2 * P3)
        return B, Q, P1, P2, P3


def Bk_triangles(delta, BoxSize, triangles, MAS='CIC', threads=1):
    """Bispectra of many triangles (k1, k2, k3) in h/Mpc sharing one FFT, one shell
    fill, one batched C2R and one reduction pass.  Returns (B, Q, Pk1, Pk2, Pk3)."""
    plan = BkPlan(delta.shape[0], BoxSize, triangles, MAS)
    plan.run(delta)
    return plan.result()


class Bk(object):
    def __init__(self, delta, BoxSize, k1, k2, theta, MAS='CIC', threads=1, *, verbose=False):
        start = time.time()
        theta = np.asarray(theta, dtype=np.float64)
        bins = theta.shape[0]
        k3 = np.sqrt((k2 * np.sin(theta)) ** 2 + (k2 * np.cos(theta) + k1) ** 2)   # :66
        tris = [(k1, k2, float(k3[j])) for j in range(bins)]
        B, Q, P1, P2, P3 = Bk_triangles(delta, BoxSize, tris, MAS, threads)
        self.B = B
        self.Q = Q
        self.k = np.concatenate([[k1, k2], k3]).astype(np.float64)
        self.Pk = np.concatenate([[P1[0], P2[0]], P3]).astype(np.float64)
        if verbose:
            print('Time to compute bispectrum = %.2f' % (time.time() - start))
