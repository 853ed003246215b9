"""Drop-in for Pylians' MAS_library: particles -> density grid on the GPU.

Mirrors library/MAS_library/MAS_library.pyx:
  MA(pos, number, BoxSize, MAS='CIC', W=None, verbose=False, renormalize_2D=True)  (:57-112)
  NGP/CIC/TSC/PCS(pos, number, BoxSize) and NGPW/CICW/TSCW/PCSW(..., W)          (:123-545)
  CICW_d(pos, number, BoxSize, W), NGPW_d(pos, number, BoxSize, W): float64 grids (:229-266, :338-358)
  NGPc3D/CICc3D/... (pos, number, BoxSize, threads), *Wc3D(pos, number, W, BoxSize, threads),
  *c2D                                                                            (:1136-1221)
  FLOAT_type()                                                                     (:11-13)
  CIC_interp(density, BoxSize, pos, den)                                           (:558-599)

`number` is accumulated in place (+=), as in the reference; numpy arrays are
copied to the device and the result written back into them, CUDA tensors are
updated in place without a copy.  Differences from the reference:
  * errors raise ValueError instead of printing and calling sys.exit();
  * `threads` is accepted and ignored;
  * keyword-only extras: `interlaced=` (a second grid that receives the same
    particles shifted by half a cell on every axis) and `strategy=`
    ('auto', 'atomic', 'tiled', 'sorted');
  * *c2D entry points share MA's 2D path (deposit S times, then divide by S),
    equal to the reference's single deposit up to float rounding.
"""
import time

import numpy as np
import torch

from . import _lib
from ._device import as_device_f32, as_device_f64, is_torch, ptr, require_cuda, stream_ptr, workspace

__all__ = ['MA', 'NGP', 'CIC', 'TSC', 'PCS', 'NGPW', 'CICW', 'TSCW', 'PCSW', 'CICW_d', 'NGPW_d', 'FLOAT_type',
           'NGPc3D', 'CICc3D', 'TSCc3D', 'PCSc3D', 'NGPWc3D', 'CICWc3D', 'TSCWc3D', 'PCSWc3D',
           'NGPc2D', 'CICc2D', 'TSCc2D', 'PCSc2D', 'NGPWc2D', 'CICWc2D', 'TSCWc2D', 'PCSWc2D',
           'CIC_interp', 'ma_device', 'overdensity_device']


def FLOAT_type():
    return np.float32


def ma_device(pos, grid, BoxSize, MAS, W=None, grid_interlaced=None, renormalize_2D=True,
              strategy='auto', stream=None):
    """Deposit into CUDA tensors (no host copies).  All tensors float32, C-contiguous."""
    require_cuda()
    if MAS not in _lib.MAS_INDEX:
        raise ValueError('option not valid: MAS=%r' % (MAS,))
    if strategy not in _lib.STRATEGY:
        raise ValueError('unknown strategy %r' % (strategy,))
    ndim = pos.shape[1] if pos.dim() == 2 else -1
    if ndim not in (2, 3):
        raise ValueError('pos must be (N,2) or (N,3)')
    if grid.dim() != ndim:
        raise ValueError('pos have %d dimensions and the density %d' % (ndim, grid.dim()))
    dims = grid.shape[0]
    if any(s != dims for s in grid.shape):
        raise ValueError('density grid must be cubic / square')
    if grid_interlaced is not None and grid_interlaced.shape != grid.shape:
        raise ValueError('interlaced grid must have the shape of the grid')
    n = pos.shape[0]
    if W is not None and (W.dim() != 1 or W.shape[0] != n):
        raise ValueError('W must have one weight per particle')
    mas = _lib.MAS_INDEX[MAS]
    strat = _lib.STRATEGY[strategy]
    L = _lib.load()
    nbytes = L.pyl_ma_workspace_size(n, ndim, dims, mas, strat, int(grid_interlaced is not None))
    ws = workspace.get(nbytes)
    _lib.call('pyl_ma', ptr(pos), ptr(W), n, ndim, ptr(grid), ptr(grid_interlaced), dims,
              float(BoxSize), mas, strat, int(bool(renormalize_2D)), ptr(ws), nbytes,
              stream_ptr(stream))


def overdensity_device(pos, grid, BoxSize, MAS='CIC', W=None, grid_interlaced=None, strategy='auto',
                       stream=None):
    """Particles straight to the overdensity (CUDA tensors): grid (and grid_interlaced) are
    overwritten with delta = n/mean - 1, mean = N/dims^3 or sum(W)/dims^3, the convention of
    library/Pk_library/Pk_snapshot.py:70-88, in one deposit pass."""
    require_cuda()
    if MAS not in _lib.MAS_INDEX:
        raise ValueError('option not valid: MAS=%r' % (MAS,))
    if pos.dim() != 2 or pos.shape[1] != 3 or grid.dim() != 3:
        raise ValueError('pos must be (N,3) and the grid 3D')
    dims, n = grid.shape[0], pos.shape[0]
    mas, strat = _lib.MAS_INDEX[MAS], _lib.STRATEGY[strategy]
    L = _lib.load()
    nbytes = L.pyl_ma_workspace_size(n, 3, dims, mas, strat, int(grid_interlaced is not None))
    ws = workspace.get(nbytes)
    _lib.call('pyl_ma_overdensity', ptr(pos), ptr(W), n, ptr(grid), ptr(grid_interlaced), dims,
              float(BoxSize), mas, strat, ptr(ws), nbytes, stream_ptr(stream))


def MA(pos, number, BoxSize, MAS='CIC', W=None, verbose=False, renormalize_2D=True, *,
       interlaced=None, strategy='auto'):
    require_cuda()
    coord = pos.shape[1]
    coord_aux = number.ndim if not is_torch(number) else number.dim()
    if coord != coord_aux:
        raise ValueError('pos have %d dimensions and the density %d!!!' % (coord, coord_aux))
    if verbose:
        print('\nUsing %s mass assignment scheme%s' % (MAS, '' if W is None else ' with weights'))
    start = time.time()
    dpos = as_device_f32(pos, 'pos')
    dW = as_device_f32(W, 'W') if W is not None else None
    dgrid = as_device_f32(number, 'number')
    dint = as_device_f32(interlaced, 'interlaced') if interlaced is not None else None
    ma_device(dpos, dgrid, BoxSize, MAS, dW, dint, renormalize_2D, strategy)
    copied = False
    for host, dev in ((number, dgrid), (interlaced, dint)):
        if host is None or dev is None:
            continue
        if is_torch(host):
            if not host.is_cuda:
                host.copy_(dev.cpu())
                copied = True
        else:
            np.copyto(host, dev.cpu().numpy())
            copied = True
    if copied:                    # host results: the call has synchronised anyway
        _lib.check_device('MA')
    if verbose:
        torch.cuda.synchronize()
        print('Time taken = %.3f seconds\n' % (time.time() - start))


def CIC_interp(density, BoxSize, pos, den):
    """MAS_library.CIC_interp: den[i] <- CIC interpolation of the 3D density grid at
    pos[i] (the eight corner terms added in the reference's order).  numpy arrays are
    copied to the device and den written back; CUDA tensors are used in place."""
    require_cuda()
    dgrid = as_device_f32(density, 'density')
    dpos = as_device_f32(pos, 'pos')
    dden = as_device_f32(den, 'den')
    if dgrid.dim() != 3 or any(s != dgrid.shape[0] for s in dgrid.shape):
        raise ValueError('density must be a cubic 3D grid')
    if dpos.dim() != 2 or dpos.shape[1] != 3 or dden.dim() != 1 or dden.shape[0] != dpos.shape[0]:
        raise ValueError('pos must be (N,3) and den (N,)')
    _lib.call('pyl_cic_interp', ptr(dgrid), dgrid.shape[0], float(BoxSize), ptr(dpos), dpos.shape[0],
              ptr(dden), stream_ptr())
    if is_torch(den):
        if not den.is_cuda:
            den.copy_(dden.cpu())
    else:
        np.copyto(den, dden.cpu().numpy())


def _single(mas, weighted):
    def f(pos, number, BoxSize, W=None):
        MA(pos, number, BoxSize, mas, W if weighted else None, renormalize_2D=False)
    f.__name__ = mas + ('W' if weighted else '')
    f.__doc__ = 'MAS_library.%s: one %s deposit, no 2D renormalisation.' % (f.__name__, mas)
    return f


NGP, CIC, TSC, PCS = (_single(m, False) for m in ('NGP', 'CIC', 'TSC', 'PCS'))
NGPW, CICW, TSCW, PCSW = (_single(m, True) for m in ('NGP', 'CIC', 'TSC', 'PCS'))


def _ma_f64(pos, number, BoxSize, mas, W):
    """Deposit into a float64 grid (number[dims][dims][depth], += in place; numpy
    arrays are copied to the device and written back)."""
    require_cuda()
    dpos = as_device_f32(pos, 'pos')
    dW = as_device_f32(W, 'W') if W is not None else None
    dgrid = as_device_f64(number, 'number')
    if dpos.dim() != 2 or dpos.shape[1] not in (2, 3):
        raise ValueError('pos must be (N,2) or (N,3)')
    if dgrid.dim() != 3:
        raise ValueError('number must be a 3D float64 array')
    n, ndim = dpos.shape
    if dW is not None and (dW.dim() != 1 or dW.shape[0] != n):
        raise ValueError('W must have one weight per particle')
    dims, depth = dgrid.shape[0], dgrid.shape[2]
    if ndim == 3 and tuple(dgrid.shape) != (dims, dims, dims):
        raise ValueError('number must be (dims, dims, dims) for 3D positions')
    if ndim == 2 and dgrid.shape[1] != dims:
        raise ValueError('number must be (dims, dims, depth) for 2D positions')
    _lib.call('pyl_ma_f64', ptr(dpos), ptr(dW), n, ndim, ptr(dgrid), dims, depth, float(BoxSize),
              _lib.MAS_INDEX[mas], stream_ptr())
    if is_torch(number):
        if not number.is_cuda:
            number.copy_(dgrid.cpu())
    else:
        np.copyto(number, dgrid.cpu().numpy())


def CICW_d(pos, number, BoxSize, W):
    """MAS_library.CICW_d: weighted CIC into a float64 grid (MAS_library.pyx:229-266)."""
    _ma_f64(pos, number, BoxSize, 'CIC', W)


def NGPW_d(pos, number, BoxSize, W):
    """MAS_library.NGPW_d: weighted NGP into a float64 grid (MAS_library.pyx:338-358)."""
    _ma_f64(pos, number, BoxSize, 'NGP', W)


def _cpath(mas, weighted, ndim):
    if weighted:
        def f(pos, number, W, BoxSize, threads=1):
            _check_nd(number, ndim)
            MA(pos, number, BoxSize, mas, W, renormalize_2D=True)
    else:
        def f(pos, number, BoxSize, threads=1):
            _check_nd(number, ndim)
            MA(pos, number, BoxSize, mas, None, renormalize_2D=True)
    f.__name__ = '%s%sc%dD' % (mas, 'W' if weighted else '', ndim)
    f.__doc__ = 'MAS_library.%s (MAS_c.c path); threads is ignored.' % f.__name__
    return f


def _check_nd(number, ndim):
    nd = number.dim() if is_torch(number) else np.ndim(number)
    if nd != ndim:
        raise ValueError('expected a %dD grid' % ndim)


for _m in ('NGP', 'CIC', 'TSC', 'PCS'):
    for _w in (False, True):
        for _d in (2, 3):
            _f = _cpath(_m, _w, _d)
            globals()[_f.__name__] = _f
del _m, _w, _d, _f
