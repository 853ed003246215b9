"""Drop-in for Pylians' smoothing_library on the GPU (smoothing_library.pyx:20-114).

  FT_filter(BoxSize, R, dims, Filter, threads): the Fourier transform of a
    'Top-Hat' or 'Gaussian' filter of radius R placed on a dims^3 grid and
    normalised to unit sum (complex64 [dims][dims][dims//2+1], numpy, as the
    reference; as_tensor=True keeps it on the device);
  field_smoothing(field, filter_k, threads): the field convolved with the
    filter (FFT, product, normalised inverse FFT); numpy in -> numpy out, CUDA
    tensors stay on the device.
"""
import numpy as np
import torch

from . import _lib
from ._device import as_device_c64, as_device_f32, is_torch, ptr, require_cuda, stream_ptr

__all__ = ['FT_filter', 'field_smoothing']


def FT_filter(BoxSize, R, dims, Filter, threads=1, as_tensor=False):
    require_cuda()
    if Filter not in ('Top-Hat', 'Gaussian'):
        raise ValueError('Filter %s not implemented!' % Filter)
    dev = torch.device('cuda', torch.cuda.current_device())
    field = torch.empty((dims, dims, dims), dtype=torch.float32, device=dev)
    norm = torch.empty(1, dtype=torch.float64, device=dev)
    _lib.call('pyl_filter_grid', ptr(field), dims, float(BoxSize), float(R), int(Filter == 'Gaussian'),
              ptr(norm), stream_ptr())
    out = torch.empty((dims, dims, dims // 2 + 1), dtype=torch.complex64, device=dev)
    _lib.call('pyl_fft_r2c', ptr(field), ptr(out), dims, 1, stream_ptr())
    return out if as_tensor else out.cpu().numpy()


def field_smoothing(field, filter_k, threads=1):
    require_cuda()
    x = as_device_f32(field, 'field')
    fk = as_device_c64(filter_k, 'filter_k')
    dims = x.shape[0]
    if fk.shape[0] != dims:
        raise ValueError('field and filter have different grids!!!')
    dk = torch.empty((dims, dims, dims // 2 + 1), dtype=torch.complex64, device=x.device)
    _lib.call('pyl_fft_r2c', ptr(x), ptr(dk), dims, 1, stream_ptr())
    _lib.call('pyl_cmul', ptr(dk), ptr(fk), dk.numel(), stream_ptr())
    out = torch.empty((dims,) * 3, dtype=torch.float32, device=x.device)
    _lib.call('pyl_fft_c2r', ptr(dk), ptr(out), dims, 1, stream_ptr())
    _lib.call('pyl_scale', ptr(out), out.numel(), float(np.float32(1.0 / float(dims) ** 3)), stream_ptr())
    return out if is_torch(field) else out.cpu().numpy()
