"""Drop-in for Pylians' redshift_space_library on the GPU.

pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis) mirrors
library/redshift_space_library.pyx:29-43: s = x + v (1+z)/H(z) along `axis`,
in place, then positions above BoxSize or below 0 are wrapped with
fmod(pos + BoxSize, BoxSize).  numpy arrays are copied to the device and the
result written back; CUDA tensors are updated in place.
"""
import numpy as np

from . import _lib
from ._device import as_device_f32, is_torch, ptr, require_cuda, stream_ptr

__all__ = ['pos_redshift_space']


def pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis):
    require_cuda()
    dpos = as_device_f32(pos, 'pos')
    dvel = as_device_f32(vel, 'vel')
    if dpos.dim() != 2 or dpos.shape[1] != 3 or tuple(dvel.shape) != tuple(dpos.shape):
        raise ValueError('pos and vel must both be (N,3)')
    if axis not in (0, 1, 2):
        raise ValueError('axis must be 0, 1 or 2')
    _lib.call('pyl_pos_redshift_space', ptr(dpos), ptr(dvel), dpos.shape[0], float(BoxSize), float(Hubble),
              float(redshift), int(axis), stream_ptr())
    if is_torch(pos):
        if not pos.is_cuda:
            pos.copy_(dpos.cpu())
    else:
        np.copyto(pos, dpos.cpu().numpy())
