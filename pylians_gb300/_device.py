"""Device plumbing for the Python facade: tensors, streams and cached workspaces.

PyTorch is used only for device memory, copies and the current CUDA stream;
all arithmetic runs in libpylgpu.so.
"""
import ctypes

import numpy as np
import torch

from ._lib import PylError


def require_cuda():
    if not torch.cuda.is_available():
        raise PylError('pylians_gb300 needs a CUDA device; it has no CPU path')


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def is_torch(a):
    return isinstance(a, torch.Tensor)


def as_device_f32(a, name, device=None):
    """float32 C-contiguous CUDA tensor viewing (or copying) `a`.

    Like the reference's typed memoryviews (np.float32_t[:,:] / FLOAT[:,::1]),
    only float32 input is accepted; CUDA tensors are used in place.
    """
    device = device or torch.device('cuda', torch.cuda.current_device())
    if is_torch(a):
        if a.dtype != torch.float32:
            raise ValueError('%s must be float32, got %s' % (name, a.dtype))
        if a.is_cuda:
            if not a.is_contiguous():
                raise ValueError('%s must be C-contiguous' % name)
            return a
        return a.contiguous().to(device, non_blocking=True)
    arr = np.asarray(a)
    if arr.dtype != np.float32:
        raise ValueError('Buffer dtype mismatch: %s must be float32, got %s' % (name, arr.dtype))
    return torch.from_numpy(np.ascontiguousarray(arr)).to(device)


def as_device_f64(a, name, device=None):
    """float64 C-contiguous CUDA tensor viewing (or copying) `a` (the reference's
    np.float64_t[:,:,:] grids of the *_d kernels)."""
    device = device or torch.device('cuda', torch.cuda.current_device())
    if is_torch(a):
        if a.dtype != torch.float64:
            raise ValueError('%s must be float64, got %s' % (name, a.dtype))
        if a.is_cuda:
            if not a.is_contiguous():
                raise ValueError('%s must be C-contiguous' % name)
            return a
        return a.contiguous().to(device)
    arr = np.asarray(a)
    if arr.dtype != np.float64:
        raise ValueError('Buffer dtype mismatch: %s must be float64, got %s' % (name, arr.dtype))
    return torch.from_numpy(np.ascontiguousarray(arr)).to(device)


def as_device_c64(a, name, device=None):
    device = device or torch.device('cuda', torch.cuda.current_device())
    if is_torch(a):
        if a.dtype != torch.complex64:
            raise ValueError('%s must be complex64' % name)
        return a.contiguous() if a.is_cuda else a.contiguous().to(device)
    arr = np.asarray(a)
    if arr.dtype != np.complex64:
        raise ValueError('%s must be complex64' % name)
    return torch.from_numpy(np.ascontiguousarray(arr)).to(device)


class _WorkspaceCache(object):
    """One growing uint8 device buffer per device, reused by every call on it.

    Calls on one stream are ordered, so reuse is safe there; a caller that runs
    several streams concurrently passes its own workspace instead."""

    def __init__(self):
        self.bufs = {}

    def get(self, nbytes, device=None):
        if nbytes <= 0:
            return None
        dev = device or torch.cuda.current_device()
        b = self.bufs.get(dev)
        if b is None or b.numel() < nbytes:
            b = torch.empty(int(nbytes * 1.1) + 256, dtype=torch.uint8, device=dev)
            self.bufs[dev] = b
        return b

    def clear(self):
        self.bufs.clear()


workspace = _WorkspaceCache()
