"""Particles -> overdensity -> R2C -> fused deconvolve/bin on one stream, buffers kept resident.

This is the caller-side chain the reference's drivers run around MA and Pk
(library/Pk_library/Pk_snapshot.py:66-89, documentation/Documentation.md:88-118):

    delta = zeros; MA(pos, delta, BoxSize, MAS[, W]); delta /= mean; delta -= 1
    Pk(delta, BoxSize, axis, MAS)

with mean = N_particles / dims^3 (or sum(W) / dims^3 with weights), plus the
interlaced second grid when `interlaced=True`.  The deposit writes the
overdensity directly (pyl_ma_overdensity: grids filled with -1, deposits
scaled by 1/mean), so there is no separate normalisation pass.  Every launch goes to one CUDA
stream, so a whole step can be captured in a CUDA graph (`capture()`), and the
grids, FFT outputs and sums stay allocated across steps.
"""
import torch

from . import _lib
from . import Pk_library as PKL
from ._device import ptr, require_cuda, stream_ptr


class ParticlePk(object):
    def __init__(self, dims, BoxSize, MAS='CIC', axis=2, interlaced=False, strategy='auto',
                 max_particles=0, weighted=False, device=None):
        require_cuda()
        if MAS not in _lib.MAS_INDEX:
            raise ValueError('MAS must be NGP, CIC, TSC or PCS')
        self.dims, self.BoxSize, self.MAS, self.axis = int(dims), float(BoxSize), MAS, int(axis)
        self.interlaced = bool(interlaced)
        self.strategy = strategy
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        ng = 2 if self.interlaced else 1
        d = self.dims
        self.grids = torch.empty((ng, d, d, d), dtype=torch.float32, device=self.device)
        self.dk = torch.empty((ng, d, d, d // 2 + 1), dtype=torch.complex64, device=self.device)
        L = _lib.load()
        self.sums = torch.empty(L.pyl_pk_sums_len(d, 1), dtype=torch.float64, device=self.device)
        self.wsum = torch.empty(1, dtype=torch.float64, device=self.device)
        self.mas_p, self._keep = PKL.ctypes_int_array([_lib.MAS_INDEX[MAS]])
        self.ws_bytes = 0
        self.ws = None
        self.pk_ws_bytes = L.pyl_pk_workspace_size(d, 1, self.axis)
        self.pk_ws = (torch.empty(self.pk_ws_bytes, dtype=torch.uint8, device=self.device)
                      if self.pk_ws_bytes else None)
        self.reserve(max_particles, weighted)
        self.geom = PKL.geometry(d, self.axis, self.device)
        self.graph = None

    def reserve(self, n, weighted=False):
        L = _lib.load()
        need = L.pyl_ma_workspace_size(int(n), 3, self.dims, _lib.MAS_INDEX[self.MAS],
                                       _lib.STRATEGY[self.strategy], int(self.interlaced))
        if need > self.ws_bytes:
            self.ws = torch.empty(need, dtype=torch.uint8, device=self.device)
            self.ws_bytes = need

    def step(self, pos, W=None, stream=None, rsd=None):
        """Enqueue one pass: overdensity deposit (grids overwritten), FFT, bin -> self.sums.

        rsd=(vel, Hubble, redshift, axis) first moves the particles to redshift space
        IN PLACE (redshift_space_library.pos_redshift_space), fused into the deposit's
        histogram pass on the tiled path."""
        n = pos.shape[0]
        d = self.dims
        st = stream_ptr(stream)
        self.reserve(n, W is not None)
        g2 = self.grids[1] if self.interlaced else None
        if rsd is not None:
            vel, hubble, redshift, axis = rsd
            if tuple(vel.shape) != tuple(pos.shape) or vel.dtype != torch.float32 or not vel.is_cuda:
                raise ValueError('vel must be a float32 CUDA tensor shaped like pos')
            _lib.call('pyl_ma_overdensity_rsd', ptr(pos), ptr(vel.contiguous()), ptr(W), n, ptr(self.grids[0]),
                      ptr(g2), d, self.BoxSize, _lib.MAS_INDEX[self.MAS], _lib.STRATEGY[self.strategy],
                      float(hubble), float(redshift), int(axis), ptr(self.ws), self.ws_bytes, st)
        else:
            _lib.call('pyl_ma_overdensity', ptr(pos), ptr(W), n, ptr(self.grids[0]), ptr(g2), d,
                      self.BoxSize, _lib.MAS_INDEX[self.MAS], _lib.STRATEGY[self.strategy],
                      ptr(self.ws), self.ws_bytes, st)
        ng = self.grids.shape[0]
        _lib.call('pyl_fft_r2c', ptr(self.grids), ptr(self.dk), d, ng, st)
        dk2 = self.dk[1] if self.interlaced else None
        _lib.call('pyl_pk_bin', ptr(self.dk[0]), ptr(dk2), 1, self.dk[0].numel(), d, self.axis,
                  self.mas_p, ptr(self.sums), ptr(self.pk_ws), self.pk_ws_bytes, st)
        return self.sums

    def capture(self, pos, W=None):
        """Capture one step on `pos` (fixed size and address) into a CUDA graph."""
        self.step(pos, W)           # warm-up: plans, workspace, function attributes
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(pos, W)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
        return self.sums

    def result(self, sums=None):
        s = (sums if sums is not None else self.sums).cpu().numpy()
        _lib.check_device('ParticlePk')
        return PKL.finalize_pk(s, self.geom, self.BoxSize, self.dims, 1, cross=False)
