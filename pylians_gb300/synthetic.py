"""Seeded synthetic inputs with the shapes of the benchmark configurations.

Simulation snapshots are not available, so the workloads run on generated
particles (the reference's own tests use none either):
  * uniform(n, BoxSize, seed): float32 positions uniform in [0, BoxSize);
  * gaussian_field(N, BoxSize, pk, sigma, seed): a Gaussian random field on an
    N^3 grid with power spectrum shape pk(k) (h/Mpc), scaled to rms sigma;
  * zeldovich(...): lattice particles displaced by the Zel'dovich displacement
    Psi_k = i k / k^2 delta_k of such a field, with the linear redshift-space
    distortion s = x + f Psi along one axis applied through
    redshift_space_library.pos_redshift_space (velocity f H Psi at z = 0).
The field FFTs, the displacement interpolation (CIC_interp) and the redshift
shift run on this library's kernels; torch element-wise operations do the rest.
"""
import math

import torch

from . import _lib
from ._device import ptr, require_cuda, stream_ptr

HUBBLE = 100.0      # (km/s)/(Mpc/h) at z = 0


def uniform(n, BoxSize, seed, device=None):
    dev = device or torch.device('cuda', torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    return torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float32) * float(BoxSize)


def _kgrid(N, BoxSize, dev):
    kf = torch.fft.fftfreq(N, d=1.0 / N, device=dev) * (2 * math.pi / BoxSize)
    kz = torch.arange(N // 2 + 1, device=dev, dtype=torch.float32) * (2 * math.pi / BoxSize)
    return kf, kz


def zeldovich_pk(k, n=-1.5, kcut=0.5):
    """P(k) shape k^n exp(-(k/kcut)^2) (amplitude set by the field's rms)."""
    return torch.where(k > 0, k.clamp_min(1e-30) ** n * torch.exp(-(k / kcut) ** 2), torch.zeros_like(k))


def gaussian_field_k(N, BoxSize, pk=zeldovich_pk, sigma=0.5, seed=0, device=None):
    """Half-complex Fourier modes (complex64 [N][N][N/2+1], unnormalised forward
    convention) of a Gaussian field whose real-space rms is `sigma`."""
    require_cuda()
    dev = device or torch.device('cuda', torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    w = torch.randn((N, N, N), generator=gen, device=dev, dtype=torch.float32)
    dk = torch.empty((N, N, N // 2 + 1), dtype=torch.complex64, device=dev)
    _lib.call('pyl_fft_r2c', ptr(w), ptr(dk), N, 1, stream_ptr())
    del w
    kf, kz = _kgrid(N, BoxSize, dev)
    k = torch.sqrt(kf[:, None, None] ** 2 + kf[None, :, None] ** 2 + kz[None, None, :] ** 2)
    dk *= torch.sqrt(pk(k))
    d = torch.empty((N, N, N), dtype=torch.float32, device=dev)
    _lib.call('pyl_fft_c2r', ptr(dk.clone()), ptr(d), N, 1, stream_ptr())
    rms = float(d.double().std().item()) / float(N) ** 3      # the C2R is unnormalised
    dk *= sigma / rms
    return dk


def displacement(dk, BoxSize):
    """Zel'dovich displacement fields Psi_a(x) = IFFT(i k_a / k^2 delta_k), a = 0, 1, 2
    (float32 [3][N][N][N], Mpc/h)."""
    N = dk.shape[0]
    dev = dk.device
    kf, kz = _kgrid(N, BoxSize, dev)
    k2 = kf[:, None, None] ** 2 + kf[None, :, None] ** 2 + kz[None, None, :] ** 2
    inv_k2 = torch.where(k2 > 0, 1.0 / k2.clamp_min(1e-30), torch.zeros_like(k2))
    out = torch.empty((3, N, N, N), dtype=torch.float32, device=dev)
    comps = (kf[:, None, None], kf[None, :, None], kz[None, None, :])
    for a in range(3):
        pk = dk * (1j * comps[a] * inv_k2)
        # Nyquist planes carry no odd (imaginary-derivative) part of a real field
        if N % 2 == 0:
            if a == 0:
                pk[N // 2] = 0
            elif a == 1:
                pk[:, N // 2] = 0
            else:
                pk[:, :, N // 2] = 0
        _lib.call('pyl_fft_c2r', ptr(pk.contiguous()), ptr(out[a]), N, 1, stream_ptr())
        out[a] /= float(N) ** 3
    return out


def zeldovich(N_field=256, N_lattice=512, BoxSize=1000.0, sigma=0.5, f=0.5, rsd_axis=2, seed=1,
              pk=zeldovich_pk, device=None):
    """N_lattice^3 particles (float32 [n][3], CUDA) at lattice cell centres displaced by
    the Zel'dovich displacement of a Gaussian field on an N_field^3 grid, then moved to
    redshift space along `rsd_axis` with linear growth rate f (skip with rsd_axis=None)."""
    require_cuda()
    from .MAS_library import CIC_interp
    from .redshift_space_library import pos_redshift_space
    dk = gaussian_field_k(N_field, BoxSize, pk, sigma, seed, device)
    psi = displacement(dk, BoxSize)
    del dk
    dev = psi.device
    M = N_lattice
    cell = BoxSize / M
    g = (torch.arange(M, device=dev, dtype=torch.float32) + 0.5) * cell
    q = torch.stack(torch.meshgrid(g, g, g, indexing='ij'), dim=-1).reshape(-1, 3).contiguous()
    n = q.shape[0]
    disp = torch.empty((n, 3), dtype=torch.float32, device=dev)
    tmp = torch.empty(n, dtype=torch.float32, device=dev)
    for a in range(3):
        CIC_interp(psi[a].contiguous(), BoxSize, q, tmp)
        disp[:, a] = tmp
    del psi, tmp
    pos = torch.remainder(q + disp, float(BoxSize))
    pos = torch.where(pos >= BoxSize, pos - BoxSize, pos).contiguous()
    del q
    if rsd_axis is not None:
        vel = (disp * (f * HUBBLE)).contiguous()
        pos_redshift_space(pos, vel, BoxSize, HUBBLE, 0.0, rsd_axis)
        del vel
    return pos
