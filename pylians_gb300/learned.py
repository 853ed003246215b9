"""Learned aliasing + window correction for coarse, non-interlaced P(k).

No counterpart in the reference.  A small MLP (4 -> 64 -> 64 -> 64 -> 1, tanh,
BF16 weights, FP32 accumulation; kernels in csrc/mlp.cu) predicts
    log(P_fine_interlaced(k) / P_coarse(k))
from four features of a monopole bin:
    x0 = k / k_Nyq (coarse grid),
    x1 = MAS exponent - 3 (CIC -1, TSC 0, PCS +1),
    x2 = power-law slope n + 1.5,
    x3 = log10(P_shot / P(k_Nyq)) / 3,  P_shot = 1 / nbar,
so that P_coarse(k) * exp(MLP(x)) stands in for the interlaced estimate on a
grid four times finer.  Training pairs come from this library itself: Gaussian
power-law fields (P ~ k^n) Poisson-sampled into particles at number density
nbar, deposited on a coarse grid without interlacing and on a 4x finer grid
with interlacing (pipeline.ParticlePk).  The plain interlaced fine-grid
estimate is both the training target and the fallback.
"""
import math
import os

import numpy as np
import torch

from . import _lib
from ._device import ptr, require_cuda, stream_ptr
from .pipeline import ParticlePk

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, 'data', 'aliasing_mlp.npz')
MAS_P = {'NGP': 1, 'CIC': 2, 'TSC': 3, 'PCS': 4}


def features(k_over_kN, MAS, slope, shot_level):
    k = np.asarray(k_over_kN, np.float64)
    x = np.empty((k.size, 4), np.float32)
    x[:, 0] = k
    x[:, 1] = MAS_P[MAS] - 3
    x[:, 2] = slope + 1.5
    x[:, 3] = shot_level / 3.0
    return x


class MLP(object):
    """Parameters on the device: FP32 master copy, BF16 working copy, Adam state."""

    def __init__(self, flat=None, seed=0, device=None):
        require_cuda()
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        self.n = _lib.load().pyl_mlp_param_count()
        if flat is None:
            flat = self.init_params(seed)
        self.master = torch.as_tensor(np.asarray(flat, np.float32), device=self.device).contiguous()
        self.bf16 = self.master.to(torch.bfloat16).contiguous()
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.grad = torch.zeros_like(self.master)
        self.step_count = 0

    @staticmethod
    def init_params(seed):
        rng = np.random.default_rng(seed)
        parts = []
        for fan_out, fan_in in ((64, 4), (64, 64), (64, 64), (1, 64)):
            parts.append(rng.normal(0.0, math.sqrt(1.0 / fan_in), fan_out * fan_in))
            parts.append(np.zeros(fan_out))
        return np.concatenate(parts).astype(np.float32)

    def forward(self, x, act=None):
        x = torch.as_tensor(x, dtype=torch.float32, device=self.device).contiguous()
        y = torch.empty(x.shape[0], dtype=torch.float32, device=self.device)
        _lib.call('pyl_mlp_forward', ptr(self.bf16), ptr(x), x.shape[0], ptr(act), ptr(y), stream_ptr())
        return y

    def gradient(self, x, t, w=None):
        """Loss gradient into self.grad; returns the loss (host float)."""
        x = torch.as_tensor(x, dtype=torch.float32, device=self.device).contiguous()
        t = torch.as_tensor(t, dtype=torch.float32, device=self.device).contiguous()
        B = x.shape[0]
        wt = None if w is None else torch.as_tensor(w, dtype=torch.float32, device=self.device).contiguous()
        wsum = float(B if w is None else wt.sum().item())
        act = torch.empty((B, 192), dtype=torch.float32, device=self.device)
        delta = torch.empty_like(act)
        dy = torch.empty(B, dtype=torch.float32, device=self.device)
        y = self.forward(x, act)
        _lib.call('pyl_mlp_backward', ptr(self.bf16), ptr(x), ptr(act), ptr(y), ptr(t), ptr(wt), wsum, B,
                  ptr(delta), ptr(dy), ptr(self.grad), stream_ptr())
        r = (y - t) ** 2
        return float(((r if wt is None else r * wt).sum() / wsum).item())

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        _lib.call('pyl_mlp_adam', ptr(self.master), ptr(self.bf16), ptr(self.grad), ptr(self.m), ptr(self.v),
                  self.n, lr, beta1, beta2, eps, self.step_count, stream_ptr())

    def params(self):
        return self.master.cpu().numpy()

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, params=self.params())

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device=None):
        return cls(np.load(path)['params'], device=device)


# ------------------------------------------------------------- training pairs
def gaussian_field(M, L, slope, seed, sigma=0.3, device=None):
    """Gaussian field on an M^3 grid with P(k) = A (k / k_ref)^slope (k_ref = pi M / (2L)),
    scaled to rms sigma; returns (delta float32 CUDA tensor, A)."""
    dev = device or torch.device('cuda', torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    w = torch.randn((M, M, M), generator=gen, device=dev, dtype=torch.float32)
    wk = torch.empty((M, M, M // 2 + 1), dtype=torch.complex64, device=dev)
    _lib.call('pyl_fft_r2c', ptr(w), ptr(wk), M, 1, stream_ptr())
    kf = torch.fft.fftfreq(M, d=1.0 / M, device=dev)
    kz = torch.arange(M // 2 + 1, device=dev, dtype=torch.float32)
    k2 = kf[:, None, None] ** 2 + kf[None, :, None] ** 2 + kz[None, None, :] ** 2
    kmag = torch.sqrt(k2) * (2 * math.pi / L)
    k_ref = math.pi * M / (2.0 * L)
    amp = torch.where(k2 > 0, (kmag / k_ref).clamp_min(1e-12) ** (slope / 2.0), torch.zeros_like(kmag))
    wk *= amp * math.sqrt((M / L) ** 3)
    d = torch.empty((M, M, M), dtype=torch.float32, device=dev)
    _lib.call('pyl_fft_c2r', ptr(wk), ptr(d), M, 1, stream_ptr())
    d /= float(M) ** 3
    s = float(d.std().item())
    d *= sigma / s
    return d, (sigma / s) ** 2


def poisson_particles(delta, L, nbar, seed):
    """Particles with expected density nbar (1 + delta), uniform inside each cell."""
    dev = delta.device
    M = delta.shape[0]
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed) + 7919)
    lam = (nbar * (L / M) ** 3) * (1.0 + delta).clamp_min(0.0)
    counts = torch.poisson(lam, generator=gen).to(torch.int64).reshape(-1)
    cells = torch.repeat_interleave(torch.arange(M ** 3, device=dev), counts)
    ix, iy, iz = cells // (M * M), (cells // M) % M, cells % M
    u = torch.rand((cells.numel(), 3), generator=gen, device=dev)
    pos = torch.stack([ix, iy, iz], 1).to(torch.float32).add_(u).mul_(L / M)
    return pos.contiguous()


def make_pair(N, slope, nbar, MAS='CIC', seed=0, n_target=2_000_000, axis=0):
    """One (coarse plain, 4x fine interlaced) pair: features, log-ratio target and both P(k)."""
    L = (n_target / nbar) ** (1.0 / 3.0)
    delta, A = gaussian_field(2 * N, L, slope, seed)
    pos = poisson_particles(delta, L, nbar, seed)
    del delta
    n = pos.shape[0]
    c = ParticlePk(N, L, MAS, axis=axis, interlaced=False, max_particles=n)
    c.step(pos)
    rc = c.result()
    f = ParticlePk(4 * N, L, MAS, axis=axis, interlaced=True, max_particles=n)
    f.step(pos)
    rf = f.result()
    kN = math.pi * N / L
    nb = len(rc.k3D)
    Pc, Pf = rc.Pk[:, 0], rf.Pk[:nb, 0]
    sel = (rc.k3D <= 0.8 * kN) & (Pc > 0) & (Pf > 0)
    shot = math.log10((1.0 / nbar) / A)
    x = features(rc.k3D[sel] / kN, MAS, slope, shot)
    t = np.log(Pf[sel] / Pc[sel]).astype(np.float32)
    return dict(x=x, t=t, k=rc.k3D[sel], Pc=Pc[sel], Pf=Pf[sel], N=N, L=L, slope=slope, nbar=nbar,
                MAS=MAS, shot=shot, n=n, Nmodes=rc.Nmodes3D[sel])


def training_set(count, seed=0, coarse=(32, 64), mas=('CIC', 'TSC', 'PCS'), n_target=1_000_000):
    """Pairs with slope n in [-2.5, -0.5] and nbar log-uniform in [1e-4, 1] (h/Mpc)^3."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        out.append(make_pair(int(rng.choice(coarse)), float(rng.uniform(-2.5, -0.5)),
                             float(10 ** rng.uniform(-4, 0)), str(rng.choice(mas)),
                             seed=seed * 100003 + i, n_target=n_target))
    return out


def train(pairs, steps=2000, lr=2e-3, seed=0, model=None):
    x = np.concatenate([p['x'] for p in pairs])
    t = np.concatenate([p['t'] for p in pairs])
    net = model or MLP(seed=seed)
    xd = torch.as_tensor(x, device=net.device)
    td = torch.as_tensor(t, device=net.device)
    losses = []
    for s in range(steps):
        rate = lr * (0.5 * (1 + math.cos(math.pi * s / steps)) * 0.95 + 0.05)
        losses.append(net.gradient(xd, td))
        net.adam(rate)
    return net, losses


class Correction(object):
    """P_coarse(k) * exp(MLP(features)) on monopole bins below 0.8 k_Nyq."""

    def __init__(self, net=None, path=DEFAULT_WEIGHTS):
        self.net = net or MLP.load(path)

    def factor(self, k, kN, MAS, slope, shot_level):
        x = features(np.asarray(k) / kN, MAS, slope, shot_level)
        return np.exp(self.net.forward(x).cpu().numpy().astype(np.float64))

    def apply(self, k, Pk0, kN, MAS, slope, shot_level):
        return np.asarray(Pk0) * self.factor(k, kN, MAS, slope, shot_level)


def estimate_slope(k, Pk0, kN, lo=0.1, hi=0.4):
    """Power-law slope from a log-log fit of the coarse monopole between lo and hi k_Nyq."""
    sel = (k > lo * kN) & (k < hi * kN) & (Pk0 > 0)
    return float(np.polyfit(np.log(k[sel]), np.log(Pk0[sel]), 1)[0])


def main():
    """Train on the device and save DEFAULT_WEIGHTS (python -m pylians_gb300.learned)."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument('--pairs', type=int, default=96)
    ap.add_argument('--steps', type=int, default=6000)
    ap.add_argument('--out', default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    pairs = training_set(a.pairs, seed=1)
    net, losses = train(pairs, steps=a.steps)
    net.save(a.out)
    print('trained on %d pairs (%d bins): loss %.3e -> %.3e, saved %s'
          % (len(pairs), sum(len(p['t']) for p in pairs), losses[0], losses[-1], a.out))


if __name__ == '__main__':
    main()
