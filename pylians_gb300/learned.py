"""Learned aliasing + window correction for coarse, non-interlaced P(k).

No counterpart in the reference.  A small MLP (4 -> 64 -> 64 -> 64 -> 1, tanh,
BF16 weights, FP32 accumulation; kernels in csrc/mlp.cu) predicts
    log(P_fine_interlaced(k) / P_coarse(k))
from four features of a monopole bin:
    x0 = k / k_Nyq (coarse grid),
    x1 = MAS exponent - 3 (CIC -1, TSC 0, PCS +1),
    x2 = power-law slope n + 1.5,
    x3 = log10(P_shot / P(k_Nyq)) / 3,  P_shot = 1 / nbar,
so that P_coarse(k) * exp(x0^2 MLP(x)) stands in for the interlaced estimate on a
grid four times finer (the x0^2 envelope makes the correction vanish as k -> 0,
where the coarse estimate is already exact).  Training pairs come from this library itself: Gaussian
power-law fields (P ~ k^n) Poisson-sampled into particles at number density
nbar, deposited on a coarse grid without interlacing and on a 4x finer grid
with interlacing (pipeline.ParticlePk).  The plain interlaced fine-grid
estimate is both the training target and the fallback.
"""
import json
import math
import os
import time

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
        """Hidden layers N(0, 1/fan_in); the output layer starts at zero, so an untrained
        network predicts no correction (the plain coarse estimate)."""
        rng = np.random.default_rng(seed)
        parts = []
        for fan_out, fan_in in ((64, 4), (64, 64), (64, 64), (1, 64)):
            std = 0.0 if fan_out == 1 else math.sqrt(1.0 / fan_in)
            parts.append(rng.normal(0.0, 1.0, fan_out * fan_in) * std)
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

    def save(self, path, provenance=None):
        """Parameters (and, when given, a JSON string saying how they were trained)."""
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        extra = {'provenance': np.array(provenance)} if provenance else {}
        np.savez(path, params=self.params(), **extra)

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


def make_pair(N, slope, nbar, MAS='CIC', seed=0, n_target=2_000_000, axis=0, sigma=0.3, kmax=0.85):
    """One (coarse plain, 4x fine interlaced) pair: features, log-ratio target and both P(k).
    The slope and shot-level features are the ones estimate_features measures on the coarse
    spectrum (as at inference); the true values are kept beside them."""
    L = (n_target / nbar) ** (1.0 / 3.0)
    delta, A = gaussian_field(2 * N, L, slope, seed, sigma=sigma)
    pos = poisson_particles(delta, L, nbar, seed)
    del delta
    n = pos.shape[0]
    c = ParticlePk(N, L, MAS, axis=axis, interlaced=False, max_particles=n)
    c.step(pos)
    rc = c.result()
    del c
    f = ParticlePk(4 * N, L, MAS, axis=axis, interlaced=True, max_particles=n)
    f.step(pos)
    rf = f.result()
    del f, pos
    torch.cuda.empty_cache()
    kN = math.pi * N / L
    nb = len(rc.k3D)
    Pc, Pf = rc.Pk[:, 0], rf.Pk[:nb, 0]
    sel = (rc.k3D > 0) & (rc.k3D <= kmax * kN) & (Pc > 0) & (Pf > 0)
    s_est, shot_est = estimate_features(rc.k3D, Pc, kN, nbar)
    x = features(rc.k3D[sel] / kN, MAS, s_est, shot_est)
    t = np.log(Pf[sel] / Pc[sel]).astype(np.float32)
    return dict(x=x, t=t, k=rc.k3D[sel], Pc=Pc[sel], Pf=Pf[sel], N=N, L=L, slope=slope, nbar=nbar,
                MAS=MAS, shot=math.log10((1.0 / nbar) / A), slope_est=s_est, shot_est=shot_est, n=n,
                Nmodes=rc.Nmodes3D[sel])


# Particles of one training pair at most: the 4N = 2048 interlaced fine grid of an N = 512
# pair (two 2048^3 grids, their transforms and the binning workspace, about 200 GB with
# 1024^3 particles) leaves no room for more.
MAX_PAIR_PARTICLES = 1 << 30


def training_set(count, seed=0, coarse=(128, 256, 512), mas=('CIC', 'TSC', 'PCS'), density=(0.25, 4.0),
                 sigma=(0.1, 0.6)):
    """Pairs with slope n in [-2.5, -0.5], nbar log-uniform in [1e-4, 1] (h/Mpc)^3, particle
    count (2N)^3 times a log-uniform factor in `density` (at most MAX_PAIR_PARTICLES), field
    rms log-uniform in `sigma`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        N = int(rng.choice(coarse))
        n_target = int((2 * N) ** 3 * math.exp(rng.uniform(math.log(density[0]), math.log(density[1]))))
        n_target = min(n_target, MAX_PAIR_PARTICLES)
        out.append(make_pair(N, float(rng.uniform(-2.5, -0.5)), float(10 ** rng.uniform(-4, 0)),
                             str(rng.choice(mas)), seed=seed * 100003 + i, n_target=n_target,
                             sigma=float(math.exp(rng.uniform(math.log(sigma[0]), math.log(sigma[1]))))))
    return out


def train(pairs, steps=2000, lr=2e-3, seed=0, model=None):
    """Adam with a cosine learning-rate decay on all bins at once.  The network output y
    enters as log ratio = x0^2 y, so it is fitted to t / x0^2 with weights x0^4: the same
    squared error in the log ratio."""
    x = np.concatenate([p['x'] for p in pairs])
    t = np.concatenate([p['t'] for p in pairs]).astype(np.float64)
    x0 = x[:, 0].astype(np.float64)
    net = model or MLP(seed=seed)
    xd = torch.as_tensor(x, device=net.device)
    td = torch.as_tensor((t / x0 ** 2).astype(np.float32), device=net.device)
    wd = torch.as_tensor((x0 ** 4 / np.mean(x0 ** 4)).astype(np.float32), device=net.device)
    losses = []
    for s in range(steps):
        rate = lr * (0.5 * (1 + math.cos(math.pi * s / steps)) * 0.95 + 0.05)
        losses.append(net.gradient(xd, td, wd))
        net.adam(rate)
    return net, losses


class Correction(object):
    """P_coarse(k) * exp((k/k_Nyq)^2 MLP(features)) on monopole bins below 0.8 k_Nyq."""

    def __init__(self, net=None, path=DEFAULT_WEIGHTS):
        self.net = net or MLP.load(path)

    def factor(self, k, kN, MAS, slope, shot_level):
        x = features(np.asarray(k) / kN, MAS, slope, shot_level)
        y = self.net.forward(x).cpu().numpy().astype(np.float64)
        return np.exp(x[:, 0].astype(np.float64) ** 2 * y)

    def apply(self, k, Pk0, kN, MAS, slope, shot_level):
        return np.asarray(Pk0) * self.factor(k, kN, MAS, slope, shot_level)


def estimate_features(k, Pk0, kN, nbar, lo=0.1, hi=0.4):
    """(slope, shot level) of a coarse monopole: a power law is fitted to P(k) - 1/nbar
    between lo and hi k_Nyq and extrapolated to k_Nyq; shot level = log10((1/nbar) / P(k_Nyq))."""
    shot = 1.0 / nbar
    sel = (k > lo * kN) & (k < hi * kN) & (Pk0 - shot > 0)
    if sel.sum() < 3:       # shot noise dominates the fit range: fit what is above it below hi
        sel = (k < hi * kN) & (Pk0 - shot > 0)
    if sel.sum() < 2:
        raise ValueError('no bins with power above shot noise below %.2f k_Nyq' % hi)
    b, a = np.polyfit(np.log(k[sel]), np.log(Pk0[sel] - shot), 1)
    lpn = (a + b * math.log(kN)) / math.log(10.0)
    return float(b), float(math.log10(shot) - lpn)


def _timed(fn, reps):
    """Median host wall time (ms) of fn() with a device synchronize on both sides."""
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        ts.append((time.perf_counter() - w0) * 1e3)
    return float(np.median(ts)), out


def _device_ms(fn, reps):
    """Mean CUDA-event time (ms) of fn()'s launches on the current stream."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def evaluate(N=512, side=1024, slope=-1.5, L=1000.0, MAS='CIC', seed=11, oracle_grid=0, reps=3,
             net=None):
    """Learned-corrected N^3 non-interlaced P(k) against the plain interlaced (2N)^3 estimate of
    the same side^3 (expected) Poisson particles of a power-law field, and optionally against
    an interlaced oracle_grid^3 estimate.

    Features are estimated from the coarse spectrum itself (estimate_features) and the
    known number density.  Returns a dict with the maximum and mean |ratio - 1| up to
    0.8 k_Nyq of the coarse grid and the wall-clock times of both paths (pipeline step,
    bin sums to host, P(k) finalisation, and for the coarse path the MLP correction)."""
    require_cuda()
    corr = Correction(net)
    nbar = float(side) ** 3 / L ** 3
    delta, _ = gaussian_field(2 * N, L, slope, seed)
    pos = poisson_particles(delta, L, nbar, seed)
    del delta
    torch.cuda.empty_cache()
    n = pos.shape[0]
    kN = math.pi * N / L
    c = ParticlePk(N, L, MAS, axis=0, interlaced=False, max_particles=n)
    f = ParticlePk(2 * N, L, MAS, axis=0, interlaced=True, max_particles=n)

    def coarse():
        c.step(pos)
        r = c.result()
        s, shot = estimate_features(r.k3D, r.Pk[:, 0], kN, nbar)
        return r, corr.apply(r.k3D, r.Pk[:, 0], kN, MAS, s, shot), s, shot

    def fine():
        f.step(pos)
        return f.result()

    t_c, (rc, Pcorr, s_est, shot_est) = _timed(coarse, reps)
    t_f, rf = _timed(fine, reps)
    dev_c = _device_ms(lambda: c.step(pos), reps)
    dev_f = _device_ms(lambda: f.step(pos), reps)
    nb = len(rc.k3D)
    sel = (rc.k3D <= 0.8 * kN) & (rc.Nmodes3D > 0)
    Pf = rf.Pk[:nb, 0]
    err_c = np.abs(Pcorr[sel] / Pf[sel] - 1.0)
    err_plain = np.abs(rc.Pk[sel, 0] / Pf[sel] - 1.0)
    out = dict(N_coarse=N, N_fine=2 * N, particles=int(n), box=L, slope=slope, MAS=MAS,
               slope_est=s_est, shot_level_est=shot_est, k_max=float(0.8 * kN), bins=int(sel.sum()),
               max_err_learned=float(err_c.max()), mean_err_learned=float(err_c.mean()),
               max_err_plain=float(err_plain.max()), mean_err_plain=float(err_plain.mean()),
               ms_coarse_learned=t_c, ms_fine_interlaced=t_f, speedup=t_f / t_c,
               device_ms_coarse_step=dev_c, device_ms_fine_step=dev_f,
               k=rc.k3D[sel].tolist(), ratio_learned=(Pcorr[sel] / Pf[sel]).tolist(),
               ratio_plain=(rc.Pk[sel, 0] / Pf[sel]).tolist())
    del c, f
    torch.cuda.empty_cache()
    if oracle_grid:
        o = ParticlePk(oracle_grid, L, MAS, axis=0, interlaced=True, max_particles=n)
        o.step(pos)
        ro = o.result()
        del o
        torch.cuda.empty_cache()
        Po = ro.Pk[:nb, 0]
        out.update(oracle_grid=oracle_grid,
                   max_err_learned_vs_oracle=float(np.abs(Pcorr[sel] / Po[sel] - 1).max()),
                   max_err_fine_vs_oracle=float(np.abs(Pf[sel] / Po[sel] - 1).max()),
                   ratio_fine_vs_oracle=(Pf[sel] / Po[sel]).tolist())
    return out


def main():
    """Train on the device and save DEFAULT_WEIGHTS (python -m pylians_gb300.learned), or
    with --evaluate write the evaluation of the saved weights as JSON."""
    import argparse
    ap = argparse.ArgumentParser()
    # the shipped weights (data/aliasing_mlp.npz) are these defaults' result
    ap.add_argument('--pairs', type=int, default=160)
    ap.add_argument('--steps', type=int, default=20000)
    ap.add_argument('--seed', type=int, default=1)
    ap.add_argument('--out', default=DEFAULT_WEIGHTS)
    ap.add_argument('--evaluate', default=None, help='write the evaluation JSON here')
    ap.add_argument('--coarse', type=int, default=512)
    ap.add_argument('--side', type=int, default=1024)
    ap.add_argument('--oracle-grid', type=int, default=0)
    ap.add_argument('--slope', type=float, default=-1.5)
    ap.add_argument('--mas', default='CIC')
    ap.add_argument('--weights', default=DEFAULT_WEIGHTS)
    ap.add_argument('--pairs-out', default=None, help='also save the training pairs (npz)')
    a = ap.parse_args()
    if a.evaluate:
        res = evaluate(N=a.coarse, side=a.side, slope=a.slope, MAS=a.mas, oracle_grid=a.oracle_grid,
                       net=MLP.load(a.weights))
        with open(a.evaluate, 'w') as fh:
            json.dump(res, fh)
        print(json.dumps({k: v for k, v in res.items() if not isinstance(v, list)}))
        return
    pairs = training_set(a.pairs, seed=a.seed)
    if a.pairs_out:
        np.savez(a.pairs_out, x=np.concatenate([p['x'] for p in pairs]),
                 t=np.concatenate([p['t'] for p in pairs]),
                 pair=np.concatenate([np.full(len(p['t']), i) for i, p in enumerate(pairs)]),
                 meta=np.array([(p['N'], p['slope'], p['slope_est'], p['shot'], p['shot_est'], p['n'],
                                 p['nbar'], MAS_P[p['MAS']]) for p in pairs]))
    net, losses = train(pairs, steps=a.steps)
    sizes = {int(N): sum(1 for p in pairs if p['N'] == N) for N in sorted({p['N'] for p in pairs})}
    net.save(a.out, json.dumps(dict(command='python -m pylians_gb300.learned --pairs %d --steps %d --seed %d'
                                            % (a.pairs, a.steps, a.seed), pairs_by_coarse_side=sizes,
                                    bins=int(sum(len(p['t']) for p in pairs)), loss_first=float(losses[0]),
                                    loss_last=float(losses[-1]))))
    print('trained on %d pairs %s (%d bins): loss %.3e -> %.3e, saved %s'
          % (len(pairs), sizes, sum(len(p['t']) for p in pairs), losses[0], losses[-1], a.out))


if __name__ == '__main__':
    main()
