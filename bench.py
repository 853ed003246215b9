"""Benchmark: CIC + interlaced P(k) of 1024^3 particles on a 1024^3 grid, one GB300.

One step = the whole particle -> P(k) chain on one batch of synthetic particles
already resident in HBM: zero both grids, CIC deposit into the grid and its
half-cell-shifted twin, overdensity (mean = N/dims^3), batched R2C of both
grids, fused interlace + deconvolve + |k|/mu binning + l=0,2,4 sums.
  value  particles/s over K device-timed steps (CUDA events, max over ranks)
  e2e    the same chain through ParticlePk with the positions copied from pinned
         host memory every step and the float64 bin sums read back every step
  roofline   the dominant stage's algorithmic bytes / its CUDA-event duration
  cpu_baseline   the oracle (C restatement of the reference's MAS_c.c scatter and
         Pk mode loop, scipy float32 FFT) on all host cores, on a 256^3 sample
--impl reference: the same CPU port timed as the reference arm.

Inputs (12.9 GB of positions) are larger than L2 (129 MB), so no flush is needed
between steps.  Synthetic data: uniform positions in a 1000 Mpc/h box, seed 1.
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'CIC+interlaced P(k) particles/s'
UNIT = 'particles/s'
BOX = 1000.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--grid', type=int, default=1024)
    ap.add_argument('--particles-side', type=int, default=1024)
    ap.add_argument('--cpu-side', type=int, default=512, help='side of the CPU baseline sample')
    ap.add_argument('--no-secondary', action='store_true')
    ap.add_argument('--secondary-only', default=None, choices=['zeldovich', 'bispectrum', 'batch', 'learned'],
                    help='run only this secondary workload and print its JSON (profiling)')
    ap.add_argument('--batch-size', type=int, default=512)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--strategy', default='auto', choices=['auto', 'atomic', 'tiled', 'sorted'])
    ap.add_argument('--owned-min-dims', type=int, default=-1,
                    help='grids from this side up take the owned-cell write-out (profiling the 1024^3 '
                         'deposit path on a smaller case; default: the library\'s own threshold)')
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest of every rank's x (one all_reduce MAX in float64 on `device`,
    a CUDA device under NCCL, 'cpu' under gloo); x itself for one rank."""
    if world == 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.item()


def whole_job_rate(units_per_rank, steps, world, ms):
    """Units per second of the whole job: every replica processes units_per_rank
    per step, and the job takes the slowest rank's ms."""
    return units_per_rank * steps * world / (ms / 1e3)


# ------------------------------------------------------------------ CPU baseline
def cpu_chain(pos, dims, threads):
    """The reference's CPU path on `pos`: MAS_c.c-style OpenMP CIC into two grids,
    overdensity, float32 FFTs, the Pk mode loop (oracle restatement)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    n = pos.shape[0]
    a = np.zeros((dims,) * 3, np.float32)
    b = np.zeros((dims,) * 3, np.float32)
    O.ma_kernel(pos, a, BOX, 'CIC', None, threads=threads, flavor=1)
    pos2 = (pos + np.float32(0.5 * BOX / dims)).astype(np.float32)
    O.ma_kernel(pos2, b, BOX, 'CIC', None, threads=threads, flavor=1)
    m = np.float32(n / dims ** 3)
    a /= m; a -= np.float32(1)
    b /= m; b -= np.float32(1)
    return O.Pk(a, BOX, 0, 'CIC', threads, interlaced=b)


def cpu_sample(side, seed=1):
    rng = np.random.default_rng(seed)
    return (rng.random((side ** 3, 3), dtype=np.float32) * np.float32(BOX)).astype(np.float32)


def run_cpu_baseline(side):
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    pos = cpu_sample(side)
    cpu_chain(pos[: min(len(pos), 4096)], 16, threads)   # warm the library
    t0 = time.perf_counter()
    cpu_chain(pos, side, threads)
    dt = time.perf_counter() - t0
    return dict(value=pos.shape[0] / dt, unit=UNIT, cores=threads, kind='port',
                sample='%d^3 particles CIC+interlaced onto %d^3 grids + P(k) axis 0 (%.2f s)'
                % (side, side, dt))


def reference_arm(a):
    """The reference's CPU path (the oracle port: MAS_c.c-style OpenMP CIC, float32 FFTs,
    the Pk mode loop) on the GPU arm's own workload.  The K timed steps together process
    exactly one headline workload: step i deposits the i-th of K equal slices of the
    particles (uniform, seeded per slice) onto the two dims^3 grids, and the last step
    also runs the overdensity, both FFTs and the mode loop.  value = particles of the
    workload / total time of the K steps.  Warm-up steps deposit slices into scratch
    grids of the same size (not timed)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    dims, side = a.grid, a.particles_side
    n = side ** 3
    K = max(1, a.steps)
    slice_n = -(-n // K)
    half = np.float32(0.5 * BOX / dims)

    def deposit(g1, g2, count, seed):
        rng = np.random.default_rng(seed)
        pos = (rng.random((count, 3), dtype=np.float32) * np.float32(BOX)).astype(np.float32)
        O.ma_kernel(pos, g1, BOX, 'CIC', None, threads=threads, flavor=1)
        pos += half
        O.ma_kernel(pos, g2, BOX, 'CIC', None, threads=threads, flavor=1)

    g1 = np.zeros((dims,) * 3, np.float32)
    g2 = np.zeros((dims,) * 3, np.float32)
    for i in range(a.warmup):
        deposit(g1, g2, slice_n, 1000 + i)
    g1[...] = 0.0
    g2[...] = 0.0
    t0 = time.perf_counter()
    done = 0
    for i in range(K):
        cnt = min(slice_n, n - done)
        deposit(g1, g2, cnt, 1 + i)
        done += cnt
        if i == K - 1:
            m = np.float32(n / dims ** 3)
            for g in (g1, g2):
                g /= m
                g -= np.float32(1)
            O.Pk(g1, BOX, 0, 'CIC', threads, interlaced=g2)
    dt = time.perf_counter() - t0
    v = n / dt
    line = dict(metric=METRIC, value=v, unit=UNIT, n_gpus=world, steps=a.steps, warmup=a.warmup,
                ms_per_step=dt / K * 1e3, higher_is_better=True, scaling='weak',
                vs_baseline=None, dtype='f32', data='synthetic',
                config=headline_config(side, dims, a.strategy),
                impl='reference',
                cpu_baseline=dict(value=v, unit=UNIT, cores=threads, kind='port',
                                  sample='the whole workload: %d^3 particles in %d slices onto two %d^3 grids, '
                                         'then overdensity, two FFTs and the P(k) mode loop (%.1f s)'
                                         % (side, K, dims, dt)),
                e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))


def headline_config(side, dims, strategy):
    return dict(workload='cic_interlaced_pk_np%d^3_grid%d^3' % (side, dims),
                particles=side ** 3, grid=dims, box_mpc_h=BOX, axis=0, MAS='CIC',
                interlaced=True, strategy=strategy, parallelism='replicas',
                l2_flush='inputs larger than L2 (%.1f GB positions)' % (12.0 * side ** 3 / 1e9))


# ----------------------------------------------------------------------- clocks
class ClockSampler(object):
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples (kept beside the run's other output when PYL_CLOCKS_DIR
        # names a directory); the JSON line carries their summary
        out_dir = os.environ.get('PYL_CLOCKS_DIR') or tempfile.gettempdir()
        self.path = os.path.join(out_dir, 'clocks_bench_%d.csv' % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.QUERY,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in open(self.path):
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        if not sm:
            return None
        return dict(sm_mhz=float(np.median(sm)), sm_max_mhz=mx, reasons=sorted(reasons),
                    samples=len(sm))


# -------------------------------------------------------------------- GPU arm
def main():
    a = parse()
    if a.impl == 'reference':
        return reference_arm(a)
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if a.secondary_only:
        import pylians_gb300.build as pb
        pb.build()
        fn = dict(zeldovich=bench_zeldovich, bispectrum=bench_bispectrum, learned=bench_learned,
                  batch=lambda: bench_batch(a.batch_size))[a.secondary_only]
        print(json.dumps({a.secondary_only: fn()}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    import pylians_gb300.build as pb
    pb.build()
    from pylians_gb300.pipeline import ParticlePk
    from pylians_gb300 import _lib
    if a.owned_min_dims > 0:
        _lib.call('pyl_ma_set_thresholds', a.owned_min_dims, -1.0)

    dims, side = a.grid, a.particles_side
    n = side ** 3
    dev = torch.device('cuda', local)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1 + rank)
    pos = torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float32) * BOX
    pp = ParticlePk(dims, BOX, 'CIC', axis=0, interlaced=True, strategy=a.strategy, max_particles=n)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(a.warmup):
        pp.step(pos)
    torch.cuda.synchronize()

    # ---- device-resident throughput
    clocks = ClockSampler(local)
    clocks.start()
    barrier(); torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        pp.step(pos)
    e1.record()
    torch.cuda.synchronize(); barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    clk = clocks.stop()
    value = whole_job_rate(n, a.steps, world, ms)
    res = pp.result()
    assert int(res.Nmodes3D.sum()) + 1 == (dims ** 3 - 8) // 2 + 8

    # ---- per-stage durations (events between C-ABI calls on the launching stream)
    stages = stage_times(pp, pos, reps=max(2, min(a.steps, 5)))
    grids = grids_per_s(pp, reps=max(3, min(a.steps, 10)))

    # ---- end to end: pinned host positions -> device -> chain -> sums to host.
    # Two device position buffers: the copy of step i+1 runs on a copy stream
    # while step i computes; every step still moves its 12.9 GB and its sums.
    e2e = None
    if not a.no_e2e:
        host = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        host.copy_(pos)
        del pos
        torch.cuda.empty_cache()
        sums_host = torch.empty(pp.sums.shape, dtype=torch.float64, pin_memory=True)
        bufs = [torch.empty((n, 3), dtype=torch.float32, device=dev) for _ in range(2)]
        comp = torch.cuda.current_stream()
        cps = torch.cuda.Stream()
        copied = [torch.cuda.Event() for _ in range(2)]
        free = [torch.cuda.Event() for _ in range(2)]
        # copy-stream events around every H2D copy: the link bandwidth each step saw
        cpy = []

        def copy_into(b):
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record(cps)
            bufs[b].copy_(host, non_blocking=True)
            c1.record(cps)
            copied[b].record(cps)
            cpy.append((c0, c1))

        def run(k2):
            with torch.cuda.stream(cps):
                copy_into(0)
            for i in range(k2):
                b = i % 2
                comp.wait_event(copied[b])
                pp.step(bufs[b])
                free[b].record(comp)
                sums_host.copy_(pp.sums, non_blocking=True)
                if i + 1 < k2:
                    nb = (i + 1) % 2
                    with torch.cuda.stream(cps):
                        if i >= 1:
                            cps.wait_event(free[nb])
                        copy_into(nb)
        run(2)
        torch.cuda.synchronize(); barrier()
        cpy.clear()
        k2 = a.steps
        t0 = time.perf_counter()
        e0.record()
        run(k2)
        e1.record()
        torch.cuda.synchronize(); barrier()
        ms2 = max_over_ranks(e0.elapsed_time(e1), world, dev)
        wall = max_over_ranks((time.perf_counter() - t0) * 1e3, world, dev)
        hbytes = host.numel() * 4
        h2d_ms = [c0.elapsed_time(c1) for c0, c1 in cpy]
        e2e = dict(value=whole_job_rate(n, k2, world, ms2), unit=UNIT,
                   h2d_bytes_per_step=int(hbytes),
                   d2h_bytes_per_step=int(sums_host.numel() * 8), ms_per_step=ms2 / k2,
                   host_wall_ms_per_step=wall / k2, overlap='h2d of step i+1 under compute of step i',
                   h2d_ms_per_step=[round(x, 2) for x in h2d_ms],
                   h2d_gbs_median=float(np.median([hbytes / (x / 1e3) / 1e9 for x in h2d_ms])),
                   device_ms_per_step=ms / a.steps)
        del host, bufs
        torch.cuda.empty_cache()

    del pp
    torch.cuda.empty_cache()
    secondary = {}
    if rank == 0 and not a.no_secondary:
        for name, fn in (('zeldovich', bench_zeldovich), ('bispectrum', bench_bispectrum),
                         ('batch', lambda: bench_batch(a.batch_size)), ('learned', bench_learned)):
            try:
                secondary[name] = fn()
            except Exception as exc:     # a failed side measurement must not hide the headline line
                secondary[name] = dict(error='%s: %s' % (type(exc).__name__, exc))
            torch.cuda.empty_cache()

    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
    hbm = peaks.get('hbm_gbs', 6800.0)
    roof = roofline(stages, n, dims, hbm, 'measured' if 'hbm_gbs' in peaks else 'fallback', ms / a.steps)

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = run_cpu_baseline(a.cpu_side)

    if rank == 0:
        line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=a.steps,
                    warmup=a.warmup, ms_per_step=ms / a.steps, higher_is_better=True,
                    scaling='weak', vs_baseline=None, dtype='f32', data='synthetic',
                    config=headline_config(side, dims, a.strategy),
                    e2e=e2e, roofline=roof, cpu_baseline=cpu, clocks=clk,
                    gpu_launches=kernels_per_step(dims) * a.steps, stages_ms=stages, grids_per_s=grids,
                    secondary=secondary)
        print(json.dumps(line))


def kernels_per_step(dims):
    """This library's kernel launches in one CIC-interlaced step (cuFFT's not counted):
    histogram, column scan, tile scan; placement (by bin in one pass up to 1024 bins,
    else the coherence-gated direct scatter + level A + level B); the deposit; on grids
    of 1024^3 and up (multiples of 32) the halo kernel, below that two fills; P(k)
    binning and the reduction of its per-CTA partial sums."""
    nt = -(-dims // 32)
    nc = -(-nt // 4)
    tiles = nc ** 3 * 64
    owned = dims % 32 == 0 and dims >= 1024
    placement = 1 if tiles <= 1024 else 3
    return 3 + placement + 1 + (1 if owned else 2) + 2


def chain_bytes(n, dims, grids):
    """Algorithmic HBM bytes of one particles -> P(k) chain: positions read once
    (12 B a particle), each grid written by the deposit (4 B a cell), transformed
    (4 B a cell read, 8 B a mode written) and binned (8 B a mode read)."""
    g, h = float(dims) ** 3, float(dims) * dims * (dims // 2 + 1)
    return 12.0 * n + grids * (4.0 * g + 4.0 * g + 8.0 * h + 8.0 * h)


def hbm_peak():
    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
    return peaks.get('hbm_gbs', 6800.0), ('measured' if 'hbm_gbs' in peaks else 'fallback')


def bench_zeldovich(reps=3):
    """512^3 lattice particles displaced by the Zel'dovich field of a 256^3 Gaussian
    field (P ~ k^-1.5 exp(-(k/0.5)^2), sigma 0.5, 1000 Mpc/h, seed 1) in redshift space
    along axis 2 (f = 0.5): TSC and PCS onto 512^3 with and without interlacing, P(k)
    l=0,2,4 + Pk2D along axis 2 (particles/s, device time per chain); then XPk of the
    TSC field against the NGP field; the interlaced TSC chain again through the
    deterministic sorted strategy."""
    import torch
    from pylians_gb300 import synthetic
    from pylians_gb300.pipeline import ParticlePk
    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.Pk_library as PKL
    pos = synthetic.zeldovich(N_field=256, N_lattice=512, BoxSize=BOX, sigma=0.5, f=0.5, rsd_axis=2, seed=1)
    n = pos.shape[0]
    hbm, src = hbm_peak()
    out = dict(workload="zeldovich 512^3 particles, 512^3 grid, RSD axis 2", particles=n,
               roofline=dict(peak=hbm, peak_source=src, unit='GB/s',
                             bytes='12 N_p + G (8 N_g + 16 N_h), G grids (chain_bytes)'))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for mas in ('TSC', 'PCS'):
        for inter in (False, True):
            pp = ParticlePk(512, BOX, mas, axis=2, interlaced=inter, max_particles=n)
            pp.step(pos)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                pp.step(pos)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            alg = chain_bytes(n, 512, 2 if inter else 1)
            out['%s%s' % (mas, '_interlaced' if inter else '')] = dict(
                ms=ms, particles_per_s=n / (ms / 1e3), alg_bytes=alg, gbs=alg / (ms / 1e3) / 1e9,
                frac=alg / (ms / 1e3) / 1e9 / hbm)
            del pp
            torch.cuda.empty_cache()
    # the deterministic sorted strategy on the same chain (TSC, interlaced)
    pp = ParticlePk(512, BOX, 'TSC', axis=2, interlaced=True, max_particles=n, strategy='sorted')
    pp.step(pos)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        pp.step(pos)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    alg = chain_bytes(n, 512, 2)
    out['TSC_interlaced_sorted'] = dict(ms=ms, particles_per_s=n / (ms / 1e3), alg_bytes=alg,
                                        gbs=alg / (ms / 1e3) / 1e9, frac=alg / (ms / 1e3) / 1e9 / hbm)
    del pp
    torch.cuda.empty_cache()
    a = torch.empty((512, 512, 512), device='cuda')
    b = torch.empty((512, 512, 512), device='cuda')
    MASL.overdensity_device(pos, a, BOX, 'TSC')
    MASL.overdensity_device(pos, b, BOX, 'NGP')
    PKL.XPk([a, b], BOX, 2, ['TSC', 'NGP'])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        PKL.XPk([a, b], BOX, 2, ['TSC', 'NGP'])
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / reps
    out['XPk_TSC_vs_NGP'] = dict(ms=t * 1e3, timing='host wall incl. sync and result copy')
    out['metric'] = 'particles/s'
    out['value'] = out['TSC_interlaced']['particles_per_s']
    del a, b, pos
    torch.cuda.empty_cache()
    return out


def bench_bispectrum(reps=5):
    """Bispectra of a 256^3 CIC overdensity (1000 Mpc/h, 256^3 uniform particles): k1=0.1,
    k2=0.2 h/Mpc with 32 theta bins, plus 20 equilateral triangles k=0.02..0.4 h/Mpc, all 52
    triangles through one BkPlan (one R2C, one shell fill, one batched C2R; the 32-theta
    group summed in Fourier space from the product of its two shared shells, the
    equilateral triangles reduced in real space; the indicator fields' sums are the
    plan's, made once).  Device time by CUDA events on the launching stream, per stage
    and for the whole chain; the call time adds the read-back and finalisation.

    Algorithmic bytes (N_g = N^3, N_h = N^2 (N/2+1) on the input grid; M_g, M_h the same on
    the reduced side M of the shell fields; R shells needed in real space, G Fourier groups):
      R2C 4 N_g + 8 N_h; deconvolution 16 N_h; shell fill R x 8 M_h (fields written); C2R
      R (8 M_h + 4 M_g); triangle sums: the real-space reduction reads each of its fields
      once (4 M_g each), and each Fourier group reads two fields and writes the product
      (12 M_g), transforms it (4 M_g + 8 M_h) and reads it back (8 M_h)."""
    import torch
    import pylians_gb300.MAS_library as MASL
    import pylians_gb300.Pk_library as PKL
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr, stream_ptr
    N = 256
    gen = torch.Generator(device='cuda')
    gen.manual_seed(3)
    pos = torch.rand((N ** 3, 3), generator=gen, device='cuda') * BOX
    d = torch.empty((N, N, N), device='cuda')
    MASL.overdensity_device(pos, d, BOX, 'CIC')
    del pos
    theta = np.linspace(0, np.pi, 32)
    k3 = np.sqrt((0.2 * np.sin(theta)) ** 2 + (0.2 * np.cos(theta) + 0.1) ** 2)
    tris = [(0.1, 0.2, float(x)) for x in k3] + [(float(k), float(k), float(k)) for k in np.linspace(0.02, 0.4, 20)]
    plan = PKL.BkPlan(N, BOX, tris, 'CIC')
    plan.run(d)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(reps):
        plan.run(d)
    ev[1].record()
    torch.cuda.synchronize()
    ms_eager = ev[0].elapsed_time(ev[1]) / reps
    # the chain as one CUDA graph (BkPlan.capture): launches without host gaps
    plan.capture(d)
    plan.replay()
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        plan.replay()
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / reps
    # stages: the steps of BkPlan.run with events between them
    st = stream_ptr()
    S = len(plan.bounds)
    se = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    acc = np.zeros(5)
    for _ in range(reps):
        se[0].record()
        _lib.call('pyl_fft_r2c', ptr(d), ptr(plan.dk), N, 1, st)
        se[1].record()
        _lib.call('pyl_mas_deconvolve', ptr(plan.dk), None, N, plan.mas_p, st)
        se[2].record()
        plan._powers(ptr(plan.dk), st)
        for c in plan._classes:
            plan._fill(c, ptr(plan.dk), st)
        se[3].record()
        for c in plan._classes:
            plan._c2r(c, st)
        se[4].record()
        for c in plan._classes:
            plan._sums(c, ptr(plan.dk), False, plan.num, st)
        se[5].record()
        torch.cuda.synchronize()
        acc += [se[k].elapsed_time(se[k + 1]) for k in range(5)]
    acc /= reps
    t0 = time.perf_counter()
    for _ in range(reps):
        plan.run(d)
        plan.result()
    t_call = (time.perf_counter() - t0) / reps * 1e3
    Ng, Nh = N ** 3, N * N * (N // 2 + 1)
    R, G = plan.R, plan.n_fourier_groups
    alg = dict(fft_r2c=4.0 * Ng + 8.0 * Nh, deconvolve=16.0 * Nh, shell_fill=0.0, fft_c2r=0.0, triangles=0.0)
    for c in plan._classes:            # per reduced side M: M_g cells, M_h stored modes
        Mg, Mh = float(c['cells']), float(c['half'])
        real_fields = len(set(int(x) for x in c['tri'][:3 * c['n_real']]))
        alg['shell_fill'] += c['R'] * 8.0 * Mh
        alg['fft_c2r'] += c['R'] * (8.0 * Mh + 4.0 * Mg)
        alg['triangles'] += real_fields * 4.0 * Mg + len(c['dots']) * (12.0 * Mg + 4.0 * Mg + 16.0 * Mh)
    names = ['fft_r2c', 'deconvolve', 'shell_fill', 'fft_c2r', 'triangles']
    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
    hbm = peaks.get('hbm_gbs', 6800.0)
    stages = {nm: dict(ms=float(acc[k]), gbs=alg[nm] / (acc[k] / 1e3) / 1e9,
                       frac=alg[nm] / (acc[k] / 1e3) / 1e9 / hbm) for k, nm in enumerate(names)}
    dom = max(names, key=lambda nm: stages[nm]['ms'])
    sides = [int(x) for x in plan.sides]
    del plan, d
    torch.cuda.empty_cache()
    return dict(metric='bispectra/s', value=len(tris) / (ms / 1e3), triangles=len(tris), shells=S,
                real_space_shells=R, fourier_groups=G, reduced_sides=sides,
                ms_per_call_device=ms, ms_per_call_device_eager=ms_eager,
                value_eager=len(tris) / (ms_eager / 1e3),
                ms_per_call_host=t_call, value_host=len(tris) / (t_call / 1e3), stages=stages,
                roofline=dict(kernel=dom, bound='hbm', achieved=stages[dom]['gbs'], peak=hbm, unit='GB/s',
                              frac=stages[dom]['frac']),
                workload='Bk 256^3 CIC, 32-theta sweep + 20 equilateral',
                timing='device: CUDA events around replays of the captured BkPlan.run (value) and around '
                       'eager BkPlan.run (value_eager); host: eager run + read-back + finalisation')


def bench_batch(count, steps=3):
    """Batched realizations: `count` uniform-particle sets with grids from {64,128,192,256}^3,
    1e5..1.7e7 particles (log-uniform), MAS from {CIC,TSC,PCS}, interlacing on/off (seed 0);
    one CUDA-graph replay per batch."""
    import torch
    from pylians_gb300 import batch
    specs = batch.random_specs(count, seed=0)
    gen = torch.Generator(device='cuda')
    gen.manual_seed(5)
    pos = [torch.rand((s['n'], 3), generator=gen, device='cuda') * BOX for s in specs]
    B = batch.RealizationBatch(specs, BOX, axis=0)
    B.capture(pos)
    B.replay()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        B.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    npart = sum(s['n'] for s in specs)
    alg = sum(chain_bytes(s['n'], s['dims'], 2 if s['interlaced'] else 1) for s in specs)
    hbm, src = hbm_peak()
    out = dict(metric='realizations/s', value=count / (ms / 1e3), particles_per_s=npart / (ms / 1e3),
               ms_per_batch=ms, realizations=count, particles=npart, ctas_per_sm=B.ctas_per_sm,
               roofline=dict(alg_bytes=alg, gbs=alg / (ms / 1e3) / 1e9, peak=hbm, peak_source=src,
                             frac=alg / (ms / 1e3) / 1e9 / hbm, unit='GB/s',
                             bytes='sum over realizations of 12 N_p + G (8 N_g + 16 N_h) (chain_bytes)'))
    del B, pos
    torch.cuda.empty_cache()
    return out


def bench_learned():
    """Learned-corrected 512^3 non-interlaced CIC P(k) against the plain interlaced 1024^3
    estimate of the same 1024^3 (expected) Poisson particles of a P ~ k^-1.5 field in a
    1000 Mpc/h box: wall-clock of both paths and the largest deviation up to 0.8 k_Nyq, and
    both against the interlaced 2048^3 estimate of the same particles."""
    from pylians_gb300 import learned
    r = learned.evaluate(N=512, side=1024, slope=-1.5, L=BOX, oracle_grid=2048)
    keep = ('particles', 'N_coarse', 'N_fine', 'k_max', 'bins', 'max_err_learned', 'mean_err_learned',
            'max_err_plain', 'mean_err_plain', 'ms_coarse_learned', 'ms_fine_interlaced', 'speedup',
            'device_ms_coarse_step', 'device_ms_fine_step', 'slope_est', 'shot_level_est', 'oracle_grid',
            'max_err_learned_vs_oracle', 'max_err_fine_vs_oracle')
    out = {k: r[k] for k in keep if k in r}
    out['metric'] = 'learned 512^3 vs interlaced 1024^3 P(k) wall-clock ratio'
    return out


STAGES = ('fill', 'hist', 'place', 'place_b', 'deposit', 'sort', 'halo')

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum, one pass of
# counters) of each kernel of the CIC-interlaced step measured by ncu, keyed by
# (particles, grid), from an ncu capture of the bench step (not measured live).
KERNEL_TRAFFIC = {
    (1024 ** 3, 1024): dict(hist=12.8850e9 + 0.0053e9, place=13.2252e9 + 17.3872e9,
                            place_b=17.3480e9 + 17.2813e9, deposit=29.0944e9 + 10.2683e9,
                            halo=4.2000e9 + 1.4836e9, pk_bin=8.6382e9 + 0.0223e9),
    (512 ** 3, 512): dict(deposit=4.017201e9 + 1.101149e9),
}


def stage_times(pp, pos, reps):
    """CUDA-event durations of each phase of one step on the launching stream: the
    library's own phase timing inside pyl_ma_overdensity (pyl_stage_timing), events
    around pyl_fft_r2c and pyl_pk_bin."""
    import ctypes
    import torch
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr, stream_ptr
    d = pp.dims
    n = pos.shape[0]
    st = stream_ptr()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    acc = np.zeros(3)
    buf = (ctypes.c_double * 8)()
    _lib.call('pyl_stage_times', buf, 8)
    _lib.call('pyl_stage_timing', 1)
    try:
        for _ in range(reps):
            ev[0].record()
            _lib.call('pyl_ma_overdensity', ptr(pos), None, n, ptr(pp.grids[0]), ptr(pp.grids[1]), d,
                      pp.BoxSize, _lib.MAS_INDEX[pp.MAS], _lib.STRATEGY[pp.strategy], ptr(pp.ws),
                      pp.ws_bytes, st)
            ev[1].record()
            _lib.call('pyl_fft_r2c', ptr(pp.grids), ptr(pp.dk), d, 2, st)
            ev[2].record()
            _lib.call('pyl_pk_bin', ptr(pp.dk[0]), ptr(pp.dk[1]), 1, pp.dk[0].numel(), d, pp.axis,
                      pp.mas_p, ptr(pp.sums), ptr(pp.pk_ws), pp.pk_ws_bytes, st)
            ev[3].record()
            torch.cuda.synchronize()
            acc += [ev[i].elapsed_time(ev[i + 1]) for i in range(3)]
        _lib.call('pyl_stage_times', buf, 8)
    finally:
        _lib.call('pyl_stage_timing', 0)
    acc /= reps
    out = dict(density=acc[0], fft_r2c=acc[1], pk_bin=acc[2])
    out['density_phases'] = {name: buf[i] / reps for i, name in enumerate(STAGES) if buf[i] > 0}
    return out


def grids_per_s(pp, reps):
    """P(k) of grids already resident in HBM (no deposit): R2C + the fused interlace /
    deconvolve / bin kernel, for the interlaced pair of the step and for one grid alone
    (pyl_pk_bin with one field), CUDA events on the launching stream."""
    import torch
    from pylians_gb300 import _lib
    from pylians_gb300._device import ptr, stream_ptr
    d, st = pp.dims, stream_ptr()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    out = {}
    for name, ng in (('interlaced_pair', 2), ('single_grid', 1)):
        def once():
            _lib.call('pyl_fft_r2c', ptr(pp.grids), ptr(pp.dk), d, ng, st)
            _lib.call('pyl_pk_bin', ptr(pp.dk[0]), ptr(pp.dk[1]) if ng == 2 else None, 1, pp.dk[0].numel(), d,
                      pp.axis, pp.mas_p, ptr(pp.sums), ptr(pp.pk_ws), pp.pk_ws_bytes, st)
        once()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            once()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = dict(value=1e3 / ms, unit='grids/s', ms=ms, grid=d)
    out['metric'] = 'P(k) of a resident %d^3 grid (R2C + fused bin), grids/s' % d
    return out


def roofline(stages, n, dims, hbm, src, ms_step):
    """Algorithmic HBM bytes per launch of each kernel or phase of the step:
      fill (two grids of -1): 2 x 4 B/cell written;
      hist: 12 B/particle read;  place (level A): 12 B read + 16 B written per particle;
      place_b: 16 B read + 16 B written per particle;
      deposit: 16 B/particle record read + 2 grids x 4 B/cell written;
      halo (owned-cell write-out): the halo blocks read once (4 B per halo cell
        of each bin) + the receiving cells read and written (8 B each);
      fft_r2c: 2 x (4 B/cell read + 8 B/mode written);  pk_bin: 2 fields x 8 B/mode read.
    The dominant single kernel is the one reported."""
    cells = dims ** 3
    modes = dims * dims * (dims // 2 + 1)
    bins = (dims // 32) ** 3
    halo_cells = 34 ** 3 - 32 ** 3          # CIC interlaced: 2 halo layers per bin side
    alg = dict(fill=2 * 4.0 * cells, hist=12.0 * n, place=28.0 * n, place_b=32.0 * n,
               deposit=16.0 * n + 2 * 4.0 * cells, fft_r2c=2 * (4.0 * cells + 8.0 * modes),
               pk_bin=2 * 8.0 * modes, halo=2 * bins * halo_cells * (4.0 + 8.0))
    ms = dict(stages['density_phases'])
    ms['fft_r2c'] = stages['fft_r2c']
    ms['pk_bin'] = stages['pk_bin']
    ms = {k: v for k, v in ms.items() if k in alg}
    top = max(ms, key=lambda k: ms[k])
    achieved = alg[top] / (ms[top] / 1e3) / 1e9
    measured = KERNEL_TRAFFIC.get((n, dims), {})
    # the whole step and the mass-assignment stage against the path's own algorithmic
    # bytes (positions read once, both grids written once, two R2C, the binning read):
    #   MA: 12 N_p + 2 x 4 N_g;  step: that + 2 (4 N_g + 8 N_h) + 2 x 8 N_h
    ma_bytes = 12.0 * n + 2 * 4.0 * cells
    step_bytes = ma_bytes + 2 * (4.0 * cells + 8.0 * modes) + 2 * 8.0 * modes
    step_gbs = step_bytes / (ms_step / 1e3) / 1e9
    ma_gbs = ma_bytes / (stages['density'] / 1e3) / 1e9
    return dict(bound='hbm', kernel=top, achieved=achieved, peak=hbm, unit='GB/s',
                frac=achieved / hbm, traffic=measured.get(top), peak_source=src,
                traffic_source='ncu capture of the bench step (dram__bytes_read.sum + dram__bytes_write.sum), '
                               'not measured in this run',
                alg_bytes=alg[top], ms=ms[top],
                step=dict(alg_bytes=step_bytes, ms=ms_step, achieved=step_gbs, frac=step_gbs / hbm),
                ma_stage=dict(alg_bytes=ma_bytes, ms=stages['density'], achieved=ma_gbs, frac=ma_gbs / hbm),
                all_kernels={k: dict(ms=ms[k], gbs=alg[k] / (ms[k] / 1e3) / 1e9,
                                     frac=alg[k] / (ms[k] / 1e3) / 1e9 / hbm, traffic=measured.get(k))
                             for k in ms})


if __name__ == '__main__':
    main()
