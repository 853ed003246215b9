"""The benchmark's JSON contract and its roofline arithmetic, no GPU: the reference
arm (the oracle port on the host cores) prints one line with the keys the GPU arm
prints, its own cpu_baseline and a zero-copy e2e; the roofline block divides the
documented algorithmic bytes by the phase times; the chain byte formula of the
secondary workloads."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--grid', '32',
                        '--particles-side', '32', '--steps', '2', '--warmup', '1'],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better',
              'scaling', 'vs_baseline', 'dtype', 'data', 'config'):
        assert k in d, k
    assert d['impl'] == 'reference' and d['steps'] == 2 and d['warmup'] == 1 and d['value'] > 0
    assert d['higher_is_better'] is True and d['vs_baseline'] is None
    assert d['config']['workload'] == 'cic_interlaced_pk_np32^3_grid32^3'
    cb = d['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['value'] == d['value'] and cb['sample']
    assert d['e2e'] == dict(value=d['value'], unit=d['unit'], h2d_bytes_per_step=0, d2h_bytes_per_step=0)


def test_roofline_arithmetic():
    n, dims = 1024 ** 3, 1024
    stages = dict(density=31.0, fft_r2c=10.8, pk_bin=2.16,
                  density_phases=dict(hist=3.0, place=7.6, place_b=6.6, deposit=12.4, halo=1.44))
    r = bench.roofline(stages, n, dims, 6677.5, 'measured', 43.96)
    assert r['kernel'] == 'deposit'                       # the longest phase
    cells, modes = dims ** 3, dims * dims * (dims // 2 + 1)
    assert r['alg_bytes'] == 16.0 * n + 2 * 4.0 * cells
    assert r['achieved'] == pytest.approx(r['alg_bytes'] / 12.4e-3 / 1e9)
    assert r['frac'] == pytest.approx(r['achieved'] / 6677.5)
    assert r['traffic'] == bench.KERNEL_TRAFFIC[(n, dims)]['deposit']
    step = 12.0 * n + 2 * 4.0 * cells + 2 * (4.0 * cells + 8.0 * modes) + 2 * 8.0 * modes
    assert r['step']['alg_bytes'] == step and step == pytest.approx(47.2e9, rel=2e-3)
    assert r['ma_stage']['alg_bytes'] == pytest.approx(21.5e9, rel=2e-3)
    assert set(r['all_kernels']) == {'hist', 'place', 'place_b', 'deposit', 'halo', 'fft_r2c', 'pk_bin'}


def test_chain_bytes_and_launch_count():
    assert bench.chain_bytes(10, 4, 1) == 12.0 * 10 + 8.0 * 64 + 16.0 * 4 * 4 * 3
    assert bench.chain_bytes(10, 4, 2) - bench.chain_bytes(10, 4, 1) == 8.0 * 64 + 16.0 * 4 * 4 * 3
    # 1024^3: histogram + two scans, gated scatter + level A + level B, deposit, halo,
    # binning + reduction; 256^3 (64 bins): one placement pass and two fills
    assert bench.kernels_per_step(1024) == 10
    assert bench.kernels_per_step(256) == 9
