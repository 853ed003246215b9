"""Autotuner for the batched deposit: work-item size per realization class and
CTAs per SM of the persistent launches, for either batch method ('tiled':
bins + one persistent bin deposit; 'atomic': red.global work queue).

Classes are (grid side, particle-count bucket (power of 2), MAS, interlaced).
For a class the tuner deposits one synthetic realization of that class through
pyl_ma_batch with each candidate item size, times it with CUDA events (median
of 3 after a warm-up) and keeps the fastest.  Results persist in a JSON cache
(PYL_AUTOTUNE_CACHE, default ~/.cache/pylians_gb300/autotune.json) keyed by
the device name, so each class is measured once per machine.
"""
import json
import math
import os
import threading

import numpy as np
import torch

from . import _lib
from ._device import ptr, stream_ptr

ITEM_CANDIDATES = (1 << 12, 1 << 14, 1 << 16, 1 << 18)
CTA_CANDIDATES = (2, 4, 8)
DEFAULT_ITEM = 1 << 16
DEFAULT_CTAS = 4

_lock = threading.Lock()
_cache = None


def _path():
    return os.environ.get('PYL_AUTOTUNE_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache', 'pylians_gb300', 'autotune.json'))


def _load():
    global _cache
    if _cache is None:
        try:
            with open(_path()) as fh:
                _cache = json.load(fh)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    try:
        os.makedirs(os.path.dirname(_path()), exist_ok=True)
        tmp = _path() + '.tmp'
        with open(tmp, 'w') as fh:
            json.dump(_cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, _path())
    except OSError:
        pass


def _device_key():
    return torch.cuda.get_device_name(torch.cuda.current_device()).replace(' ', '_')


def class_key(dims, n, MAS, interlaced, method='atomic'):
    bucket = 1 << max(10, int(math.ceil(math.log2(max(n, 1)))))
    return '%s/%s/%d/%d/%s/%d' % (_device_key(), method, dims, bucket, MAS, int(interlaced))


def _time_deposit(dims, n, MAS, interlaced, item, ctas, reps=3, method='atomic'):
    from .batch import ITEM_DT, REAL_DT
    dev = torch.device('cuda', torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(12345)
    pos = torch.rand((n, 3), generator=gen, device=dev) * 1000.0
    g = torch.empty((2 if interlaced else 1, dims, dims, dims), device=dev)
    real = np.zeros(1, dtype=REAL_DT)
    real[0]['pos'] = pos.data_ptr()
    real[0]['grid'] = g[0].data_ptr()
    real[0]['grid2'] = g[1].data_ptr() if interlaced else 0
    real[0]['inv'] = np.float32(dims) / np.float32(1000.0)
    real[0]['halfcell'] = np.float32(500.0 / dims)
    real[0]['scale'] = np.float32(1.0)
    real[0]['dims'] = dims
    real[0]['mas'] = _lib.MAS_INDEX[MAS]
    items = np.array([(f, min(item, n - f), 0) for f in range(0, n, item)], dtype=ITEM_DT)
    rd = torch.from_numpy(real.view(np.uint8)).to(dev)
    idv = torch.from_numpy(items.view(np.uint8)).to(dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    st = stream_ptr()
    tiles = (-(-dims // 32)) ** 3
    tb = torch.zeros(1, dtype=torch.int32, device=dev)
    L = _lib.load()
    ws_bytes = L.pyl_ma_batch_tiled_workspace_size(tiles, n) if method == 'tiled' else 1
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev) if method == 'tiled' else None
    times = []
    for r in range(reps + 1):
        g.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        if method == 'tiled':
            _lib.call('pyl_ma_batch_tiled', ptr(rd), 1, ptr(idv), len(items), ptr(tb), tiles, n, ptr(ws), ws_bytes,
                      ctas, st)
        else:
            _lib.call('pyl_ma_batch', ptr(rd), 1, ptr(idv), len(items), ptr(cnt), ctas, st)
        e1.record()
        torch.cuda.synchronize()
        if r:
            times.append(e0.elapsed_time(e1))
    return float(np.median(times))


def item_size(dims, n, MAS, interlaced, tune=True, method='atomic'):
    key = class_key(dims, n, MAS, interlaced, method)
    with _lock:
        c = _load()
        if key in c:
            return int(c[key])
        if not tune:
            return DEFAULT_ITEM
        n_probe = min(max(n, 1 << 12), 1 << 22)
        best = min(ITEM_CANDIDATES, key=lambda it: _time_deposit(dims, n_probe, MAS, interlaced, it, DEFAULT_CTAS,
                                                                 method=method))
        c[key] = int(best)
        _save()
        return int(best)


def ctas_per_sm(tune=True, method='atomic'):
    key = '%s/%s/ctas_per_sm' % (_device_key(), method)
    with _lock:
        c = _load()
        if key in c:
            return int(c[key])
        if not tune:
            return DEFAULT_CTAS
        cands = CTA_CANDIDATES if method == 'atomic' else (1, 2)     # tiled kernels run 1024 threads per CTA
        best = min(cands, key=lambda k: _time_deposit(128, 1 << 22, 'CIC', True, DEFAULT_ITEM, k, method=method))
        c[key] = int(best)
        _save()
        return int(best)
