"""Batched realizations: many particle sets -> many P(k) in one graph-capturable pass.

A batch holds realizations with uneven particle counts, grid sizes, MAS and
interlacing.  One step runs:
  * one fill of every grid with -1 per grid-size class (pyl_fill);
  * the deposit of all realizations at once, fed by a device work list whose
    item sizes the autotuner picks per (grid, particle count, MAS, interlacing)
    class: method 'tiled' (grids <= 512^3) bins every realization's particles
    into 32^3-cell bins and deposits all bins in ONE persistent launch
    (pyl_ma_batch_tiled); method 'atomic' is ONE persistent launch of
    red.global deposits (pyl_ma_batch);
  * one batched cuFFT R2C per grid-size class;
  * one launch of the fused P(k) bin kernel per (grid size, interlacing) class
    over all of its realizations (pyl_pk_bin_batch), or pyl_pk_bin per
    realization where a grid's bins do not fit that kernel's shared memory.
Everything is stream-ordered, so `capture()` turns a step into one CUDA graph
and `replay()` launches the whole batch at once.  Results equal the
one-at-a-time path (pipeline.ParticlePk) up to float summation order.
"""
import numpy as np
import torch

from . import _lib
from . import Pk_library as PKL
from . import autotune
from ._device import ptr, require_cuda, stream_ptr

REAL_DT = np.dtype([('pos', '<u8'), ('grid', '<u8'), ('grid2', '<u8'), ('inv', '<f4'),
                    ('halfcell', '<f4'), ('scale', '<f4'), ('dims', '<i4'), ('mas', '<i4'),
                    ('reserved', '<i4')])
ITEM_DT = np.dtype([('first', '<i8'), ('count', '<u4'), ('real', '<u4')])
PK_ITEM_DT = np.dtype([('dk', '<u8'), ('dk2', '<u8'), ('sums', '<u8'), ('mas_p', '<i4'), ('reserved', '<i4')])


class RealizationBatch(object):
    """specs: list of dicts with keys dims, MAS, interlaced, n (particle count)."""

    def __init__(self, specs, BoxSize, axis=0, device=None, tune=True, ctas_per_sm=None, order='size',
                 method='auto'):
        require_cuda()
        self.specs = [dict(s) for s in specs]
        self.BoxSize, self.axis = float(BoxSize), int(axis)
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        L = _lib.load()
        # grids grouped by size class so that one batched R2C covers each class
        self.classes = {}
        for i, s in enumerate(self.specs):
            if s['MAS'] not in _lib.MAS_INDEX:
                raise ValueError('MAS must be NGP, CIC, TSC or PCS')
            c = self.classes.setdefault(int(s['dims']), [])
            s['slot'] = len(c)
            c.append(i)
            if s.get('interlaced'):
                s['slot2'] = len(c)
                c.append(i)
        self.grids, self.dk = {}, {}
        for d, members in self.classes.items():
            self.grids[d] = torch.empty((len(members), d, d, d), dtype=torch.float32, device=self.device)
            self.dk[d] = torch.empty((len(members), d, d, d // 2 + 1), dtype=torch.complex64, device=self.device)
        self.sums = [torch.empty(L.pyl_pk_sums_len(int(s['dims']), 1), dtype=torch.float64, device=self.device)
                     for s in self.specs]
        self.mas_p = [PKL.ctypes_int_array([_lib.MAS_INDEX[s['MAS']]]) for s in self.specs]
        # binning: one pyl_pk_bin_batch launch per (grid size, interlacing) class, each
        # realization a device record (field, partner, sums, MAS); classes whose bins do
        # not fit the batched kernel go one realization at a time
        self.bin_classes, self.bin_single = [], []
        nbytes = 0
        for d in sorted(self.classes):
            for inter in (False, True):
                members = [i for i in sorted(set(self.classes[d]))
                           if bool(self.specs[i].get('interlaced')) == inter]
                if not members:
                    continue
                ws = L.pyl_pk_bin_batch_workspace_size(d, len(members), self.axis, int(inter))
                if ws == 0:
                    self.bin_single.extend(members)
                    continue
                rec = np.zeros(len(members), dtype=PK_ITEM_DT)
                for j, i in enumerate(members):
                    sp = self.specs[i]
                    rec[j]['dk'] = self.dk[d][sp['slot']].data_ptr()
                    rec[j]['dk2'] = self.dk[d][sp['slot2']].data_ptr() if inter else 0
                    rec[j]['sums'] = self.sums[i].data_ptr()
                    rec[j]['mas_p'] = _lib.MAS_INDEX[sp['MAS']]
                table = torch.from_numpy(rec.view(np.uint8)).to(self.device)
                self.bin_classes.append((d, inter, len(members), table))
                nbytes = max(nbytes, ws)
        for i in self.bin_single:
            nbytes = max(nbytes, L.pyl_pk_workspace_size(int(self.specs[i]['dims']), 1, self.axis))
        self.pk_ws_bytes = nbytes
        self.pk_ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
        self.counter = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.geom = {d: PKL.geometry(d, self.axis, self.device) for d in self.classes}

        if order not in ('size', 'realization'):
            raise ValueError("order must be 'size' or 'realization'")
        self.order = order
        if method not in ('auto', 'tiled', 'atomic'):
            raise ValueError("method must be 'auto', 'tiled' or 'atomic'")
        fits = all(int(s['dims']) <= 512 for s in self.specs)
        if method == 'tiled' and not fits:
            raise ValueError('the tiled batch needs grids of at most 512^3')
        self.method = 'tiled' if (method == 'auto' and fits) else ('atomic' if method == 'auto' else method)
        nts = [-(-int(s['dims']) // 32) for s in self.specs]
        tb = np.concatenate([[0], np.cumsum([t ** 3 for t in nts])]).astype(np.uint32)
        self.total_tiles = int(tb[-1])
        self.tile_base = torch.from_numpy(tb[:-1].copy().view(np.int32)).to(self.device)
        self.total_particles = int(sum(int(s['n']) for s in self.specs))
        self.bt_ws = None
        if self.method == 'tiled':
            nb = L.pyl_ma_batch_tiled_workspace_size(self.total_tiles, self.total_particles)
            self.bt_ws_bytes = nb
            self.bt_ws = torch.empty(max(nb, 1), dtype=torch.uint8, device=self.device)
        self.item_sizes = [autotune.item_size(int(s['dims']), int(s['n']), s['MAS'], bool(s.get('interlaced')),
                                              tune=tune, method=self.method) for s in self.specs]
        self.ctas_per_sm = ctas_per_sm or autotune.ctas_per_sm(tune=tune, method=self.method)
        self.reals_dev = None
        self.items_dev = None
        self.graph = None

    def _tables(self, positions):
        reals = np.zeros(len(self.specs), dtype=REAL_DT)
        items = []
        for i, (s, pos) in enumerate(zip(self.specs, positions)):
            d = int(s['dims'])
            n = pos.shape[0]
            if n != int(s['n']):
                raise ValueError('realization %d has %d particles, spec says %d' % (i, n, s['n']))
            if pos.dtype != torch.float32 or not pos.is_cuda or not pos.is_contiguous():
                raise ValueError('positions must be contiguous float32 CUDA tensors')
            g = self.grids[d]
            reals[i]['pos'] = pos.data_ptr()
            reals[i]['grid'] = g[s['slot']].data_ptr()
            reals[i]['grid2'] = g[s['slot2']].data_ptr() if s.get('interlaced') else 0
            reals[i]['inv'] = np.float32(d) / np.float32(self.BoxSize)
            reals[i]['halfcell'] = np.float32(0.5 * self.BoxSize / d)
            reals[i]['scale'] = np.float32(float(d) ** 3 / n)
            reals[i]['dims'] = d
            reals[i]['mas'] = _lib.MAS_INDEX[s['MAS']]
            step = self.item_sizes[i]
            for first in range(0, n, step):
                items.append((first, min(step, n - first), i))
        if self.order == 'size':
            # longest items first: the persistent CTAs balance the tail with the short ones
            items.sort(key=lambda t: -t[1])
        # 'realization': realization by realization, so the CTAs in flight share few grids
        it = np.array(items, dtype=ITEM_DT)
        self.reals_dev = torch.from_numpy(reals.view(np.uint8)).to(self.device)
        self.items_dev = torch.from_numpy(it.view(np.uint8)).to(self.device)
        self.n_items = len(items)

    def step(self, positions, stream=None):
        """Enqueue one batch pass on `positions` (list of [n_i, 3] float32 CUDA tensors)."""
        if self.reals_dev is None:
            self._tables(positions)
        st = stream_ptr(stream)
        for d, g in self.grids.items():
            _lib.call('pyl_fill', ptr(g), g.numel(), -1.0, st)
        if self.method == 'tiled':
            _lib.call('pyl_ma_batch_tiled', ptr(self.reals_dev), len(self.specs), ptr(self.items_dev), self.n_items,
                      ptr(self.tile_base), self.total_tiles, self.total_particles, ptr(self.bt_ws), self.bt_ws_bytes,
                      self.ctas_per_sm, st)
        else:
            _lib.call('pyl_ma_batch', ptr(self.reals_dev), len(self.specs), ptr(self.items_dev), self.n_items,
                      ptr(self.counter), self.ctas_per_sm, st)
        for d, g in self.grids.items():
            _lib.call('pyl_fft_r2c', ptr(g), ptr(self.dk[d]), d, g.shape[0], st)
        for d, inter, n, table in self.bin_classes:
            _lib.call('pyl_pk_bin_batch', ptr(table), n, d, self.axis, int(inter), ptr(self.pk_ws),
                      self.pk_ws_bytes, st)
        for i in self.bin_single:
            s = self.specs[i]
            d = int(s['dims'])
            dk = self.dk[d]
            dk2 = dk[s['slot2']] if s.get('interlaced') else None
            _lib.call('pyl_pk_bin', ptr(dk[s['slot']]), ptr(dk2), 1, dk[0].numel(), d, self.axis,
                      self.mas_p[i][0], ptr(self.sums[i]), ptr(self.pk_ws), self.pk_ws_bytes, st)

    def capture(self, positions):
        self._tables(positions)
        self.step(positions)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(positions)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def results(self):
        out = []
        for i, s in enumerate(self.specs):
            d = int(s['dims'])
            out.append(PKL.finalize_pk(self.sums[i].cpu().numpy(), self.geom[d], self.BoxSize, d, 1,
                                       cross=False))
        return out


def random_specs(count, seed=0, dims_choices=(64, 128, 192, 256), n_range=(100000, 17000000),
                 mas_choices=('CIC', 'TSC', 'PCS')):
    """Uneven realizations drawn from `seed`: grid side, particle count (log-uniform),
    MAS and interlacing per realization."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        specs.append(dict(dims=int(rng.choice(dims_choices)), MAS=str(rng.choice(mas_choices)),
                          interlaced=bool(rng.integers(0, 2)), n=n))
    return specs
