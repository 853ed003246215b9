"""C-ABI checks that need no GPU: the library loads, exports exactly what
include/pylians_gb300.h declares, and rejects bad arguments on the host."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, 'include', 'pylians_gb300.h')


@pytest.fixture(scope='module')
def lib():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import _lib
    return _lib.load()


def declared():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(pyl_\w+)\s*\(', text)))


def test_header_matches_bindings():
    from pylians_gb300 import _lib
    assert declared() == sorted(_lib.SIGNATURES)


def test_every_declared_symbol_is_exported(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_strerror_and_version(lib):
    assert lib.pyl_strerror(0) == b'success'
    assert lib.pyl_strerror(1) == b'invalid argument'
    assert lib.pyl_strerror(99) == b'unknown status'
    assert lib.pyl_version() >= 100


def test_sizes_are_host_side(lib):
    # 128^3: nb3 = 111, nb1 = 65, nb2 = 65*91
    assert lib.pyl_pk_sums_len(128, 1) == 111 * 4 + 65 + 65 * 91
    assert lib.pyl_pk_sums_len(128, 2) == 111 * (3 * 3 + 2) + 65 * 3 + 65 * 91 * 3
    assert lib.pyl_pk_geometry_len(128) == 2 * 65 + 65 * 91 + 2 * 111
    assert lib.pyl_ma_workspace_size(1000, 3, 64, 2, 1, 0) == 256        # atomic: the mass-sum tail only
    assert lib.pyl_ma_workspace_size(10 ** 6, 3, 512, 2, 2, 1) >= 12 * 10 ** 6


@pytest.mark.parametrize('kw,msg', [
    (dict(ndim=4), 'ndim'), (dict(mas=7), 'MAS'), (dict(dims=0), 'dims'),
    (dict(box=-1.0), 'BoxSize'), (dict(strategy=9), 'strategy'), (dict(n=-5), 'negative'),
])
def test_ma_rejects_bad_arguments(lib, kw, msg):
    a = dict(ndim=3, mas=2, dims=16, box=1.0, strategy=0, n=10)
    a.update(kw)
    buf = ctypes.c_void_p(16)   # never dereferenced: validation fails first
    rc = lib.pyl_ma(buf, None, a['n'], a['ndim'], buf, None, a['dims'], a['box'], a['mas'],
                    a['strategy'], 1, None, 0, None)
    assert rc == 1
    assert msg in lib.pyl_last_error().decode()


def test_pk_rejects_bad_arguments(lib):
    buf = ctypes.c_void_p(16)
    mp = (ctypes.c_int * 1)(2)
    assert lib.pyl_pk_bin(buf, None, 1, 0, 32, 3, mp, buf, None, 0, None) == 1
    assert 'axis' in lib.pyl_last_error().decode()
    mp5 = (ctypes.c_int * 5)(2, 2, 2, 2, 2)
    assert lib.pyl_pk_bin(buf, None, 5, 10 ** 6, 32, 0, mp5, buf, None, 0, None) == 5
    bad = (ctypes.c_int * 1)(7)
    assert lib.pyl_pk_bin(buf, None, 1, 0, 32, 0, bad, buf, None, 0, None) == 1


def test_pk_batch_sizes_and_arguments(lib):
    lib.pyl_pk_bin_batch_workspace_size.restype = ctypes.c_size_t
    size = lib.pyl_pk_bin_batch_workspace_size
    # per-item partial sums grow with the item count; axis 2 adds the row table
    one, two = size(64, 1, 0, 1), size(64, 2, 0, 1)
    assert 0 < one < two
    assert size(64, 2, 2, 0) > 0
    # 0: not batchable (bad sizes, or bins beyond the one-field kernel's shared memory)
    assert size(1, 4, 0, 0) == 0 and size(64, 0, 0, 0) == 0 and size(64, 4, 3, 0) == 0
    assert size(8192, 1, 0, 1) == 0
    buf = ctypes.c_void_p(16)
    assert lib.pyl_pk_bin_batch(None, 4, 64, 0, 0, buf, 1 << 30, None) == 1
    assert lib.pyl_pk_bin_batch(buf, 0, 64, 0, 0, buf, 1 << 30, None) == 1
    assert lib.pyl_pk_bin_batch(buf, 4, 64, 0, 0, buf, 16, None) == 4
    assert 'workspace' in lib.pyl_last_error().decode()
    assert lib.pyl_pk_bin_batch(buf, 4, 8192, 0, 1, buf, 1 << 30, None) == 5


def test_bk_rejects_bad_arguments(lib):
    buf = ctypes.c_void_p(16)
    lo = (ctypes.c_int64 * 1)(1)
    assert lib.pyl_bk_shell_fill(buf, 32, 32, lo, lo, None, 0, buf, buf, buf, None) == 1
    # a reduced side must exceed 3 K (here K = 9 for k^2 < 90): 27 is too small
    hi = (ctypes.c_int64 * 1)(90)
    assert lib.pyl_bk_shell_fill(buf, 64, 27, lo, hi, None, 1, buf, buf, buf, None) == 1
    assert 'out_dims' in lib.pyl_last_error().decode()
    assert lib.pyl_bk_shell_fill(buf, 64, 80, lo, hi, None, 1, buf, buf, buf, None) == 1
    tri = (ctypes.c_int * 3)(0, 0, 5)
    assert lib.pyl_bk_triangles(buf, buf, 16, 4096, 2, tri, 1, buf, buf, None) == 1
    # either field set may be omitted, not both; each set needs its sum buffer
    assert lib.pyl_bk_shell_fill(None, 64, 64, lo, hi, None, 1, None, None, buf, None) == 1
    assert 'no output' in lib.pyl_last_error().decode()
    assert lib.pyl_bk_shell_fill(buf, 64, 64, lo, hi, None, 1, None, None, buf, None) == 1
    assert 'out_delta is NULL' in lib.pyl_last_error().decode()
    assert lib.pyl_bk_shell_fill(None, 64, 64, lo, hi, None, 1, buf, None, buf, None) == 1
    assert 'need dk' in lib.pyl_last_error().decode()
    tri = (ctypes.c_int * 3)(0, 0, 1)
    assert lib.pyl_bk_triangles(None, None, 16, 4096, 2, tri, 1, buf, buf, None) == 1
    assert lib.pyl_bk_triangles(buf, None, 16, 4096, 2, tri, 1, None, buf, None) == 1
    assert 'sum buffer' in lib.pyl_last_error().decode()
    assert lib.pyl_bk_triangles(None, buf, 16, 4096, 2, tri, 1, buf, None, None) == 1
    # slots address output fields or -1 (power only); nothing past the shell count
    slot = (ctypes.c_int * 1)(1)
    assert lib.pyl_bk_shell_fill(buf, 64, 64, lo, hi, slot, 1, buf, None, buf, None) == 1
    assert 'slot' in lib.pyl_last_error().decode()
    # Fourier-space sums: buffers, bounds, output indices, the reduced side
    assert lib.pyl_bk_product(buf, buf, None, 10, None) == 1
    assert lib.pyl_bk_product(ctypes.c_void_p(20), buf, buf, 10, None) == 1
    assert 'aligned' in lib.pyl_last_error().decode()
    dst = (ctypes.c_int * 1)(0)
    assert lib.pyl_bk_shell_dots(buf, 64, buf, 64, lo, hi, dst, 0, buf, None) == 1
    assert lib.pyl_bk_shell_dots(buf, 64, buf, 27, lo, hi, dst, 1, buf, None) == 1
    assert 'out_dims' in lib.pyl_last_error().decode()
    neg = (ctypes.c_int * 1)(-1)
    assert lib.pyl_bk_shell_dots(buf, 64, buf, 64, lo, hi, neg, 1, buf, None) == 1


def test_python_facade_errors_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    import numpy as np
    import pylians_gb300.MAS_library as MASL
    from pylians_gb300._lib import PylError
    with pytest.raises(PylError):
        MASL.MA(np.zeros((4, 3), np.float32), np.zeros((8, 8, 8), np.float32), 1.0, 'CIC')


def test_overdensity_rejects_bad_arguments(lib):
    buf = ctypes.c_void_p(16)   # never dereferenced: validation fails first
    nan = float('nan')
    assert lib.pyl_ma_overdensity(buf, None, 0, buf, None, 16, 1.0, 2, 0, None, 0, None) == 1
    assert 'at least one particle' in lib.pyl_last_error().decode()
    assert lib.pyl_ma_overdensity(buf, None, 10, buf, None, 16, nan, 2, 0, None, 0, None) == 1
    assert 'BoxSize' in lib.pyl_last_error().decode()
    assert lib.pyl_ma_overdensity(buf, None, 10, buf, None, 16, 1.0, 5, 0, None, 0, None) == 1
    assert 'MAS' in lib.pyl_last_error().decode()
    # the redshift-space variant: line of sight, Hubble rate, velocities
    rsd = lib.pyl_ma_overdensity_rsd
    assert rsd(buf, buf, None, 10, buf, None, 16, 1.0, 2, 0, 100.0, 0.0, 3, None, 0, None) == 1
    assert 'axis' in lib.pyl_last_error().decode()
    assert rsd(buf, buf, None, 10, buf, None, 16, 1.0, 2, 0, 0.0, 0.0, 0, None, 0, None) == 1
    assert 'Hubble' in lib.pyl_last_error().decode()
    assert rsd(buf, None, None, 10, buf, None, 16, 1.0, 2, 0, 100.0, 0.0, 0, None, 0, None) == 1
    assert 'null' in lib.pyl_last_error().decode()


def test_noalloc_limits_are_checked_on_the_host(lib):
    buf = ctypes.c_void_p(16)
    assert lib.pyl_ma_noalloc(buf, None, 524289, buf, None, 64, 1.0, 2, None) == 1
    assert 'at most 524288 particles' in lib.pyl_last_error().decode()
    assert lib.pyl_ma_noalloc(buf, None, 1000, buf, None, 513, 1.0, 2, None) == 1
    assert 'dims <= 512' in lib.pyl_last_error().decode()
    assert lib.pyl_ma_noalloc(buf, None, 1000, buf, None, 64, 1.0, 0, None) == 1
    assert 'MAS' in lib.pyl_last_error().decode()


def test_interp_and_shift_reject_bad_arguments(lib):
    buf = ctypes.c_void_p(16)
    assert lib.pyl_cic_interp(buf, 16, -1.0, buf, 10, buf, None) == 1
    assert 'BoxSize' in lib.pyl_last_error().decode()
    assert lib.pyl_cic_interp(buf, 16, 1.0, None, 10, buf, None) == 1
    assert 'null' in lib.pyl_last_error().decode()
    assert lib.pyl_pos_redshift_space(buf, buf, 10, 1.0, 100.0, 0.0, 5, None) == 1
    assert 'axis' in lib.pyl_last_error().decode()
    assert lib.pyl_pos_redshift_space(buf, buf, -1, 1.0, 100.0, 0.0, 0, None) == 1
    assert 'negative' in lib.pyl_last_error().decode()


def test_f64_grid_rejects_bad_arguments(lib):
    buf = ctypes.c_void_p(16)
    f64 = lib.pyl_ma_f64
    assert f64(buf, buf, 10, 3, buf, 16, 8, 1.0, 2, None) == 1
    assert 'depth' in lib.pyl_last_error().decode()
    assert f64(buf, buf, 10, 4, buf, 16, 16, 1.0, 2, None) == 1
    assert 'ndim' in lib.pyl_last_error().decode()
    assert f64(buf, buf, 10, 3, None, 16, 16, 1.0, 2, None) == 1
    assert 'grid' in lib.pyl_last_error().decode()
    assert f64(buf, buf, 10, 3, buf, 16, 16, 0.0, 2, None) == 1
    assert 'BoxSize' in lib.pyl_last_error().decode()
    assert f64(buf, buf, 10, 3, buf, 16, 16, 1.0, 9, None) == 1
    assert 'MAS' in lib.pyl_last_error().decode()
    assert f64(buf, buf, 0, 3, buf, 16, 16, 1.0, 2, None) == 0     # nothing to deposit, nothing launched


def test_wait_probe_and_thresholds_reject_bad_arguments(lib):
    buf = ctypes.c_void_p(16)
    assert lib.pyl_wait_probe(16, 0, buf, None) == 1
    assert 'cycles' in lib.pyl_last_error().decode()
    assert lib.pyl_wait_probe(16, 10 ** 9, buf, None) == 1
    assert lib.pyl_wait_probe(12, 1000, buf, None) == 1
    assert 'arm_bytes' in lib.pyl_last_error().decode()
    assert lib.pyl_wait_probe(16, 1000, None, None) == 1
    assert lib.pyl_ma_set_thresholds(0, 1.0) == 1
    assert lib.pyl_ma_set_thresholds(-1, float('nan')) == 1
    assert lib.pyl_ma_set_thresholds(-1, -1.0) == 0
    assert lib.pyl_sorted_set_stage_limit(1025) == 1
    assert 'capacity' in lib.pyl_last_error().decode()
    assert lib.pyl_sorted_set_stage_limit(0) == 0
    assert lib.pyl_sorted_set_stage_limit(-1) == 0


def test_pass_limit_sizes_the_workspace(lib):
    size = lib.pyl_ma_workspace_size
    size.restype = ctypes.c_size_t
    size.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.pyl_ma_set_pass_limit.argtypes = [ctypes.c_int64]
    # a call of 2048^3 particles needs one pass's workspace, not the whole call's
    big = size(2048 ** 3, 3, 2048, 2, 2, 1)
    assert big == size((1 << 32) - 4096, 3, 2048, 2, 2, 1)
    assert big < 16 * 2048 ** 3
    try:
        assert lib.pyl_ma_set_pass_limit(0) == 1
        assert lib.pyl_ma_set_pass_limit(1000) == 1            # below one 1024-particle block
        assert lib.pyl_ma_set_pass_limit(5000) == 0            # rounded down to 4096
        assert size(10 ** 6, 3, 64, 2, 2, 0) == size(4096, 3, 64, 2, 2, 0)
    finally:
        assert lib.pyl_ma_set_pass_limit(-1) == 0
    assert size(10 ** 6, 3, 64, 2, 2, 0) > size(4096, 3, 64, 2, 2, 0)



def test_check_device_reads_clears_and_raises(monkeypatch):
    """pylians_gb300._lib.check_device reads the device error word with reset = 1
    and raises PylError when it was set; a failing read raises too (no GPU: a fake
    library stands in for pyl_device_error)."""
    from pylians_gb300 import _lib

    class Fake:
        def __init__(self, word, rc=0):
            self.word, self.rc, self.calls = word, rc, []

        def pyl_device_error(self, reset, out):
            self.calls.append(reset)
            ctypes.cast(out, ctypes.POINTER(ctypes.c_uint))[0] = self.word
            return self.rc

        def pyl_strerror(self, rc):
            return b'CUDA error'

        def pyl_last_error(self):
            return b'no device'

    fake = Fake(0)
    monkeypatch.setattr(_lib, 'load', lambda: fake)
    _lib.check_device('MA')
    assert fake.calls == [1]
    fake.word = 1
    with pytest.raises(_lib.PylError, match='MA: a device-side wait gave up'):
        _lib.check_device('MA')
    fake.word, fake.rc = 0, _lib.PYL_ERR_CUDA
    with pytest.raises(_lib.PylError, match='pyl_device_error'):
        _lib.check_device('MA')
