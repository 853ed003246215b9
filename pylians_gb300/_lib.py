"""ctypes binding of libpylgpu.so (declared in include/pylians_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every compute entry point raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libpylgpu.so')

PYL_OK, PYL_ERR_INVALID, PYL_ERR_CUDA, PYL_ERR_CUFFT, PYL_ERR_WORKSPACE, PYL_ERR_UNSUPPORTED = range(6)
MAS_INDEX = {'NGP': 1, 'CIC': 2, 'TSC': 3, 'PCS': 4}
STRATEGY = {'auto': 0, 'atomic': 1, 'tiled': 2, 'sorted': 3}

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_F = ctypes.c_float
_D = ctypes.c_double
_SZ = ctypes.c_size_t

# name -> (restype, argtypes); the exact list of exported C-ABI symbols
SIGNATURES = {
    'pyl_strerror': (ctypes.c_char_p, [_I]),
    'pyl_last_error': (ctypes.c_char_p, []),
    'pyl_version': (_I, []),
    'pyl_ma_workspace_size': (_SZ, [_I64, _I, _I, _I, _I, _I]),
    'pyl_ma': (_I, [_P, _P, _I64, _I, _P, _P, _I, _F, _I, _I, _I, _P, _SZ, _P]),
    'pyl_ma_noalloc': (_I, [_P, _P, _I64, _P, _P, _I, _F, _I, _P]),
    'pyl_ma_f64': (_I, [_P, _P, _I64, _I, _P, _I, _I, _F, _I, _P]),
    'pyl_ma_overdensity': (_I, [_P, _P, _I64, _P, _P, _I, _F, _I, _I, _P, _SZ, _P]),
    'pyl_ma_overdensity_rsd': (_I, [_P, _P, _P, _I64, _P, _P, _I, _F, _I, _I, _F, _F, _I, _P, _SZ, _P]),
    'pyl_ma_batch': (_I, [_P, _I, _P, _I, _P, _I, _P]),
    'pyl_fill': (_I, [_P, _I64, _F, _P]),
    'pyl_scale': (_I, [_P, _I64, _F, _P]),
    'pyl_ma_batch_tiled_workspace_size': (_SZ, [ctypes.c_uint32, _I64]),
    'pyl_ma_batch_tiled': (_I, [_P, _I, _P, _I, _P, ctypes.c_uint32, _I64, _P, _SZ, _I, _P]),
    'pyl_grid_sum': (_I, [_P, _I64, _P, _P]),
    'pyl_overdensity': (_I, [_P, _I64, _P, _D, _P]),
    'pyl_fft_r2c': (_I, [_P, _P, _I, _I, _P]),
    'pyl_fft_c2r': (_I, [_P, _P, _I, _I, _P]),
    'pyl_fft_cache_clear': (_I, []),
    'pyl_pk_sums_len': (_I64, [_I, _I]),
    'pyl_pk_geometry_len': (_I64, [_I]),
    'pyl_pk_workspace_size': (_SZ, [_I, _I, _I]),
    'pyl_pk_bin': (_I, [_P, _P, _I, _I64, _I, _I, _P, _P, _P, _SZ, _P]),
    'pyl_pk_geometry': (_I, [_I, _I, _P, _P, _SZ, _P]),
    'pyl_pk_bin_batch_workspace_size': (_SZ, [_I, _I, _I, _I]),
    'pyl_pk_bin_batch': (_I, [_P, _I, _I, _I, _I, _P, _SZ, _P]),
    'pyl_mas_deconvolve': (_I, [_P, _P, _I, _I, _P]),
    'pyl_bk_shell_fill': (_I, [_P, _I, _I, _P, _P, _P, _I, _P, _P, _P, _P]),
    'pyl_bk_product': (_I, [_P, _P, _P, _I64, _P]),
    'pyl_bk_shell_dots': (_I, [_P, _I, _P, _I, _P, _P, _P, _I, _P, _P]),
    'pyl_bk_triangles': (_I, [_P, _P, _I, _I64, _I, _P, _I, _P, _P, _P]),
    'pyl_mlp_param_count': (_I, []),
    'pyl_mlp_forward': (_I, [_P, _P, _I, _P, _P, _P]),
    'pyl_mlp_backward': (_I, [_P, _P, _P, _P, _P, _P, _F, _I, _P, _P, _P, _P]),
    'pyl_mlp_adam': (_I, [_P, _P, _P, _P, _P, _I, _F, _F, _F, _F, _I, _P]),
    'pyl_fft2_r2c': (_I, [_P, _P, _I, _I, _P]),
    'pyl_pk_plane_bins': (_I, [_I]),
    'pyl_pk_plane_bin': (_I, [_P, _P, _I, _I, _I, _P, _P]),
    'pyl_filter_grid': (_I, [_P, _I, _F, _F, _I, _P, _P]),
    'pyl_cmul': (_I, [_P, _P, _I64, _P]),
    'pyl_correct_mas': (_I, [_P, _I, _I, _P]),
    'pyl_xi_sums_len': (_I64, [_I]),
    'pyl_xi_power': (_I, [_P, _I, _I, _P]),
    'pyl_xi_bin': (_I, [_P, _I, _I, _P, _P]),
    'pyl_stage_timing': (_I, [_I]),
    'pyl_stage_times': (_I, [_P, _I]),
    'pyl_device_error': (_I, [_I, _P]),
    'pyl_ma_set_thresholds': (_I, [_I, _D]),
    'pyl_ma_set_pass_limit': (_I, [_I64]),
    'pyl_sorted_set_stage_limit': (_I, [_I]),
    'pyl_wait_probe': (_I, [ctypes.c_uint, ctypes.c_longlong, _P, _P]),
    'pyl_cic_interp': (_I, [_P, _I, _F, _P, _I64, _P, _P]),
    'pyl_pos_redshift_space': (_I, [_P, _P, _I64, _F, _F, _F, _I, _P]),
}

_lib = None
_lock = threading.Lock()


class PylError(RuntimeError):
    pass


def load():
    """Load (never build) libpylgpu.so and declare every signature."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise PylError('libpylgpu.so is not built (%s); run pylians_gb300.build.build() '
                               'or __graft_entry__.build()' % LIB_PATH)
            lib = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(rc, what=''):
    if rc == PYL_OK:
        return
    lib = load()
    msg = '%s: %s (%s)' % (what, lib.pyl_strerror(rc).decode(), lib.pyl_last_error().decode())
    if rc == PYL_ERR_INVALID:
        raise ValueError(msg)
    raise PylError(msg)


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc


def check_device(what=''):
    """Raise if a device-side bounded wait gave up since the last check (the device
    error word, read and cleared; the read waits for the device).  The tiled
    deposits launched while the word was set deposited nothing."""
    out = ctypes.c_uint(0)
    check(load().pyl_device_error(1, ctypes.byref(out)), 'pyl_device_error')
    if out.value:
        raise PylError('%s: a device-side wait gave up (error word %#x); the results of the calls '
                       'since the last check are incomplete' % (what, out.value))
