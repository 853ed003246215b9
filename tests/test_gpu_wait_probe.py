"""The staged kernels' bounded mbarrier wait, made to run out on purpose.

pyl_wait_probe arms a shared-memory mbarrier for 16 bytes of bulk-copy data and
issues no copy, so the phase never completes: the bounded wait must give up
after the given number of cycles, set the device error word and let the kernel
return, leaving the context usable.  No copy is ever in flight, nothing faults
and nothing hangs (the limit here is 1e5 cycles, about 50 microseconds).
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def lib():
    import pylians_gb300.build as b
    b.build()
    from pylians_gb300 import _lib
    return _lib.load()


def _error_word(lib, reset):
    u = ctypes.c_uint(0xFFFFFFFF)
    assert lib.pyl_device_error(int(reset), ctypes.byref(u)) == 0
    return u.value


def test_wait_runs_out_sets_error_word(lib):
    out = torch.full((1,), 7, dtype=torch.int32, device='cuda')
    _error_word(lib, True)
    try:
        assert lib.pyl_wait_probe(16, 100000, ctypes.c_void_p(out.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert out.item() == 0                  # the wait gave up
        assert _error_word(lib, True) == 1      # and reported it
        assert _error_word(lib, False) == 0     # reset clears the word
        # the context is intact: a phase that completes, and a deposit afterwards
        assert lib.pyl_wait_probe(0, 100000, ctypes.c_void_p(out.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert out.item() == 1
        assert _error_word(lib, False) == 0
        import pylians_gb300.MAS_library as MASL
        pos = torch.rand((2_000_000, 3), device='cuda') * 100.0
        g = torch.zeros((64, 64, 64), device='cuda')
        MASL.MA(pos, g, 100.0, 'NGP', strategy='tiled')
        assert g.sum().item() == 2_000_000
        assert _error_word(lib, False) == 0
    finally:
        _error_word(lib, True)


def test_error_word_stops_tiled_deposits_and_raises(lib):
    """While the error word is set the tiled deposit leaves the grid as it was (its
    placement's input may be incomplete), and MA with host results raises, reading
    and clearing the word; the next call deposits normally."""
    import numpy as np
    import pylians_gb300.MAS_library as MASL
    from pylians_gb300._lib import PylError
    out = torch.full((1,), 7, dtype=torch.int32, device='cuda')
    _error_word(lib, True)
    try:
        assert lib.pyl_wait_probe(16, 100000, ctypes.c_void_p(out.data_ptr()), None) == 0
        torch.cuda.synchronize()
        pos = (np.random.default_rng(3).random((2_000_000, 3)) * 100.0).astype(np.float32)
        g = np.zeros((64, 64, 64), np.float32)
        with pytest.raises(PylError, match='wait gave up'):
            MASL.MA(pos, g, 100.0, 'NGP', strategy='tiled')
        assert g.sum() == 0.0
        assert _error_word(lib, False) == 0
        MASL.MA(pos, g, 100.0, 'NGP', strategy='tiled')
        assert g.sum() == 2_000_000
    finally:
        _error_word(lib, True)
