"""Stand-in for the two pyFFTW entry points the reference's P(k) code calls.

Test infrastructure only: this module is put on ``sys.path`` ahead of
everything else when the compiled reference (``oracle/_ref``) is imported to
generate golden vectors.  pyFFTW/FFTW3 are not installed in this image, and the
reference pins no version of either (Pylians README lists "pyfftw" unpinned).

The reference uses exactly two things (Pk_library.pyx:120-245):
  * ``pyfftw.empty_aligned(shape, dtype)``
  * ``pyfftw.FFTW(a_in, a_out, axes, flags, direction, threads)`` called as
    ``plan(a_in, a_out)``, i.e. through ``FFTW.__call__``, whose
    ``normalise_idft`` defaults to True: FFTW_FORWARD is an unnormalised R2C,
    FFTW_BACKWARD a C2R divided by the number of grid points.  The reference
    relies on that: ``Xi`` scales the inverse transform of |delta_k|^2 by
    1/dims^3 only (Pk_library.pyx:2088,2144-2146), and ``correct_MAS`` returns
    the corrected field at the input's scale (Pk_library.pyx:1801).

Both are served by ``scipy.fft`` in the input's own precision (float32 stays
float32, as FFTW's single-precision plans do) with ``workers=threads``.
"""
import numpy as np
import scipy.fft as _sfft


def empty_aligned(shape, dtype='float32', n=None):
    return np.empty(shape, dtype=dtype)


class FFTW(object):
    def __init__(self, a_in, a_out, axes=(0, 1, 2), flags=None,
                 direction='FFTW_FORWARD', threads=1, **kw):
        self.direction = direction
        self.axes = tuple(axes)
        self.threads = max(1, int(threads))

    def __call__(self, a_in=None, a_out=None):
        if self.direction == 'FFTW_FORWARD':
            a_out[...] = _sfft.rfftn(a_in, axes=self.axes, workers=self.threads)
        else:
            shape = tuple(a_out.shape[i] for i in self.axes)
            a_out[...] = _sfft.irfftn(a_in, s=shape, axes=self.axes,
                                      norm='backward', workers=self.threads)
        return a_out
