"""Recipe: compile the reference's own density-field / P(k) / B(k) code into ``oracle/_ref``.

Test infrastructure only.  The compiled reference is used in this container to
pin the oracle restatement (``oracle/oracle.py``, ``oracle/pyl_oracle.c``) and to
generate the golden fixtures under ``tests/golden``.  It is never shipped and no
product code imports it.

What is compiled (read from the reference tree, never copied into the repo):
  library/MAS_library/MAS_library.pyx + MAS_c.c   -> MAS_library*.so
  library/Pk_library/Pk_library.pyx               -> Pk_library*.so
  library/Pk_library/bispectrum_library.pyx       -> bispectrum_library*.so
  library/redshift_space_library.pyx              -> redshift_space_library*.so
  library/smoothing_library/smoothing_library.pyx -> smoothing_library*.so
with the reference's own compiler flags (library/setup.py:8-46):
  MAS: -O3 -ffast-math -march=native -fopenmp (+ -fopenmp at link, libm)
  Pk : -O3 -ffast-math -march=native -fopenmp
  Bk, redshift space: no extra flags
  smoothing: -O3 -ffast-math -march=native -fopenmp (+ -fopenmp at link, libm)

The sources are Python 2 Cython.  Three things are needed to run them on
Python 3 and they are applied to a temporary copy outside the repository
(the reference tree is read-only and nothing of it is committed):
  1. Cython ``language_level=2``;
  2. ``dims/2`` -> ``dims//2`` (and ``grid/2``, ``Nmesh/2``) in
     Pk_library.pyx, where ``def`` functions divide Python ints
     (Pk_library.pyx:60,68,125-236): Python 3 makes that a float;
  3. at import time ``time.clock = time.perf_counter`` (MAS_library.pyx:71)
     and the ``oracle/pyfftw_shim`` module for pyFFTW (see ``load_reference``).

Usage:  python oracle/build_ref.py [--reference /path/to/Pylians]
"""
import argparse
import os
import re
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
DEFAULT_REF = os.environ.get('PYLIANS_REFERENCE', '/root/reference')

_SOURCES = {
    'MAS_library': ['library/MAS_library/MAS_library.pyx', 'library/MAS_library/MAS_c.c',
                    'library/MAS_library/MAS_c.h', 'library/MAS_library/MAS_c.pxd'],
    'Pk_library': ['library/Pk_library/Pk_library.pyx'],
    'bispectrum_library': ['library/Pk_library/bispectrum_library.pyx'],
    'redshift_space_library': ['library/redshift_space_library.pyx'],
    'smoothing_library': ['library/smoothing_library/smoothing_library.pyx'],
}


def _patch_py3_division(text):
    return re.sub(r'\b(dims|grid|Nmesh)/2(?![.\d])', r'\1//2', text)


def built(out=OUT):
    if not os.path.isdir(out):
        return False
    names = os.listdir(out)
    return all(any(n.startswith(m + '.') and n.endswith('.so') for n in names)
               for m in _SOURCES)


def build(reference=DEFAULT_REF, out=OUT, quiet=True):
    """Compile the three reference extension modules into ``out``."""
    if not os.path.isdir(os.path.join(reference, 'library', 'MAS_library')):
        raise FileNotFoundError('reference sources not found at %s' % reference)
    from setuptools import Extension
    from setuptools.dist import Distribution
    from Cython.Build import cythonize
    import numpy

    os.makedirs(out, exist_ok=True)
    with tempfile.TemporaryDirectory(prefix='pyl_refbuild_') as tmp:
        for mod, files in _SOURCES.items():
            for f in files:
                src = os.path.join(reference, f)
                dst = os.path.join(tmp, os.path.basename(f))
                with open(src) as fh:
                    text = fh.read()
                if os.path.basename(f) == 'Pk_library.pyx':
                    text = _patch_py3_division(text)
                with open(dst, 'w') as fh:
                    fh.write(text)
        inc = [numpy.get_include(), tmp]
        native = ['-O3', '-ffast-math', '-march=native', '-fopenmp']
        exts = [
            Extension('MAS_library', [os.path.join(tmp, 'MAS_library.pyx'),
                                      os.path.join(tmp, 'MAS_c.c')],
                      include_dirs=inc, extra_compile_args=native,
                      extra_link_args=['-fopenmp'], libraries=['m']),
            Extension('Pk_library', [os.path.join(tmp, 'Pk_library.pyx')],
                      include_dirs=inc, extra_compile_args=native),
            Extension('bispectrum_library', [os.path.join(tmp, 'bispectrum_library.pyx')],
                      include_dirs=inc),
            Extension('redshift_space_library', [os.path.join(tmp, 'redshift_space_library.pyx')],
                      include_dirs=inc),
            Extension('smoothing_library', [os.path.join(tmp, 'smoothing_library.pyx')],
                      include_dirs=inc, extra_compile_args=native, extra_link_args=['-fopenmp'],
                      libraries=['m']),
        ]
        exts = cythonize(exts, compiler_directives={'language_level': 2},
                         include_path=[tmp], quiet=quiet, build_dir=os.path.join(tmp, 'c'))
        dist = Distribution({'name': 'pylians_ref', 'ext_modules': exts})
        cmd = dist.get_command_obj('build_ext')
        cmd.build_lib = out
        cmd.build_temp = os.path.join(tmp, 'obj')
        cmd.inplace = False
        cmd.ensure_finalized()
        cwd = os.getcwd()
        try:
            os.chdir(tmp)
            cmd.run()
        finally:
            os.chdir(cwd)
    return out


def load_reference(out=OUT):
    """Import the compiled reference modules (MAS_library, Pk_library, bispectrum_library)."""
    import time
    if not hasattr(time, 'clock'):
        time.clock = time.perf_counter
    for p in (os.path.join(HERE, 'pyfftw_shim'), out):
        if p not in sys.path:
            sys.path.insert(0, p)
    import MAS_library
    import Pk_library
    import bispectrum_library
    return MAS_library, Pk_library, bispectrum_library


def load_smoothing(out=OUT):
    """Import the compiled reference smoothing_library (it imports Pk_library itself)."""
    load_reference(out)
    import smoothing_library
    return smoothing_library


def load_redshift_space(out=OUT):
    """Import the compiled reference redshift_space_library."""
    load_reference(out)
    import redshift_space_library
    return redshift_space_library


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=DEFAULT_REF)
    ap.add_argument('--out', default=OUT)
    a = ap.parse_args()
    if os.path.isdir(a.out):
        shutil.rmtree(a.out)
    print(build(a.reference, a.out, quiet=False))
