"""Build libpylgpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

The sources in csrc/ are compiled in parallel (one nvcc per translation unit,
one -gencode) and linked against cuFFT.  The result lands beside this file as
pylians_gb300/libpylgpu.so; it is rebuilt when any source or header is newer.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libpylgpu.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
SOURCES = ['capi.cu', 'mas.cu', 'tiled_ngp.cu', 'tiled_cic.cu', 'tiled_tsc.cu', 'tiled_pcs.cu', 'pk.cu', 'pkbin.cu', 'fft.cu', 'bk.cu', 'batch.cu', 'mlp.cu', 'sorted.cu', 'interp.cu', 'xi.cu', 'plane.cu', 'smooth.cu']


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cu', '.cuh'))]
    files.append(os.path.join(ROOT, 'include', 'pylians_gb300.h'))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                    '-I' + os.path.join(ROOT, 'include'), '--expt-relaxed-constexpr'] + list(extra_flags)

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace('.cu', '.o'))
        cmd = [cc] + flags + ['-c', os.path.join(CSRC, src), '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + '.tmp'
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcufft', '-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv,
                extra_flags=['-Xptxas', '-v'] if '--ptxas' in sys.argv else ()))
