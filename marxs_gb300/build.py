"""In-tree build of the CUDA library ``marxs_gb300/libmarxs_gb300.so``.

Each translation unit is compiled for sm_103a in parallel, then linked into
one shared library with a plain C ABI (``include/marxs_gb300.h``).  The
library has no PyTorch dependency; Python reaches it through ``ctypes``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libmarxs_gb300.so')
SOURCES = ['chain_fp64.cu', 'chain_fp32local.cu', 'grid_build.cu', 'capi.cu', 'adjoint.cu',
           'adjoint32.cu', 'source.cu', 'analysis.cu', 'poses.cu', 'peaks.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']
# per-file flags: the FP32-local chain divides and takes square roots with
# the approximate float32 instructions (a few ulp; measured 5.8 % faster at
# 1e8 photons, within the FP32-local precision bars); logf, sincospif and
# the other math functions keep their accurate versions
FILE_FLAGS = {'chain_fp32local.cu': ['-prec-div=false', '-prec-sqrt=false'],
              'adjoint32.cu': ['-prec-div=false', '-prec-sqrt=false']}


def nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return 'nvcc'


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    """Compile and link the library if any source changed; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cuh')]
    headers.append(os.path.join(os.path.dirname(HERE), 'include', 'marxs_gb300.h'))
    headers.append(os.path.abspath(__file__))          # flags live here
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace('.cu', '.o'))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nvcc()] + ARCH + FLAGS + FILE_FLAGS.get(src, []) + ['-c', s, '-o', o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed:\n%s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not _newer(LIB, objs):
        run([nvcc()] + ARCH + ['-shared', '-o', LIB] + objs)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
