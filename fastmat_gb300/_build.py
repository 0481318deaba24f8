"""Build the native engine (libfmgpu.so) in-tree with nvcc for sm_103a.

The translation units compile in parallel; the library is rebuilt only when a
source or header is newer than it.  Nothing here needs a GPU: nvcc
cross-compiles, so the build runs on any machine with the CUDA toolkit.
"""

import concurrent.futures
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
OBJDIR = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libfmgpu.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-std=c++17', '-O3', '-lineinfo', '-Xcompiler', '-fPIC',
         '-Xcompiler', '-O2', '-diag-suppress', '177']


def nvcc():
    exe = shutil.which('nvcc')
    if exe:
        return exe
    for cand in ('/usr/local/cuda/bin/nvcc',):
        if os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to '
                       'build fastmat_gb300')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _headers():
    return (glob.glob(os.path.join(CSRC, '*.cuh')) +
            glob.glob(os.path.join(ROOT, 'include', '*.h')))


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src):
    obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + '.o')
    cmd = [nvcc()] + ARCH + FLAGS + ['-c', src, '-o', obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s%s' % (
            os.path.basename(src), res.stdout, res.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile every CUDA translation unit and link libfmgpu.so."""
    srcs = _sources()
    if (not force and os.path.exists(LIB) and
            os.path.getmtime(LIB) >= _newest(srcs + _headers())):
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with concurrent.futures.ThreadPoolExecutor(workers) as pool:
        objs = list(pool.map(_compile, srcs))
    tmp = LIB + '.tmp'
    cmd = [nvcc()] + ARCH + ['-shared', '-o', tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s%s' % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print('built', LIB)
    return LIB
