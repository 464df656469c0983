"""In-tree build of libvk_gb300.so (nvcc, sm_103a only, no cmake).

Each translation unit is compiled in parallel to ``vulcan_gb300/_build/*.o``
and linked into ``vulcan_gb300/libvk_gb300.so``.  A unit is rebuilt when its
source or any header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libvk_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path():
    p = shutil.which('nvcc')
    if p:
        return p
    cand = '/usr/local/cuda/bin/nvcc'
    if os.path.exists(cand):
        return cand
    raise RuntimeError('nvcc not found')


def _flags():
    return ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                   '-Xcompiler', '-fvisibility=hidden', '--expt-relaxed-constexpr',
                   '-I', os.path.join(REPO, 'include')]


def _headers():
    return glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(REPO, 'include', '*.h'))


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + '.o')
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc_path()] + _flags() + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s%s' % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        print(r.stderr)
    return obj


def build(verbose=False, force=False):
    """Compile every CUDA/C++ source and link libvk_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for o in glob.glob(os.path.join(BUILD, '*.o')):
            os.remove(o)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc_path()] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n%s%s' % (r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    import sys
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
