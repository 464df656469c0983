import os
import sys

# Single-threaded BLAS for the CPU oracle, as the reference runs
# (vulcan.py:52 sets OMP_NUM_THREADS=1); threaded OpenBLAS is ~25x slower on
# the banded solves.  Must be set before numpy is imported.
for _v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
    os.environ.setdefault(_v, '1')

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built library')


def gpu_available():
    """True when the CUDA driver reports at least one device."""
    import ctypes
    try:
        cu = ctypes.CDLL('libcuda.so.1')
        if cu.cuInit(0) != 0:
            return False
        n = ctypes.c_int(0)
        return cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason='no CUDA GPU in this environment')
    for it in items:
        if 'gpu' in it.keywords:
            it.add_marker(skip)
