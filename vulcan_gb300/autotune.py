"""Launch autotuner for the per-column kernels.

The work-queue kernels (the FP32 and FP64 block-Thomas factorisations, the
FP64 sweeps and the mixed-precision refinement) run ``ctas_per_sm`` CTAs per
SM, and the FP32 Gauss-Jordan keeps its block in one of four register
tilings.  Which choice fills the SMs best depends on the species count, the
batch's number of columns and spread of nz, the precision path and the GPU.
``tune`` measures candidate settings on the caller's own batch -- one Ros2
attempt per measurement, the attempt's device time from vk_get_timing -- and
keeps the fastest for each kernel in turn (coordinate descent, every kernel
once per pass).  The result can be stored per (GPU, species, columns,
precision) in a JSON file and applied to later handles of the same shape.

No counterpart in the reference (its solve is one LAPACK call per step).
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import capi

# kernel name -> (vk_set_launch id, precision paths it runs in)
KERNELS = {
    'lu32': (capi.VK_TUNE_LU32, (capi.VK_PREC_MIXED,)),
    'refine': (capi.VK_TUNE_REFINE, (capi.VK_PREC_MIXED,)),
    'lu64': (capi.VK_TUNE_LU64, (capi.VK_PREC_FP64, capi.VK_PREC_MIXED)),
    'sweep64': (capi.VK_TUNE_SWEEP64, (capi.VK_PREC_FP64, capi.VK_PREC_MIXED)),
}
CTAS_PER_SM = (1, 2, 3, 4)


def candidates(kernel, ni, ctas=CTAS_PER_SM):
    """(ctas_per_sm, variant) settings worth measuring for one kernel: every
    CTAs-per-SM value, and for lu32 every register tiling that covers ni."""
    if kernel == 'lu32':
        tilings = [t for t, cap in enumerate(capi.LU32_TILING_CAP) if cap >= ni]
        return [(c, t) for t in tilings for c in ctas]
    return [(c, -1) for c in ctas]


def attempt_ms(h, dt, flags, repeats=3):
    """Median device time (ms) of ``repeats`` Ros2 attempts of the handle's
    batch at step dt (the state is not advanced by an attempt)."""
    out = []
    for _ in range(repeats):
        h.attempt(dt, flags)
        t = h.timing()
        out.append(t['rates'] + t['lu'] + t['solve'] + t['stage'])
    return float(np.median(out))


def tune(h, dt, flags=capi.VK_F_MOLDIFF, precision=capi.VK_PREC_MIXED, ni=None,
         repeats=3, passes=1, kernels=None, log=None):
    """Coordinate-descent search over the launch settings of the kernels the
    precision path runs.  Leaves the best settings applied to ``h`` and
    returns {kernel: (ctas_per_sm, variant)} plus '_ms' (best attempt time)
    and '_default_ms' (time with every setting at its default)."""
    ni = ni if ni is not None else h.ni
    names = [k for k, (_, paths) in KERNELS.items() if precision in paths
             and (kernels is None or k in kernels)]
    for k in names:                          # start from the built-in defaults
        h.set_launch(KERNELS[k][0], 0, -1)
    h.attempt(dt, flags)                     # warm-up (captures nothing, loads code)
    best_ms = default_ms = attempt_ms(h, dt, flags, repeats)
    best = {k: (0, -1) for k in names}
    for _ in range(passes):
        for k in names:
            kid = KERNELS[k][0]
            for c, v in candidates(k, ni):
                h.set_launch(kid, c, v)
                ms = attempt_ms(h, dt, flags, repeats)
                if log is not None:
                    log('%-8s ctas/SM %d variant %2d: %.3f ms' % (k, c, v, ms))
                if ms < best_ms:
                    best_ms, best[k] = ms, (c, v)
            h.set_launch(kid, *best[k])
    out = dict(best)
    out['_ms'], out['_default_ms'] = best_ms, default_ms
    return out


def apply(h, settings):
    """Apply settings returned by ``tune`` (or loaded from a cache)."""
    for k, val in settings.items():
        if k in KERNELS:
            h.set_launch(KERNELS[k][0], int(val[0]), int(val[1]))


def cache_key(gpu, ni, ncols, precision):
    return '%s|ni=%d|ncols=%d|prec=%d' % (gpu, ni, ncols, precision)


def load(path, key):
    """Settings stored under key, or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    v = d.get(key)
    return None if v is None else {k: tuple(x) if isinstance(x, list) else x
                                   for k, x in v.items()}


def save(path, key, settings):
    d = {}
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
    d[key] = {k: list(v) if isinstance(v, tuple) else v for k, v in settings.items()}
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
