"""Benchmark: batched Ros2 steps of uneven NCHO columns on one GB300.

Workload: 512 seeded columns on the NCHO thermo network (ni=69, 782 rate
slots), nz ~ U{60..200} (sum 66 752 layers), T/Kzz/metallicity/C-O seeded
(vulcan_gb300.configs.config2_columns, seed 2).  One bench step = one Ros2 step
(attempts until accepted, device step control) of every column.

value  = accepted column-steps per second with the state resident in HBM.
e2e    = the same through the C-ABI with host buffers: every step copies the
         state (y, ymix) host->device, runs one step, and copies y back.
roofline = the dominant kernel (block LU) against the measured FP64 peak
         (cuBLAS DGEMM) -- GB300's FP64 rate, not HBM, bounds it; the rate
         kernel is also reported against the measured HBM copy bandwidth.
cpu_baseline = the numpy restatement of the reference's step (banded LAPACK
         solve, as the reference does it) on a bounded sample of the same
         workload, on the host cores.

--impl reference  times that CPU path alone (process pool over host cores).
"""
from __future__ import annotations

import os

# The CPU path runs single-threaded BLAS per process, as the reference does
# (vulcan.py:52); set before numpy is imported (inherited by spawned workers).
for _v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
    os.environ.setdefault(_v, '1')

import argparse
import json
import multiprocessing as mp
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "columns-to-steady-state/hr & Ros2 steps/s: learned+mixed vs plain FP64, 1 GB300"
UNIT = "column-steps/s"
NCOLS = 512
SEED = 2
ATOMS = ['H', 'O', 'C', 'He', 'N']
NET = os.path.join(REPO, 'tests', 'golden', 'net_NCHO_thermo.npz')


def peaks():
    p = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get('hbm_gbs', 6800.0), 'measured'
    return 6800.0, 'fallback'


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    """Integrate one column with the numpy oracle for a fixed number of steps."""
    idx, nsteps = args
    sys.path.insert(0, REPO)
    from oracle import ros2 as O
    from vulcan_gb300 import batch, configs
    from vulcan_gb300.network import Network
    net = Network.from_npz(NET)
    spec = configs.config2_columns(ncols=NCOLS, seed=SEED)[idx]
    it = batch.build_items([spec], net)[0]
    on = O.OracleNet.from_npz(NET, ATOMS)
    col = it['col']
    atm = dict(M=col.M, n_0=col.n_0, Tco=col.Tco, Kzz=col.Kzz, vz=col.vz, Dzz=col.Dzz, Ti=col.Ti,
               ms=col.ms, alpha=col.alpha, pico=col.pico, dzi=col.dzi, Hpi=col.Hpi, g=col.g,
               Hp=col.Hp, dz=col.dz, zco=col.zco)
    st = O.ColState(y=it['y'].copy(), ymix=it['ymix'].copy(), dt=1e-10, atom_ini=it['atom_ini'],
                    atom_loss=np.zeros(len(ATOMS)))
    t0 = time.perf_counter()
    O.integrate(on, st, it['k'], atm, O.Flags(), O.Tol(), configs.GS, configs.RP,
                col.pref_indx, max_steps=nsteps, solve='banded')
    return st.count, time.perf_counter() - t0, st.attempts


def cpu_baseline(ncols_sample, nsteps, workers):
    ctx = mp.get_context('spawn')
    jobs = [(i, nsteps) for i in range(ncols_sample)]
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    steps = sum(r[0] for r in res)
    return dict(value=steps / wall, unit=UNIT, cores=workers, kind='port',
                sample='%d columns x %d Ros2 steps of the 512-column workload (numpy port of '
                       'the reference step, LAPACK banded solve), %d worker processes; '
                       '%.1f s wall' % (ncols_sample, nsteps, workers, wall),
                wall_s=wall, attempts=sum(r[2] for r in res))


# ------------------------------------------------------------ clocks
class Clocks:
    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.f = open(self.path, 'w')
            self.p = subprocess.Popen(['nvidia-smi', '--query-gpu=' + q, '--format=csv,noheader,nounits',
                                       '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            self.p.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(',') for l in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        rows = [[x.strip() for x in r] for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith('active')})
        return dict(sm_mhz=float(np.median(sm)) if sm else None,
                    sm_max_mhz=max(mx) if mx else None, reasons=reasons, samples=len(rows))


def fp64_peak_tflops():
    """cuBLAS DGEMM throughput (the measured FP64 denominator)."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device='cuda')
    b = torch.randn(n, n, dtype=torch.float64, device='cuda')
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


# ------------------------------------------------------------ GPU arm
def run_gpu(args):
    from vulcan_gb300 import _build, batch, capi, configs
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import ctrl_from
    _build.build()
    net = Network.from_npz(NET)
    specs = configs.config2_columns(ncols=NCOLS, seed=SEED)[:args.ncols]
    items = batch.build_items(specs, net)
    h, b = batch.make_batch_handle(net, items, ATOMS)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    # warm-up steps (also advances the columns past the very first steps)
    h.run(ctrl, max_steps=args.warmup, timeout_s=1800)
    st0 = h.state()
    c0 = h.counters()
    clocks = Clocks(os.path.join(REPO, 'gpurun_out', 'bench_clocks.csv')
                    if os.path.isdir(os.path.join(REPO, 'gpurun_out')) else '/tmp/bench_clocks.csv')
    with clocks:
        time.sleep(0.3)
        t0 = time.perf_counter()
        h.run(ctrl, max_steps=args.steps, timeout_s=3600)
        wall = time.perf_counter() - t0
    tm = h.timing()
    st1 = h.state()
    c1 = h.counters()
    steps = int((st1['count'] - st0['count']).sum())
    attempts = int((c1[:, 0] - c0[:, 0]).sum())
    ms_dev = tm['rates']                 # device time of the whole run (CUDA events)
    value = steps / (ms_dev * 1e-3)
    # per-kernel attempt timing (for the roofline): one instrumented attempt
    dt = st1['dt'].copy()
    h2, _ = batch.make_batch_handle(net, items, ATOMS)
    h2.set_state(st1['y'], st1['ymix'])
    for _ in range(2):
        h2.attempt(dt)
    kt = h2.timing()
    h2.close()
    # e2e: host state in, one step, host state out -- through the public API
    y_host = np.ascontiguousarray(st1['y'])
    ym_host = np.ascontiguousarray(st1['ymix'])
    e2e_steps = max(2, min(args.steps, 5))
    t0 = time.perf_counter()
    n_e2e = 0
    for _ in range(e2e_steps):
        c_before = h.state()['count']
        h.set_state(y_host, ym_host)
        h.run(ctrl, max_steps=1, timeout_s=600)
        s = h.state()
        y_host, ym_host = s['y'], s['ymix']
        n_e2e += int((s['count'] - c_before).sum())
    e2e_wall = time.perf_counter() - t0
    bytes_state = b.L * net.ni * 8
    # roofline of the dominant kernel (block LU, FP64): algorithmic flops
    nz = b.nz.astype(np.float64)
    ni = net.ni
    lu_flops = float(np.sum(nz) * 2.0 * ni ** 3)      # in-place Gauss-Jordan: n^3 FMA per layer
    peak64 = fp64_peak_tflops()
    lu_tflops = lu_flops / (kt['lu'] * 1e-3) / 1e12
    hbm, hbm_kind = peaks()
    rate_bytes = float(b.L * (2 * net.npair * 8 + 3 * ni * 8))   # k + y (3 layers) per layer, 2 evals
    out = {
        'metric': METRIC, 'value': round(value, 2), 'unit': UNIT, 'n_gpus': 1,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': round(ms_dev / max(args.steps, 1), 3),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic (seeded columns; no dataset)',
        'config': {'workload': 'batched Ros2, 512 uneven NCHO-thermo columns (ni=69, nz 60-200, '
                               'sum nz=%d), plain FP64 block LU' % b.L,
                   'ncols': NCOLS, 'layers': int(b.L), 'network': 'NCHO_thermo (69 species, 391 pairs)',
                   'precision': 'fp64', 'l2': 'inputs larger than L2 (state+inverses %.1f GB)'
                   % ((b.L * ni * ni * 8 + bytes_state * 6) / 1e9)},
        'e2e': {'value': round(n_e2e / e2e_wall, 2), 'unit': UNIT,
                'h2d_bytes_per_step': 2 * bytes_state, 'd2h_bytes_per_step': 2 * bytes_state},
        'gpu_launches': int(tm['launches']),
        'attempts_per_step': round(attempts / max(steps, 1), 3),
        'roofline': {'bound': 'fp64', 'kernel': 'k_lu_fwd_f64',
                     'achieved': round(lu_tflops, 4), 'peak': round(peak64, 4),
                     'unit': 'TFLOP/s', 'frac': round(lu_tflops / peak64, 4),
                     'peak_source': 'measured cuBLAS DGEMM 8192^3 in this run',
                     'traffic': None},
        'rates_kernel': {'bound': 'hbm', 'achieved': round(rate_bytes / (kt['rates'] * 1e-3) / 1e9, 1),
                         'peak': hbm, 'unit': 'GB/s', 'peak_source': hbm_kind,
                         'frac': round(rate_bytes / (kt['rates'] * 1e-3) / 1e9 / hbm, 4)},
        'attempt_ms': {k: round(v, 3) for k, v in kt.items() if k != 'launches'},
    }
    out['clocks'] = clocks.summary()
    if not args.no_cpu:
        out['cpu_baseline'] = cpu_baseline(args.cpu_cols, args.cpu_steps, args.cpu_workers)
    print(json.dumps(out))
    h.close()


def run_profile(args):
    """Fixed kernel sequence for profiling: set-up, then --attempts attempts of
    every column of the first --ncols columns of the workload."""
    from vulcan_gb300 import _build, batch, configs
    from vulcan_gb300.network import Network
    _build.build()
    net = Network.from_npz(NET)
    specs = configs.config2_columns(ncols=NCOLS, seed=SEED)[:args.ncols]
    items = batch.build_items(specs, net)
    prec = 1 if args.precision == 'mixed' else 0
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=prec)
    dt = np.full(b.ncols, 1e-10)
    for _ in range(args.attempts):
        h.attempt(dt)
    print(json.dumps({'profile': True, 'precision': args.precision, 'ncols': b.ncols,
                      'layers': int(b.L), 'attempts': args.attempts, 'attempt_ms': h.timing(),
                      'refine_sweeps_fallbacks': h.refine_stats()}))
    h.close()


def run_reference(args):
    res = cpu_baseline(args.cpu_cols, args.cpu_steps, args.cpu_workers)
    out = {'metric': METRIC, 'value': round(res['value'], 3), 'unit': UNIT, 'n_gpus': args.gpus,
           'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
           'data': 'synthetic (seeded columns; no dataset)', 'impl': 'reference',
           'config': {'workload': 'batched Ros2, 512 uneven NCHO-thermo columns (ni=69, nz 60-200), '
                                  'bounded sample on host cores'},
           'cpu_baseline': res,
           'e2e': {'value': round(res['value'], 3), 'unit': UNIT, 'h2d_bytes_per_step': 0,
                   'd2h_bytes_per_step': 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--cpu-cols', type=int, default=16)
    ap.add_argument('--cpu-steps', type=int, default=8)
    ap.add_argument('--ncols', type=int, default=NCOLS)
    ap.add_argument('--profile', action='store_true',
                    help='only run --attempts instrumented attempts (for ncu captures)')
    ap.add_argument('--attempts', type=int, default=2)
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--cpu-workers', type=int, default=min(16, os.cpu_count() or 1))
    args = ap.parse_args()
    rank = int(os.environ.get('RANK', '0'))
    if args.impl == 'reference':
        if rank == 0:
            run_reference(args)
        return
    if args.profile:
        run_profile(args)
        return
    run_gpu(args)


if __name__ == '__main__':
    main()
