"""Benchmark: batched Ros2 steps of uneven NCHO columns on one GB300, and
columns to steady state per hour.

Workload: 512 seeded columns on the NCHO thermo network (ni=69, 782 rate
slots), nz ~ U{60..200} (sum 66 752 layers), T/Kzz/metallicity/C-O seeded
(vulcan_gb300.configs.config2_columns, seed 2).  One bench step = one Ros2 step
(attempts until accepted, device step control) of every column.

value  = accepted column-steps per second of the mixed path (FP32 tensor-core
         block LU + FP64 refinement) with the state resident in HBM, over the
         timed steps after the warm-up (early steps from const_mix).
e2e    = the same through the C-ABI with host buffers: every step copies the
         state (y, ymix) host->device, runs one step, and copies y back.
roofline = the dominant kernel of that path against its measured peak; the
         rate kernel is also reported against the measured HBM bandwidth.
plain_fp64 = the same for the FP64 path.
columns_to_steady_state = learned start + mixed vs const_mix + plain FP64:
         every column under the reference's convergence test within a wall
         budget per path (--converge-budget); converged columns per hour,
         column-steps per second over the whole trajectories, and the final
         mixing ratios against the FP64 path's.
cpu_baseline = the numpy restatement of the reference's step (banded LAPACK
         solve, as the reference does it) on a bounded sample of the same
         workload, on the host cores, timed inside the worker processes.

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
C4_NCOLS = 128
SEED = 2
ATOMS = ['H', 'O', 'C', 'He', 'N']
NET = os.path.join(REPO, 'tests', 'golden', 'net_NCHO_thermo.npz')


def peaks():
    p = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get('hbm_gbs', 6800.0), 'measured'
    return 6800.0, 'fallback'


def tf32_peak():
    """Dense TF32 tensor rate: half the measured dense BF16 burst rate (the
    same tensor cores at half the BF16 throughput), else the fallback."""
    p = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        if 'bf16_tflops' in d:
            return d['bf16_tflops'] / 2, 'measured bf16 burst / 2 (TF32 dense)'
    return 1900.0 / 2, 'fallback bf16 / 2 (TF32 dense)'


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    """Integrate one column with the numpy oracle for a fixed number of steps;
    returns (steps, seconds inside the integration loop, attempts)."""
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


def _syn_npz(write=True):
    """The 150-species synthetic network written by synthnet (deterministic)
    and its compiled npz, in the build folder (write=False: only the paths of
    files an earlier call wrote -- the CPU workers read them concurrently)."""
    from vulcan_gb300 import synthnet
    from vulcan_gb300.network import Network
    d = os.path.join(REPO, '_build', 'syn150')
    npz = os.path.join(d, 'net.npz')
    if not write:
        return os.path.join(d, 'SYN150_network.txt'), npz
    path = synthnet.generate(d)
    Network.from_file(path, use_photo=True).to_npz(npz)
    return path, npz


def _cpu_worker_c4(args):
    """One column of the 150-species stress workload (nz = 200, frozen J) with
    the numpy oracle for a fixed number of steps; (steps, seconds, attempts)."""
    idx, nsteps = args
    sys.path.insert(0, REPO)
    from oracle import ros2 as O
    from vulcan_gb300 import batch, configs, synthnet
    from vulcan_gb300.network import Network
    path, npz = _syn_npz(write=False)
    net = Network.from_file(path, use_photo=True)
    spec = configs.config4_columns(sorted(net.photo_index()), ncols=C4_NCOLS)[idx]
    it = batch.build_items([spec], net)[0]
    atoms = list(synthnet.ATOMS)
    on = O.OracleNet.from_npz(npz, atoms)
    col = it['col']
    atm = dict(M=col.M, n_0=col.n_0, Tco=col.Tco, Kzz=col.Kzz, vz=col.vz, Dzz=col.Dzz, Ti=col.Ti,
               ms=col.ms, alpha=col.alpha, pico=col.pico, dzi=col.dzi, Hpi=col.Hpi, g=col.g,
               Hp=col.Hp, dz=col.dz, zco=col.zco)
    st = O.ColState(y=it['y'].copy(), ymix=it['ymix'].copy(), dt=1e-10, atom_ini=it['atom_ini'],
                    atom_loss=np.zeros(len(atoms)))
    t0 = time.perf_counter()
    O.integrate(on, st, it['k'], atm, O.Flags(), O.Tol(), configs.GS, configs.RP,
                col.pref_indx, max_steps=nsteps, solve='banded')
    return st.count, time.perf_counter() - t0, st.attempts


def _cpu_warm(_):
    """Pool warm-up: the imports every job needs (not timed)."""
    sys.path.insert(0, REPO)
    from oracle import ros2  # noqa: F401
    from vulcan_gb300 import batch, configs  # noqa: F401
    return os.getpid()


def cpu_baseline(ncols_sample, nsteps, workers, workload='c2'):
    """The numpy restatement of the reference step on `workers` host cores.
    value = steps / (integration seconds summed over jobs / workers): the rate
    of `workers` cores each integrating columns back to back, measured inside
    the jobs (no interpreter start-up, imports or column set-up)."""
    ctx = mp.get_context('spawn')
    jobs = [(i, nsteps) for i in range(ncols_sample)]
    if workload == 'c4':
        _syn_npz()                       # written once before the workers read it
    with ctx.Pool(workers) as pool:
        pool.map(_cpu_warm, range(workers))
        t0 = time.perf_counter()
        res = pool.map(_cpu_worker_c4 if workload == 'c4' else _cpu_worker, jobs)
        wall = time.perf_counter() - t0
    steps = sum(r[0] for r in res)
    busy = sum(r[1] for r in res)
    value = steps / (busy / workers)
    what = ('the 128-column 150-species stress workload (nz = 200)' if workload == 'c4'
            else 'the 512-column workload')
    return dict(value=value, unit=UNIT, cores=workers, kind='port',
                sample='%d columns x %d Ros2 steps of %s (numpy port of the reference step, '
                       'LAPACK banded solve), %d worker processes; %.1f s of integration per '
                       'core, timed inside the jobs' % (ncols_sample, nsteps, what, workers,
                                                        busy / workers),
                wall_s=round(wall, 2), wall_rate=round(steps / wall, 3),
                attempts=sum(r[2] for r in res))


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
        except OSError:         # no nvidia-smi: no clock record
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
        except OSError:
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
def _workload(args, ncols=None):
    """(network, column specs) of the selected workload."""
    from vulcan_gb300 import configs
    from vulcan_gb300.network import Network
    if getattr(args, 'workload', 'c2') == 'c4':
        from vulcan_gb300 import synthnet
        net = Network.from_file(synthnet.generate(os.path.join(REPO, '_build', 'syn150')),
                                use_photo=True)
        specs = configs.config4_columns(sorted(net.photo_index()), ncols=C4_NCOLS)
        return net, specs[:ncols or args.ncols or C4_NCOLS]
    net = Network.from_npz(NET)
    n = ncols or args.ncols or NCOLS
    from vulcan_gb300 import replicas
    rank, ws, _ = replicas.world()
    if ws > 1 and not getattr(args, 'converge', False):
        # replicas: every rank integrates its own n columns (weak scaling),
        # a balanced share of n * world_size seeded columns
        allspecs = configs.config2_columns(ncols=n * ws, seed=SEED)
        part = replicas.column_shards([sp.pco.size for sp in allspecs], ws)[rank]
        return net, [allspecs[i] for i in part]
    return net, configs.config2_columns(ncols=NCOLS, seed=SEED)[:n]


def _setup(args, precision, ncols=None, warm_model=None, start='const_mix'):
    """Handle over the workload's columns, started from const_mix, from
    thermochemical equilibrium (start='eq') or from the learned proposal
    (warm_model; returns the mask of warm-started columns too)."""
    from vulcan_gb300 import _build, batch, configs
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import ctrl_from
    _build.build()
    net, specs = _workload(args, ncols)
    items = batch.build_items(specs, net)
    args._t_items = time.perf_counter()   # common set-up done: a start's own cost begins
    used = None
    items_const = items
    if warm_model is not None:
        from vulcan_gb300 import warmstart
        items, used = warmstart.warm_items(warm_model, specs, net, items, ATOMS, precision)
    elif start == 'eq':
        from vulcan_gb300 import warmstart
        items = warmstart.eq_items(specs, net, items, ATOMS)
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=precision)
    if warm_model is not None:
        # the proposal stands only where it does not raise the chemical residual
        from vulcan_gb300 import warmstart
        items, used = warmstart.judge_proposals(h, b, items, items_const)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    if warm_model is not None:
        return net, items, h, b, ctrl, used
    return net, items, h, b, ctrl


def _measure(args, precision, clocks=None, dist=None):
    """Warm-up, then args.steps timed steps of every column (state resident).
    With several ranks: barrier on both sides, steps summed, time the max."""
    from vulcan_gb300 import replicas
    net, items, h, b, ctrl = _setup(args, precision)
    h.run(ctrl, max_steps=args.warmup, timeout_s=1800)
    st0, c0 = h.state(), h.counters()
    launch = None
    if getattr(args, 'autotune', False):
        # launch settings measured on this batch at its current step sizes
        # (attempts do not advance the state; the clock is put back after)
        from vulcan_gb300 import autotune
        launch = autotune.tune(h, st0['dt'], precision=precision, repeats=2)
        h.set_state(st0['y'], st0['ymix'])
        h.set_clock(dt=st0['dt'], t=st0['t'], count=st0['count'])
    if clocks is not None:
        clocks.__enter__()
        time.sleep(0.3)
    replicas.barrier(dist)
    try:
        h.run(ctrl, max_steps=args.steps, timeout_s=3600)
    finally:
        if clocks is not None:
            clocks.__exit__()
    replicas.barrier(dist)
    tm = h.timing()
    st1, c1 = h.state(), h.counters()
    final = (st1['ymix'].copy(), st1['count'].copy(), st1['t'].copy(), b.off.copy())
    steps = int((st1['count'] - st0['count']).sum())
    attempts = int((c1[:, 0] - c0[:, 0]).sum())
    ms_dev = tm['rates']                  # device time of the whole run (CUDA events)
    steps_all, sec_max = replicas.reduce_run(dist, steps, ms_dev * 1e-3)
    out = dict(value=steps_all / sec_max, ms=sec_max * 1e3, steps=steps, attempts=attempts,
               launches=tm['launches'], fallbacks=int((c1[:, 4] - c0[:, 4]).sum()))
    if launch is not None:
        out['launch'] = {k: (list(v) if isinstance(v, tuple) else round(v, 3))
                         for k, v in launch.items()}
    # per-kernel device times of one attempt from the current state
    h.set_state(st1['y'], st1['ymix'])
    for _ in range(2):
        h.attempt(st1['dt'])
    out['attempt_ms'] = {k: round(v, 3) for k, v in h.timing().items() if k != 'launches'}
    # e2e: host state in (pinned), one step, host state out (pinned) -- through
    # the public API, every step
    import torch
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = {k: pin(st1[k]) for k in ('y', 'ymix', 'dt', 't', 'delta')}
    host['count'] = pin(st1['count'])
    host['end_case'] = pin(st1['end_case'])
    h.set_clock(dt=st1['dt'], t=st1['t'], count=st1['count'])
    replicas.barrier(dist)
    n_e2e, t0 = 0, time.perf_counter()
    for _ in range(max(2, min(args.steps, 5))):
        c_before = host['count'].copy()
        h.set_state(host['y'], host['ymix'])
        h.run(ctrl, max_steps=1, timeout_s=600)
        h.state(out=host)
        n_e2e += int((host['count'] - c_before).sum())
    sec = time.perf_counter() - t0
    replicas.barrier(dist)
    e2e_steps, e2e_sec = replicas.reduce_run(dist, n_e2e, sec)
    out['e2e'] = e2e_steps / e2e_sec
    out['bytes_state'] = b.L * net.ni * 8
    out['layers'] = int(b.L)
    out['ni'] = net.ni
    out['nr'] = net.nr
    out['npair'] = net.npair
    out['_final'] = final
    h.close()
    return out


def profile_traffic(kernel):
    """(DRAM bytes per layer, summary file) of `kernel` from the committed ncu
    summaries (a line 'roofline-traffic <kernel> bytes_per_layer=<B>' in
    profiles/*.md), or (None, None).  The bench does not run ncu itself: the
    traffic it reports is this capture's figure scaled to the launch."""
    import glob
    import re
    for path in sorted(glob.glob(os.path.join(REPO, 'profiles', '*.md'))):
        with open(path) as f:
            for line in f:
                m = re.match(r'\s*roofline-traffic\s+(\S+)\s+bytes_per_layer=([0-9.eE+]+)', line)
                if m and m.group(1) == kernel:
                    return float(m.group(2)), os.path.relpath(path, REPO)
    return None, None


def run_gpu(args):
    from vulcan_gb300 import replicas
    dist = replicas.init()
    rank, ws, _ = replicas.world()
    hbm, hbm_kind = peaks()
    # nvidia-smi samples of the timed region (VK_BENCH_CLOCKS overrides the file)
    clocks_csv = os.environ.get('VK_BENCH_CLOCKS', os.path.join(REPO, '_build', 'bench_clocks.csv'))
    os.makedirs(os.path.dirname(clocks_csv), exist_ok=True)
    clocks = Clocks(clocks_csv)
    mixed = _measure(args, 1, clocks if rank == 0 else None, dist)
    plain = _measure(args, 0, None, dist)
    if rank != 0:
        return
    ni, L = mixed['ni'], mixed['layers']
    # roofline of the dominant kernel of the headline path
    am = mixed['attempt_ms']
    dom = max(('lu', 'solve', 'rates'), key=lambda k: am[k])
    stride = (ni * ni + 3) // 4 * 4
    peak32 = fp32_peak_tflops()
    if dom == 'lu':
        fl = float(L) * ni ** 3 * 2.0          # Gauss-Jordan: ni^3 FMA per layer
        ach = fl / (am['lu'] * 1e-3) / 1e12
        if ni <= 128:                          # the tensor-core factorisation (default)
            ptf, src = tf32_peak()
            roof = {'bound': 'tensor', 'kernel': 'k_lu_tc (+k_prep32)', 'achieved': ach, 'peak': ptf,
                    'unit': 'TFLOP/s', 'peak_source': src,
                    'fp32_core': {'peak': round(peak32, 3), 'frac': round(ach / peak32, 4),
                                  'peak_source': 'measured cuBLAS SGEMM 8192^3 (no TF32) in this run'}}
        else:
            roof = {'bound': 'fp32', 'kernel': 'k_lu32 (+k_prep32)', 'achieved': ach, 'peak': peak32,
                    'unit': 'TFLOP/s', 'peak_source': 'measured cuBLAS SGEMM 8192^3 (no TF32) in this run'}
    else:
        # refinement + second RHS: every sweep streams the FP32 inverses twice
        by = float(L) * stride * 4 * 2 * 2 * 3
        roof = {'bound': 'hbm', 'kernel': 'k_refine', 'achieved': by / (am['solve'] * 1e-3) / 1e9,
                'peak': hbm, 'unit': 'GB/s', 'peak_source': hbm_kind}
    roof['frac'] = roof['achieved'] / roof['peak']
    # DRAM bytes per launch: the ncu capture's bytes per layer (captured on the
    # 69-species workload) x this launch's layers; none for other networks
    tpl, tsrc = profile_traffic(roof['kernel'].split()[0]) if args.workload == 'c2' else (None, None)
    roof['traffic'] = round(tpl * L) if tpl else None
    if tpl:
        roof['traffic_source'] = ('ncu capture summarised in %s: DRAM bytes per layer x the '
                                  'launch\'s %d layers (not measured in this run)' % (tsrc, L))
    for k in ('achieved', 'peak', 'frac'):
        roof[k] = round(roof[k], 4)
    peak64 = fp64_peak_tflops()
    lu64 = float(L) * ni ** 3 * 2.0 / (plain['attempt_ms']['lu'] * 1e-3) / 1e12
    rate_bytes = float(L) * (mixed['nr'] * 8 + 3 * ni * 8 + 4 * ni * 8)
    if args.workload == 'c4':
        wl = ('batched Ros2 steps, %d columns of nz=200 on a synthetic 150-species network '
              '(1200 reversible + 60 frozen photolysis reactions)' % args.ncols)
        netname = 'synthetic SYN150 (150 species, %d pairs)' % mixed['npair']
    else:
        wl = ('batched Ros2 steps, %d uneven NCHO-thermo columns (ni=69, nz 60-200, '
              'sum nz=%d)' % (args.ncols, L))
        netname = 'NCHO_thermo (69 species, 391 pairs)'
    out = {
        'metric': METRIC, 'value': round(mixed['value'], 2), 'unit': UNIT, 'n_gpus': ws,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': round(mixed['ms'] / max(args.steps, 1), 3),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64+f32',
        'data': 'synthetic (seeded columns; no dataset)',
        'config': {'workload': wl + '; FP32 scaled block LU + FP64 refinement',
                   'ncols': args.ncols, 'layers': L, 'network': netname,
                   'precision': 'mixed (FP64 rates/residual/error control, FP32 LU)',
                   'l2': 'inputs larger than L2 (state, k, Jacobian, inverses > 3 GB)'},
        'e2e': {'value': round(mixed['e2e'], 2), 'unit': UNIT,
                'h2d_bytes_per_step': 2 * mixed['bytes_state'], 'd2h_bytes_per_step': 2 * mixed['bytes_state']},
        'gpu_launches': int(mixed['launches']),
        'attempts_per_step': round(mixed['attempts'] / max(mixed['steps'], 1), 3),
        'fp64_fallback_attempts': mixed['fallbacks'],
        'roofline': roof,
        'attempt_ms': mixed['attempt_ms'],
        'plain_fp64': {'value': round(plain['value'], 2), 'unit': UNIT, 'e2e': round(plain['e2e'], 2),
                       'attempt_ms': plain['attempt_ms'],
                       'lu_roofline': {'bound': 'fp64', 'achieved': round(lu64, 4), 'peak': round(peak64, 4),
                                       'unit': 'TFLOP/s', 'frac': round(lu64 / peak64, 4),
                                       'peak_source': 'measured cuBLAS DGEMM 8192^3 in this run'}},
        'mixed_over_plain': round(mixed['value'] / plain['value'], 3),
        'launch_tuning': ({'mixed': mixed['launch'], 'plain_fp64': plain['launch']}
                          if 'launch' in mixed else 'built-in defaults'),
        'rates_kernel': {'bound': 'hbm', 'achieved': round(rate_bytes / (am['rates'] * 1e-3) / 1e9, 1),
                         'peak': hbm, 'unit': 'GB/s', 'peak_source': hbm_kind,
                         'frac': round(rate_bytes / (am['rates'] * 1e-3) / 1e9 / hbm, 4)},
    }
    # precision: mixed vs FP64 after the same timed steps, on the columns
    # whose step sequence matched (same count and time)
    ymm, cm, tmm, off = mixed.pop('_final')
    ymp, cp, tp, _ = plain.pop('_final')
    same = (cm == cp) & (np.abs(tmm / tp - 1) < 1e-9)
    em = np.where(same, 1, 0)
    out['mixed_vs_fp64_after_timed_steps'] = dict(err_vs_fp64(ymm, em, ymp, em, off),
                                                  same_step_sequence=int(same.sum()))
    out['clocks'] = clocks.summary()
    if args.converge_budget > 0 and args.workload == 'c2' and ws == 1:
        out['columns_to_steady_state'] = converge_block(args)
    if not args.no_cpu and ws == 1:
        if args.workload == 'c4':       # a step of a 150 x 200 column costs seconds on one core
            out['cpu_baseline'] = cpu_baseline(args.cpu_cols, 3, args.cpu_workers, 'c4')
        else:
            out['cpu_baseline'] = cpu_baseline(args.cpu_cols, args.cpu_steps, args.cpu_workers)
    print(json.dumps(out))


def converge_block(args):
    """Columns to steady state per hour, learned + mixed vs plain FP64: a
    stream of args.stream_cols seeded columns through 512 slots
    (continuous batching, batch.run_stream), each path for a wall budget."""
    from vulcan_gb300 import batch, configs, warmstart
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import ctrl_from
    model = None
    if os.path.exists(args.weights):
        model = warmstart.MLP.load(args.weights)
    net = Network.from_npz(NET)
    specs = configs.config2_columns(ncols=args.stream_cols, seed=SEED)
    items_const = batch.build_items(specs, net)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = args.count_max
    paths = ([('learned_mixed', 1)] if model is not None else []) + [('plain_fp64', 0)]
    res, fin = {}, {}
    for name, prec in paths:
        t0 = time.perf_counter()
        extra = {}
        items = items_const
        if name == 'learned_mixed':
            items, used = warmstart.judged_items(model, specs, net, items_const, ATOMS, prec)
            extra = {'warm_started': int(used.sum()), 'proposal_s': round(time.perf_counter() - t0, 2)}
        left = args.converge_budget - (time.perf_counter() - t0)
        sst = {}
        out, wall = batch.run_stream(net, items, ATOMS, nslots=min(NCOLS, len(items)), ctrl=ctrl,
                                     precision=prec, slot_cap=200, chunk=args.chunk_stream,
                                     budget_s=left, keep_state=True, stats=sst,
                                     chunk_attempts=args.chunk_attempts or None,
                                     route_dt0=args.route_dt if prec == 1 else None)
        wall = time.perf_counter() - t0
        conv = [i for i, r in out.items() if r['end_case'] == 1]
        steps = sorted(out[i]['count'] for i in conv)
        res[name] = {'wall_s': round(wall, 2), 'streamed_columns': len(items),
                     'ended': len(out), 'converged': len(conv),
                     'columns_per_hour': round(len(conv) / wall * 3600, 1),
                     'steps_to_converge_median': float(np.median(steps)) if steps else None,
                     'steps_to_converge_mean': float(np.mean(steps)) if steps else None,
                     'end_cases': {str(k): sum(1 for r in out.values() if r['end_case'] == k)
                                   for k in sorted({r['end_case'] for r in out.values()})},
                     # whole trajectories: every accepted step of every column
                     # that ran (ended or still in a slot at the end)
                     'column_steps': sst['steps'], 'attempts': sst['attempts'],
                     'column_steps_per_s': round(sst['steps'] / wall, 1),
                     'device_s': round(sst['device_s'], 2),
                     'column_steps_per_device_s': round(sst['steps'] / max(sst['device_s'], 1e-9), 1),
                     **extra}
        fin[name] = out
    if 'learned_mixed' in res:
        both = [i for i in fin['learned_mixed'] if i in fin['plain_fp64']
                and fin['learned_mixed'][i]['end_case'] == 1 and fin['plain_fp64'][i]['end_case'] == 1]
        errs = []
        for i in both:
            a, r = fin['learned_mixed'][i]['ymix'], fin['plain_fp64'][i]['ymix']
            m = r > 1e-20
            errs.append(float(np.max(np.abs(a[m] - r[m]) / r[m])))
        res['learned_mixed']['vs_fp64_ymix_rel_gt_1e-20'] = {
            'both_converged_with_fp64': len(both),
            'median_over_columns_of_max': float(np.median(errs)) if errs else None,
            'max_over_columns_of_max': max(errs) if errs else None,
            'columns_within_1e-3': int(sum(e <= 1e-3 for e in errs))}
        # no ratio when the FP64 stream converged no column within its budget
        fp64_cph = res['plain_fp64']['columns_per_hour']
        res['learned_mixed']['columns_per_hour_over_fp64'] = (
            round(res['learned_mixed']['columns_per_hour'] / fp64_cph, 3) if fp64_cph > 0 else None)
    res['setup'] = ('a stream of %d seeded columns through %d slots (continuous batching: a slot '
                    'whose column ends takes the next one, checked every %s), %.0f s of wall time '
                    'per path including the learned proposals and their judge (the residual of the '
                    'Ros2 system, vk_rhs); learned+mixed: FP32 factors below dt = %g s, FP64 above '
                    '(vk_set_route); count_max %d; the reference convergence test; columns per '
                    'hour = converged columns / wall' % (
                        args.stream_cols, NCOLS,
                        ('%d attempts of the batch' % args.chunk_attempts) if args.chunk_attempts
                        else ('%d steps of every column' % args.chunk_stream),
                        args.converge_budget, args.route_dt, args.count_max))
    return res


def fp32_peak_tflops():
    """cuBLAS SGEMM throughput with TF32 off (the measured FP32 denominator)."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, dtype=torch.float32, device='cuda')
    b = torch.randn(n, n, dtype=torch.float32, device='cuda')
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


def converge_path(args, name, prec, model=None, budget=None):
    """One path to steady state: every column of the workload from its start
    (learned proposal, equilibrium or const_mix) under the reference's
    convergence test (op.py:1018-1085), replayed in chunks of args.chunk steps
    until every column has ended or `budget` seconds of wall time have passed.
    Returns (result dict, final (y, ymix, end_case, count, dt, t), items)."""
    from vulcan_gb300 import capi
    budget = args.converge_timeout if budget is None else budget
    t0 = time.perf_counter()
    extra = {}
    if name == 'learned_mixed':
        net, items, h, b, ctrl, used = _setup(args, prec, warm_model=model)
        t0 = args._t_items                # the proposal and its judge count, the set-up does not
        extra = {'warm_started': int(used.sum()), 'proposal_s': round(time.perf_counter() - t0, 2)}
    elif name == 'eq_mixed':
        net, items, h, b, ctrl = _setup(args, prec, start='eq')
        t0 = args._t_items
        extra = {'proposal_s': round(time.perf_counter() - t0, 2)}
    else:
        net, items, h, b, ctrl = _setup(args, prec)
        t0 = time.perf_counter()
    ctrl.count_max = args.count_max
    if args.yconv:
        ctrl.yconv_cri = ctrl.yconv_min = args.yconv
    curve = []
    dev_s = 0.0
    while True:
        left = budget - (time.perf_counter() - t0)
        try:
            h.run(ctrl, max_steps=args.chunk, timeout_s=max(left, 1.0))
        except capi.VkError as e:
            if e.code != capi.VK_ETIMEOUT:
                raise
        dev_s += h.timing()['rates'] * 1e-3
        st = h.state()
        wall = time.perf_counter() - t0
        curve.append((round(wall, 1), int(st['count'].max()), int((st['end_case'] == 1).sum()),
                      int((st['end_case'] != 0).sum())))
        if (st['end_case'] != 0).all() or wall >= budget:
            break
    cnt = h.counters()
    conv = st['end_case'] == 1
    res = {'wall_s': round(wall, 2), 'device_s': round(dev_s, 2),
           'converged': int(conv.sum()), 'ncols': b.ncols,
           'steps_to_converge_mean': float(st['count'][conv].mean()) if conv.any() else None,
           'steps_to_converge_median': float(np.median(st['count'][conv])) if conv.any() else None,
           'steps_max': int(st['count'].max()),
           'attempts': int(cnt[:, 0].sum()), 'fp64_fallbacks': int(cnt[:, 4].sum()),
           'columns_per_hour': round(conv.sum() / wall * 3600, 1),
           'column_steps_per_s': round(float(st['count'].sum()) / wall, 1),
           'column_steps_per_device_s': round(float(st['count'].sum()) / max(dev_s, 1e-9), 1),
           'end_cases': {str(k): int(v) for k, v in zip(*np.unique(st['end_case'], return_counts=True))},
           'curve_wall_maxcount_converged_done': curve, **extra}
    final = (st['y'], st['ymix'], st['end_case'], st['count'], st['dt'], st['t'])
    h.close()
    return res, final, (net, items, b)


def err_vs_fp64(ym, em, yp, ep, off):
    """Per column converged on both paths: max |ymix - ymix_fp64| / ymix_fp64
    over species with ymix_fp64 > 1e-20; summary over those columns."""
    both = (em == 1) & (ep == 1)
    errs, meds = [], []
    for c in np.nonzero(both)[0]:
        a, r = ym[off[c]:off[c + 1]], yp[off[c]:off[c + 1]]
        m = r > 1e-20
        rel = np.abs(a[m] - r[m]) / r[m]
        errs.append(float(rel.max()))
        meds.append(float(np.median(rel)))
    return {'both_converged_with_fp64': int(both.sum()),
            'max_over_columns_of_max': max(errs) if errs else None,
            'median_over_columns_of_max': float(np.median(errs)) if errs else None,
            'median_over_columns_of_median': float(np.median(meds)) if meds else None,
            'columns_within_1e-3': int(sum(e <= 1e-3 for e in errs))}


def run_converge(args):
    """Every column to steady state on the selected paths, in chunks of steps:
    steps to converge, columns per hour, agreement of the final states."""
    from vulcan_gb300 import capi
    res = {}
    finals = {}
    paths = [('learned_mixed', 1), ('eq_mixed', 1), ('mixed', 1), ('plain_fp64', 0)]
    model = None
    if os.path.exists(args.weights):
        from vulcan_gb300 import warmstart
        model = warmstart.MLP.load(args.weights)
    else:
        paths = paths[1:]
        res['learned_mixed'] = {'skipped': 'no warm-start weights at %s' % args.weights}
    if args.precision_only:
        keep = args.precision_only.split(',')
        paths = [p for p in paths if p[0] in keep]
    items_by = {}
    for name, prec in paths:
        res[name], finals[name], items_by[name] = converge_path(args, name, prec, model)
        if args.polish:
            # continue every column from its final state for args.polish more
            # steps with a criterion that never fires: the slow transport modes
            # the convergence test does not resolve keep relaxing
            from vulcan_gb300 import batch
            from vulcan_gb300.solver import ctrl_from
            from vulcan_gb300 import configs
            net, items, b = items_by[name]
            y, ymix, ec, count, dt, t = finals[name]
            pol = [dict(it, y=y[b.off[c]:b.off[c + 1]], ymix=ymix[b.off[c]:b.off[c + 1]])
                   for c, it in enumerate(items)]
            hp, bp = batch.make_batch_handle(net, pol, ATOMS, precision=prec)
            hp.set_clock(dt=dt, t=t, count=count)
            ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
            ctrl.yconv_cri = ctrl.yconv_min = 1e-12
            ctrl.count_max = int(count.max()) + args.polish + 1
            try:
                hp.run(ctrl, max_steps=args.polish, timeout_s=args.converge_timeout)
            except capi.VkError as e:
                if e.code != capi.VK_ETIMEOUT:
                    raise
            sp = hp.state()
            hp.close()
            finals[name + '_polished'] = (sp['y'], sp['ymix'], ec, sp['count'], sp['dt'], sp['t'])
            res[name]['polished_t_median'] = float(np.median(sp['t']))
    res['metric'] = METRIC
    res['workload'] = ('%d uneven NCHO-thermo columns to steady state (%s, count_max %d)'
                       % (args.ncols, 'reference conv criterion' if not args.yconv else
                          'yconv_cri = yconv_min = %g' % args.yconv, args.count_max))
    if 'plain_fp64' in finals:
        off = items_by['plain_fp64'][2].off
        pairs = [(n, 'plain_fp64') for n in finals if n != 'plain_fp64' and not n.endswith('_polished')]
        if 'plain_fp64_polished' in finals:
            pairs += [(n, 'plain_fp64_polished') for n in finals
                      if n.endswith('_polished') and n != 'plain_fp64_polished']
            pairs += [('plain_fp64_polished', 'plain_fp64')]
        for name, refname in pairs:
            e = err_vs_fp64(finals[name][1], finals[name][2], finals[refname][1], finals[refname][2], off)
            key = name if name in res else name.replace('_polished', '')
            if name.endswith('_polished') or refname.endswith('_polished'):
                res.setdefault('polish', {})['%s_vs_%s' % (name, refname)] = e
            else:
                res[key]['vs_fp64_ymix_rel_gt_1e-20'] = e
                res[key]['speedup_columns_per_hour_vs_fp64'] = round(
                    res[key]['columns_per_hour'] / max(res['plain_fp64']['columns_per_hour'], 1e-9), 3)
    print(json.dumps(res))


def run_c1_converge(args):
    """Config 1 to steady state: one NCHO-photochemistry column (nz = 150,
    frozen seeded J, T with a seeded perturbation, Kzz log-linear 1e7-1e10)
    from const_mix under the reference's convergence test, plain FP64 and
    mixed (FP32 factors + FP64 refinement); steps, attempts, FP64 solves of
    the mixed run, device and wall time, and the final mixing ratios of the
    mixed run against the FP64 run's (where the FP64 value exceeds 1e-20)."""
    from vulcan_gb300 import _build, batch, capi, configs
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import ctrl_from
    _build.build()
    net = Network.from_npz(os.path.join(REPO, 'tests', 'golden', 'net_NCHO_photo.npz'))
    spec = configs.config1(sorted(net.photo_index()))
    items = batch.build_items([spec], net)
    res, fin = {}, {}
    for name, prec in (('plain_fp64', 0), ('mixed', 1)):
        h, b = batch.make_batch_handle(net, items, ATOMS, precision=prec)
        ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
        ctrl.count_max = args.count_max
        t0 = time.perf_counter()
        dev = 0.0
        while True:
            try:
                h.run(ctrl, max_steps=500, timeout_s=args.converge_timeout)
            except capi.VkError as e:
                if e.code != capi.VK_ETIMEOUT:
                    raise
            dev += h.timing()['rates'] * 1e-3
            st = h.state()
            if st['end_case'][0] != 0 or time.perf_counter() - t0 > args.converge_timeout:
                break
        wall = time.perf_counter() - t0
        cnt = h.counters()
        h.close()
        res[name] = {'end_case': int(st['end_case'][0]), 'steps': int(st['count'][0]),
                     't_s': float(st['t'][0]), 'attempts': int(cnt[0, 0]),
                     'fp64_solves': int(cnt[0, 4]), 'device_s': round(dev, 3), 'wall_s': round(wall, 3),
                     'steps_per_device_s': round(float(st['count'][0]) / max(dev, 1e-9), 1)}
        fin[name] = st['ymix']
    m = fin['plain_fp64'] > 1e-20
    rel = np.abs(fin['mixed'][m] - fin['plain_fp64'][m]) / fin['plain_fp64'][m]
    res['mixed_vs_fp64_ymix_rel_gt_1e-20'] = {'max': float(rel.max()), 'median': float(np.median(rel)),
                                              'within_1e-3': float((rel <= 1e-3).mean())}
    res['workload'] = ('config 1: one NCHO_photo column (69 species, nz = 150, frozen seeded J), '
                       'const_mix start, the reference convergence test, count_max %d' % args.count_max)
    print(json.dumps(res))


def run_group(args):
    """Several networks in one launch: 64 NCHO-thermo columns (69 species)
    and 16 columns of the 150-species synthetic network (nz = 200), 10 steps
    of every column after 10 warm-up steps, the two handles run one after
    the other (vk_run each) and as one group (vk_group_run), mixed and FP64;
    wall time of the calls and whether the group's final states equal the
    separate runs' bit for bit."""
    from vulcan_gb300 import _build, batch, capi, configs, synthnet
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import Ros2Group, ctrl_from
    _build.build()
    ncho = Network.from_npz(NET)
    ia = batch.build_items(configs.config2_columns(ncols=64, seed=11), ncho)
    syn = Network.from_file(synthnet.generate(os.path.join(REPO, '_build', 'syn150')),
                            use_photo=True)
    ib = batch.build_items(configs.config4_columns(sorted(syn.photo_index()), ncols=16, nz=200),
                           syn)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    out = {}
    for prec in (capi.VK_PREC_MIXED, capi.VK_PREC_FP64):
        def handles():
            return [batch.make_batch_handle(ncho, ia, ATOMS, prec)[0],
                    batch.make_batch_handle(syn, ib, ATOMS, prec)[0]]
        hs = handles()
        for h in hs:
            h.run(ctrl, max_steps=10, timeout_s=600)
        per = []
        for h in hs:
            t1 = time.perf_counter()
            h.run(ctrl, max_steps=10, timeout_s=600)
            per.append(time.perf_counter() - t1)
        ys = [h.state()['y'].copy() for h in hs]
        for h in hs:
            h.close()
        hs = handles()
        g = Ros2Group(hs)
        g.run(ctrl, max_steps=10, timeout_s=600)
        t1 = time.perf_counter()
        g.run(ctrl, max_steps=10, timeout_s=600)
        grp = time.perf_counter() - t1
        same = all(np.array_equal(y, h.state()['y']) for y, h in zip(ys, hs))
        g.close()
        for h in hs:
            h.close()
        out['mixed' if prec else 'fp64'] = dict(separate_s=[round(x, 4) for x in per],
                                                separate_total_s=round(sum(per), 4),
                                                group_s=round(grp, 4), bit_identical=same)
    print(json.dumps({'group': out, 'workload': '64 NCHO-thermo columns + 16 columns of the '
                      '150-species synthetic network (nz = 200), 10 steps each after 10'}))


def run_photo(args):
    """Radiative transfer throughput: vk_photo_update over --ncols columns of
    the NCHO photochemistry workload (nz = 150) on the reference's binned
    tables recorded in tests/golden (1 nm bins below 240 nm), against the
    numpy oracle of the same call on one column (host, one core)."""
    from vulcan_gb300 import _build, batch, configs, photo
    from vulcan_gb300.network import Network
    _build.build()
    net = Network.from_npz(os.path.join(REPO, 'tests', 'golden', 'net_NCHO_photo.npz'))
    d = dict(np.load(os.path.join(REPO, 'tests', 'golden', 'golden_c1rt.npz'), allow_pickle=False))
    tables = photo.PhotoTables.from_fixture(d)
    spec = configs.config1(sorted(net.photo_index()))
    items = batch.build_items([spec] * args.ncols, net)
    h, b = batch.make_batch_handle(net, items, ATOMS)
    photo.attach(h, tables, net)
    for _ in range(2):
        h.photo_update()
    reps = 10
    t0 = time.perf_counter()
    for _ in range(reps):
        h.photo_update()
    sec = (time.perf_counter() - t0) / reps
    h.close()
    from oracle import photo as P
    spec_list = [str(x) for x in d['spec_list']]
    ai = [spec_list.index(str(x)) for x in d['absp_sp']]
    si = [spec_list.index(str(x)) for x in d['scat_sp']]
    pi = [spec_list.index(str(x)) for x in d['photo_sp']]
    nz, nb = d['rec0_y'].shape[0], len(d['bins'])
    t0 = time.perf_counter()
    tau = P.compute_tau(d['rec0_y'], d['rec0_dz'], ai, d['cross'], si, d['cross_scat'])
    af, _, _ = P.compute_flux(tau, d['rec0_ymix'], pi, d['cross'], si, d['cross_scat'],
                              d['sflux_top'], d['bins'], float(d['sl_angle']), float(d['edd']),
                              np.zeros((nz + 1, nb)), np.zeros((nz + 1, nb)))
    P.compute_J(af, d['cross_J'], tables.weights())
    cpu = time.perf_counter() - t0
    print(json.dumps({'photo': True, 'ncols': args.ncols, 'layers': int(b.L), 'nbins': nb,
                      'channels': len(tables.ch_sp), 'update_ms': round(sec * 1e3, 3),
                      'columns_per_s': round(args.ncols / sec, 1),
                      'oracle_one_column_ms': round(cpu * 1e3, 1)}))


def run_profile(args):
    """Fixed kernel sequence for profiling: set-up, then --attempts attempts of
    every column of the first --ncols columns of the workload."""
    from vulcan_gb300 import _build, batch, configs
    from vulcan_gb300.network import Network
    _build.build()
    net, specs = _workload(args)
    items = batch.build_items(specs, net)
    prec = 1 if args.precision == 'mixed' else 0
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=prec)
    if args.lu_variant >= 0:
        from vulcan_gb300 import capi
        h.set_launch(capi.VK_TUNE_LU32, 0, args.lu_variant)
    dt = np.full(b.ncols, 1e-10)
    for _ in range(args.attempts):
        h.attempt(dt)
    print(json.dumps({'profile': True, 'precision': args.precision, 'ncols': b.ncols,
                      'layers': int(b.L), 'attempts': args.attempts, 'attempt_ms': h.timing(),
                      'refine_sweeps_fallbacks': h.refine_stats()}))
    h.close()


def run_reference(args):
    # one bounded sample: cpu_cols columns x the run's timed steps, all host cores
    res = cpu_baseline(args.cpu_cols, max(args.cpu_steps, args.steps), args.cpu_workers)
    from vulcan_gb300 import configs
    L = int(sum(sp.pco.size for sp in configs.config2_columns(ncols=NCOLS, seed=SEED)))
    out = {'metric': METRIC, 'value': round(res['value'], 3), 'unit': UNIT, 'n_gpus': args.gpus,
           'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
           'data': 'synthetic (seeded columns; no dataset)', 'impl': 'reference',
           'config': {'workload': ('batched Ros2 steps, %d uneven NCHO-thermo columns (ni=69, '
                                   'nz 60-200, sum nz=%d)' % (NCOLS, L)),
                      'ncols': NCOLS, 'layers': L, 'network': 'NCHO_thermo (69 species, 391 pairs)',
                      'precision': 'f64 (the reference step restated, LAPACK banded solve)',
                      'sample': res.get('sample')},
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
    ap.add_argument('--ncols', type=int, default=None,
                    help='columns (default 512 for c2, 128 for c4)')
    ap.add_argument('--workload', default='c2', choices=['c2', 'c4'],
                    help='c2: uneven NCHO-thermo batch; c4: synthetic 150-species network, nz=200')
    ap.add_argument('--profile', action='store_true',
                    help='only run --attempts instrumented attempts (for ncu captures)')
    ap.add_argument('--attempts', type=int, default=2)
    ap.add_argument('--lu-variant', type=int, default=-1,
                    help='profile mode: FP32 factorisation variant (vk_set_launch; -1: default)')
    ap.add_argument('--group', action='store_true',
                    help='two networks (69 and 150 species) in one graph launch against one after the other')
    ap.add_argument('--photo', action='store_true',
                    help='radiative-transfer update throughput (photochemistry workload)')
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--no-autotune', dest='autotune', action='store_false',
                    help='skip tuning the per-column kernels\' launch settings on the batch '
                         '(after the warm-up, outside the timed region) and keep the defaults')
    ap.add_argument('--converge', action='store_true',
                    help='run --ncols columns to steady state on both paths')
    ap.add_argument('--converge-c1', action='store_true',
                    help='config 1 (one NCHO-photochemistry column, nz = 150) to steady state, '
                         'plain FP64 and mixed')
    ap.add_argument('--converge-timeout', type=float, default=1800.0)
    ap.add_argument('--stream-cols', type=int, default=1536,
                    help='default run: columns streamed through the 512 slots per path')
    ap.add_argument('--chunk-stream', type=int, default=20,
                    help='steps between refills of the streamed slots (with --chunk-attempts 0)')
    ap.add_argument('--chunk-attempts', type=int, default=24,
                    help='attempts of the batch between refills of the streamed slots '
                         '(vk_run_budget; 0: refill every --chunk-stream steps of every column)')
    ap.add_argument('--route-dt', type=float, default=1e-6,
                    help='learned+mixed stream: step size from which attempts go straight to FP64 '
                         '(vk_set_route; inf: only after a failed refinement).  Columns started '
                         'near steady state fail FP32-preconditioned refinement from dt ~1e-6 s on, '
                         'and a failed refinement costs the mixed work plus a serial FP64 redo')
    ap.add_argument('--converge-budget', type=float, default=180.0,
                    help='default run: wall seconds per path for the columns-to-steady-state '
                         'measurement (0: skip)')
    ap.add_argument('--count-max', type=int, default=3000)
    ap.add_argument('--chunk', type=int, default=500)
    ap.add_argument('--polish', type=int, default=0,
                    help='converge mode: continue every column this many steps past its stop '
                         'and compare the continued states between paths')
    ap.add_argument('--yconv', type=float, default=None,
                    help='converge mode: yconv_cri = yconv_min = this (tighter than the defaults)')
    ap.add_argument('--precision-only', default=None,
                    help='comma-separated subset of learned_mixed,eq_mixed,mixed,plain_fp64 (converge mode)')
    ap.add_argument('--weights', default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                      'vulcan_gb300', 'warmstart_weights.npz'),
                    help='learned warm-start weights (converge mode)')
    ap.add_argument('--cpu-workers', type=int, default=min(16, os.cpu_count() or 1))
    args = ap.parse_args()
    if args.ncols is None:
        args.ncols = C4_NCOLS if args.workload == 'c4' else NCOLS
    rank = int(os.environ.get('RANK', '0'))
    if args.impl == 'reference':
        if rank == 0:
            run_reference(args)
        return
    if args.profile:
        run_profile(args)
        return
    if args.group:
        run_group(args)
        return
    if args.photo:
        run_photo(args)
        return
    if args.converge:
        run_converge(args)
        return
    if args.converge_c1:
        run_c1_converge(args)
        return
    run_gpu(args)


if __name__ == '__main__':
    main()
