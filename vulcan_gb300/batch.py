"""Batched columns: build many seeded columns and integrate them on the device.

``build_items`` turns column specifications (configs.ColumnSpec) into the
inputs of a ColumnBatch: FP64 set-up (rate constants, atmosphere, initial
constant mixing ratios, element totals).  ``run_batch`` integrates every
column to steady state on the GPU (the per-column loop of the reference's
op.Integration, one CUDA-graph replay per group of attempts).
"""
from __future__ import annotations

import numpy as np

from . import column as C
from .solver import ColumnBatch, GPUNetwork, Ros2Handle, ctrl_from
from . import capi, configs


def build_items(specs, net):
    """Column set-up for a list of ColumnSpec on one network."""
    items = []
    for sp in specs:
        pco = sp.pco
        n_0 = pco / (C.KB * sp.Tco)
        y, ymix = C.const_mix_state(net, n_0, sp.const_mix)
        col = C.build_column(net, pco, sp.Tco, sp.Kzz, gs=configs.GS, Rp=configs.RP,
                             rocky=getattr(sp, 'rocky', False),
                             use_moldiff=getattr(sp, 'use_moldiff', True),
                             atm_base=getattr(sp, 'atm_base', 'H2'), vz=getattr(sp, 'vz', None),
                             ymix0=ymix)
        for name, v in (getattr(sp, 'top_flux', None) or {}).items():     # BC_flux, build_atm.py:742-762
            col.top_flux[net.species.index(name)] = v
        for name, (v, vdep) in (getattr(sp, 'bot_flux', None) or {}).items():
            col.bot_flux[net.species.index(name)] = v
            col.bot_vdep[net.species.index(name)] = vdep
        k = net.rate_constants(sp.Tco, col.M)
        if sp.photo_J:
            pidx = net.photo_index()
            for key, J in sp.photo_J.items():
                k[pidx[key] - 1] = J
        atom_ini = C.atom_totals(net, y, sp.atom_list)
        items.append(dict(col=col, k=k, y=y, ymix=ymix, atom_ini=atom_ini,
                          ignore=[s for s in sp.conver_ignore if s in net.species]))
    return items


def ignore_masks(net, items):
    """[n][ni] steady-state ignore masks (conver_ignore) of column items."""
    mask = np.zeros((len(items), net.ni), dtype=np.int32)
    for c, it in enumerate(items):
        for sp in it['ignore']:
            mask[c, net.species.index(sp)] = 1
    return mask


def make_batch_handle(net, items, atom_list, precision=capi.VK_PREC_FP64, slot_cap=0):
    """Handle with the items' columns loaded (slot_cap > 0: the slotted layout
    of continuous batching, each column in a slot of slot_cap layers)."""
    gnet = GPUNetwork(net, atom_list)
    b = ColumnBatch(items, net.ni, slot_cap)
    h = Ros2Handle(gnet, b.ncols, b.L, precision)
    h.set_columns(b)
    h.set_atom_ini(np.stack([it['atom_ini'] for it in items]))
    h.set_conv_ignore(ignore_masks(net, items))
    h.set_clock(dt=configs.SOLVER_DEFAULTS['dttry'], t=0.0, count=0)
    return h, b


def run_stream(net, items, atom_list, nslots, ctrl, precision=capi.VK_PREC_FP64, slot_cap=None,
               chunk=20, budget_s=None, keep_state=False, stats=None, route_dt0=None,
               chunk_attempts=None):
    """Continuous batching: the column items (build_items order) stream
    through nslots slots of one handle; every `chunk` steps the slots whose
    column has ended (converged, count_max, runtime, error) take the next
    items (vk_refill), so the GPU keeps a full batch while columns finish at
    different times.  Each column runs the reference's loop (op.py:808-936)
    from its own start, exactly as in a batch of its own.  Stops when every
    item has ended or after budget_s seconds of wall time.  route_dt0 (mixed
    precision): the step size from which attempts go straight to FP64
    (vk_set_route).  chunk_attempts: refill after that many attempts of the
    batch (vk_run_budget) instead of after `chunk` steps of every column, so
    a column whose steps need many rejected attempts does not hold the
    others' slots idle.

    Returns (results, wall_s): results[i] = dict(end_case, count, t, wall_s
    at which it ended[, y, ymix]) for every item that ended.  A dict passed as
    ``stats`` receives the accepted steps of every column that ran (ended or
    still in a slot when the budget ran out), the attempts, and the device
    time of the runs (CUDA events, s)."""
    import time
    from . import capi as _capi
    slot_cap = slot_cap or int(max(it['col'].nz for it in items))
    first = list(items[:nslots])
    h, b = make_batch_handle(net, first, atom_list, precision, slot_cap=slot_cap)
    if route_dt0 is not None and precision == _capi.VK_PREC_MIXED:
        h.set_route(route_dt0)
    slot_item = list(range(len(first)))
    nxt = len(first)
    results = {}
    steps_done = attempts_done = 0
    dev_s = 0.0
    t0 = time.perf_counter()
    try:
        while True:
            left = None if budget_s is None else budget_s - (time.perf_counter() - t0)
            if left is not None and left <= 0:
                break
            try:
                tmo = max(left, 1.0) if left is not None else 0.0
                if chunk_attempts:
                    h.run(ctrl, max_steps=0, timeout_s=tmo, max_attempts=chunk_attempts)
                else:
                    h.run(ctrl, max_steps=chunk, timeout_s=tmo)
            except _capi.VkError as e:
                if e.code != _capi.VK_ETIMEOUT:
                    raise
            dev_s += h.timing()['rates'] * 1e-3
            st = h.state()
            now = time.perf_counter() - t0
            ended = [c for c in range(b.ncols) if slot_item[c] is not None and st['end_case'][c] != 0]
            if ended:
                cnt = h.counters()
                steps_done += int(st['count'][ended].sum())
                attempts_done += int(cnt[ended, 0].sum())
            for c in ended:
                r = dict(end_case=int(st['end_case'][c]), count=int(st['count'][c]),
                         t=float(st['t'][c]), wall_s=now)
                if keep_state:
                    r['y'] = st['y'][b.off[c]:b.end[c]].copy()
                    r['ymix'] = st['ymix'][b.off[c]:b.end[c]].copy()
                results[slot_item[c]] = r
                slot_item[c] = None
            new = list(range(nxt, min(nxt + len(ended), len(items))))
            if new:
                slots = ended[:len(new)]
                nitems = [items[i] for i in new]
                h.refill(slots, nitems, np.stack([it['atom_ini'] for it in nitems]),
                         ignore_masks(net, nitems))
                for c, i in zip(slots, new):
                    slot_item[c] = i
                nxt += len(new)
            if all(si is None for si in slot_item):
                break
        if stats is not None:
            live = [c for c in range(b.ncols) if slot_item[c] is not None]
            st = h.state()
            cnt = h.counters()
            stats['steps'] = steps_done + int(st['count'][live].sum())
            stats['attempts'] = attempts_done + int(cnt[live, 0].sum())
            stats['device_s'] = dev_s
    finally:
        h.close()
    return results, time.perf_counter() - t0


def run_batch(net, specs, atom_list, max_steps=0, timeout_s=0.0, cfg=None,
              precision=capi.VK_PREC_FP64):
    """Integrate every column to steady state (or max_steps); returns state
    dict.  ``cfg`` (dict or vulcan_cfg-like module) gives the solver knobs and
    use_moldiff / use_topflux / use_botflux."""
    items = build_items(specs, net)
    h, b = make_batch_handle(net, items, atom_list, precision)
    h.run(ctrl_from(cfg, gs=configs.GS, Rp=configs.RP), max_steps=max_steps, timeout_s=timeout_s)
    st = h.state()
    st['counters'] = h.counters()
    st['batch'] = b
    return st


def run_with_photo(h, ctrl, max_steps, ini_frq=100, final_frq=5, chunk=5, timeout_s=0.0):
    """vk_run with the reference's photochemistry schedule (Integration.__call__,
    op.py:811-830): before a step whose count is a multiple of the column's
    update_photo_frq, recompute its J from the current state
    (vk_photo_update); a column's frequency switches from ini_frq to final_frq
    once longdy < 10 yconv_min and longdydt < 1e-6.  Runs chunks of ``chunk``
    steps (a divisor of both frequencies) until every column has ended or
    max_steps steps were taken; returns the final state."""
    from . import capi
    if ini_frq % chunk or final_frq % chunk:
        raise ValueError('chunk must divide both photo update frequencies')
    n = h.batch.ncols
    final = np.zeros(n, dtype=bool)
    done_steps = 0
    while done_steps < max_steps:
        st = h.state()
        live = st['end_case'] == 0
        if not live.any():
            break
        ld, ldt = h.conv_stats()
        final |= (ld < ctrl.yconv_min * 10.) & (ldt < 1.e-6)
        frq = np.where(final, final_frq, ini_frq)
        due = live & (st['count'] % frq == 0)
        if due.any():
            h.photo_update(due.astype(np.int32))
        try:
            h.run(ctrl, max_steps=chunk, timeout_s=timeout_s)
        except capi.VkError as e:
            if e.code != capi.VK_ETIMEOUT:
                raise
        done_steps += chunk
    return h.state()
