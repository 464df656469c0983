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
        col = C.build_column(net, pco, sp.Tco, sp.Kzz, gs=configs.GS, Rp=configs.RP, ymix0=ymix)
        k = net.rate_constants(sp.Tco, col.M)
        if sp.photo_J:
            pidx = net.photo_index()
            for key, J in sp.photo_J.items():
                k[pidx[key] - 1] = J
        atom_ini = C.atom_totals(net, y, sp.atom_list)
        items.append(dict(col=col, k=k, y=y, ymix=ymix, atom_ini=atom_ini,
                          ignore=[s for s in sp.conver_ignore if s in net.species]))
    return items


def make_batch_handle(net, items, atom_list, precision=capi.VK_PREC_FP64):
    gnet = GPUNetwork(net, atom_list)
    b = ColumnBatch(items, net.ni)
    h = Ros2Handle(gnet, b.ncols, b.L, precision)
    h.set_columns(b)
    h.set_atom_ini(np.stack([it['atom_ini'] for it in items]))
    mask = np.zeros(net.ni, dtype=np.int32)
    for sp in items[0]['ignore']:
        mask[net.species.index(sp)] = 1
    h.set_conv_ignore(mask)
    h.set_clock(dt=configs.SOLVER_DEFAULTS['dttry'], t=0.0, count=0)
    return h, b


def run_batch(net, specs, atom_list, max_steps=0, timeout_s=0.0, cfg=None,
              precision=capi.VK_PREC_FP64):
    """Integrate every column to steady state (or max_steps); returns state dict."""
    items = build_items(specs, net)
    h, b = make_batch_handle(net, items, atom_list, precision)
    h.run(ctrl_from(cfg, gs=configs.GS, Rp=configs.RP), max_steps=max_steps, timeout_s=timeout_s)
    st = h.state()
    st['counters'] = h.counters()
    st['batch'] = b
    return st
