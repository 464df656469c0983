"""Host side of the GPU Ros2 step: network upload, column batches, handles.

* ``GPUNetwork``    compiles a ``network.Network`` into the device tables
                    (C-ABI ``vk_network_compile``).
* ``ColumnBatch``   packs columns (state, rate constants, atmosphere) into the
                    flat layer-major arrays of ``vk_set_columns``.
* ``Ros2Handle``    owns a ``vk_handle``: one attempt for every column
                    (``attempt``, = op.Ros2.solver) or a device-side run to
                    steady state (``run``, = op.Integration for every column).
* ``Ros2Group``     several handles (networks of any size) run by one graph.
* ``make_ros2gpu``  builds the drop-in solver class for the reference's
                    ``op`` module (see ``Ros2GPU`` below).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, lib, ptr
from .configs import SOLVER_DEFAULTS


class GPUNetwork:
    """Device tables of one network (species order = ``net.species``)."""

    def __init__(self, net, atom_list):
        self.net = net
        self.atom_list = list(atom_list)
        sidx = {s: i for i, s in enumerate(net.species)}
        rp, rs, rn, pp, ps, pn = [0], [], [], [0], [], []
        for r in net.reactions:
            for nu, name in r.reac:
                rs.append(-1 if name == 'M' else sidx[name])
                rn.append(nu)
            for nu, name in r.prod:
                ps.append(-1 if name == 'M' else sidx[name])
                pn.append(nu)
            rp.append(len(rs))
            pp.append(len(ps))
        a = lambda v: np.ascontiguousarray(v, dtype=np.int32)
        self._keep = [a(rp), a(rs), a(rn), a(pp), a(ps), a(pn),
                      net.compo_for(self.atom_list)]
        k = self._keep
        desc = capi.VkNetworkDesc(
            net.ni, net.npair, ptr(k[0], C.c_int), ptr(k[1], C.c_int), ptr(k[2], C.c_int),
            ptr(k[3], C.c_int), ptr(k[4], C.c_int), ptr(k[5], C.c_int),
            len(self.atom_list), ptr(k[6]))
        L = lib()
        h = C.c_void_p()
        rc = L.vk_network_compile(C.byref(desc), C.byref(h))
        if rc != capi.VK_OK:
            raise capi.VkError(rc, L.vk_network_last_error().decode())
        self.handle = h
        nnz, nw, nsrc = C.c_int(), C.c_int(), C.c_int()
        check(L.vk_network_info(h, C.byref(nnz), C.byref(nw), C.byref(nsrc)))
        self.nnz, self.nw, self.nsrc = nnz.value, nw.value, nsrc.value

    def jac_pattern(self):
        rows = np.zeros(self.nnz, dtype=np.int32)
        cols = np.zeros(self.nnz, dtype=np.int32)
        check(lib().vk_network_jac_pattern(self.handle, ptr(rows, C.c_int), ptr(cols, C.c_int)))
        return rows, cols

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h:
            lib().vk_network_free(h)
            self.handle = None


def pack_atm(col, M=None, n_0=None, Tco=None):
    """Layer-major [nz][ATM_NF] atmosphere array of one Column."""
    nz = col.nz
    a = np.zeros((nz, capi.ATM_NF))
    a[:, capi.ATM_M] = col.M if M is None else M
    a[:, capi.ATM_N0] = col.n_0 if n_0 is None else n_0
    a[:, capi.ATM_TCO] = col.Tco if Tco is None else Tco
    a[:, capi.ATM_G] = col.g
    a[:-1, capi.ATM_DZI] = col.dzi
    a[:-1, capi.ATM_KZZ] = col.Kzz
    a[:-1, capi.ATM_VZ] = col.vz
    if col.Ti is not None:
        a[:-1, capi.ATM_TI] = col.Ti
    if col.Hpi is not None:
        a[:-1, capi.ATM_HPI] = col.Hpi
    a[:, capi.ATM_HP] = col.Hp
    a[:, capi.ATM_PICO] = col.pico[:-1]
    a[:, capi.ATM_PICOU] = col.pico[1:]
    if col.dz is not None:
        a[:, capi.ATM_DZ] = col.dz
    return a


def pack_spf(col, ni):
    s = np.zeros((capi.SP_NF, ni))
    s[capi.SP_MS] = col.ms
    s[capi.SP_ALPHA] = col.alpha
    s[capi.SP_TOPFLUX] = col.top_flux
    s[capi.SP_BOTFLUX] = col.bot_flux
    s[capi.SP_BOTVDEP] = col.bot_vdep
    return s


class ColumnBatch:
    """Flat arrays for vk_set_columns built from a list of column inputs.

    Each item is a dict with ``col`` (column.Column), ``k`` ([nr, nz] rate
    constants, row i-1 = k[i]), ``y`` and ``ymix`` ([nz, ni])."""

    def __init__(self, items, ni, slot_cap=0):
        self.nz = np.array([it['col'].nz for it in items], dtype=np.int32)
        self.ncols = len(items)
        self.slot_cap = int(slot_cap)
        if self.slot_cap:
            # slotted device layout (vk_set_columns_slotted): column c at c*slot_cap
            self.off = (np.arange(self.ncols + 1) * self.slot_cap).astype(np.int64)
        else:
            self.off = np.concatenate([[0], np.cumsum(self.nz)]).astype(np.int64)
        self.end = self.off[:-1] + self.nz
        self.L = int(self.off[-1])               # device layers
        self.ni = ni
        self.k = np.ascontiguousarray(np.concatenate([it['k'].T for it in items]))
        self.atm = np.ascontiguousarray(np.concatenate([pack_atm(it['col']) for it in items]))
        Dz = []
        for it in items:
            d = np.zeros((it['col'].nz, ni))
            d[:-1] = it['col'].Dzz
            Dz.append(d)
        self.Dzz = np.ascontiguousarray(np.concatenate(Dz))
        self.spf = np.ascontiguousarray(np.stack([pack_spf(it['col'], ni) for it in items]))
        self.y = np.ascontiguousarray(np.concatenate([it['y'] for it in items]))
        self.ymix = np.ascontiguousarray(np.concatenate([it['ymix'] for it in items]))
        self.pref = np.array([it['col'].pref_indx for it in items], dtype=np.int32)

    def split(self, arr):
        """Per-column views of a device-layout array [L][...]."""
        return [arr[self.off[c]:self.end[c]] for c in range(self.ncols)]

    def expand(self, packed):
        """A packed per-layer array [sum nz][...] in the device layout [L][...]."""
        if not self.slot_cap:
            return packed
        out = np.zeros((self.L,) + packed.shape[1:], dtype=packed.dtype)
        p = np.concatenate([[0], np.cumsum(self.nz)])
        for c in range(self.ncols):
            out[self.off[c]:self.end[c]] = packed[p[c]:p[c + 1]]
        return out


def ctrl_from(cfg=None, flags=None, gs=2140., Rp=1.138 * 7.1492E9, max_attempts=400):
    """vk_ctrl from a dict / module of vulcan_cfg-style knobs (defaults = reference).
    flags: VK_F_* bits; by default those of the cfg's use_moldiff / use_topflux
    / use_botflux (molecular diffusion only without a cfg)."""
    if flags is None:
        if cfg is None:
            flags = capi.VK_F_MOLDIFF
        else:
            get = cfg.get if isinstance(cfg, dict) else (lambda k, d: getattr(cfg, k, d))
            flags = ((capi.VK_F_MOLDIFF if get('use_moldiff', True) else 0)
                     | (capi.VK_F_TOPFLUX if get('use_topflux', False) else 0)
                     | (capi.VK_F_BOTFLUX if get('use_botflux', False) else 0))
    v = dict(SOLVER_DEFAULTS)
    if cfg is not None:
        for k in v:
            if isinstance(cfg, dict):
                if k in cfg:
                    v[k] = cfg[k]
            elif hasattr(cfg, k):
                v[k] = getattr(cfg, k)
    c = capi.VkCtrl()
    for k in ('rtol', 'atol', 'mtol', 'mtol_conv', 'pos_cut', 'nega_cut', 'loss_eps',
              'dt_min', 'dt_max', 'dt_var_min', 'dt_var_max', 'yconv_cri', 'slope_cri',
              'yconv_min', 'st_factor', 'trun_min', 'runtime', 'flux_cri'):
        setattr(c, k, float(v[k]))
    for k in ('conv_step', 'count_min', 'count_max', 'update_frq'):
        setattr(c, k, int(v[k]))
    c.max_attempts = int(max_attempts)
    c.flags = int(flags)
    c.gs, c.Rp = float(gs), float(Rp)
    return c


class Ros2Handle:
    """A device batch of columns on one network."""

    def __init__(self, gnet: GPUNetwork, max_cols, max_layers, precision=capi.VK_PREC_FP64):
        self.gnet = gnet
        self.ni = gnet.net.ni
        L = lib()
        h = C.c_void_p()
        rc = L.vk_create(gnet.handle, int(max_cols), int(max_layers), int(precision), C.byref(h))
        if rc != capi.VK_OK:
            raise capi.VkError(rc, L.vk_last_error(None).decode())
        self.h = h
        self.batch = None

    def close(self):
        if getattr(self, 'h', None):
            lib().vk_destroy(self.h)
            self.h = None

    __del__ = close

    def set_columns(self, batch: ColumnBatch):
        self.batch = batch
        L = lib()
        if batch.slot_cap:
            check(L.vk_set_columns_slotted(self.h, batch.ncols, batch.slot_cap,
                                           ptr(batch.nz, C.c_int), ptr(batch.k), ptr(batch.atm),
                                           ptr(batch.Dzz), ptr(batch.spf), ptr(batch.y),
                                           ptr(batch.ymix)), self.h)
        else:
            check(L.vk_set_columns(self.h, batch.ncols, ptr(batch.nz, C.c_int), ptr(batch.k),
                                   ptr(batch.atm), ptr(batch.Dzz), ptr(batch.spf), ptr(batch.y),
                                   ptr(batch.ymix)), self.h)
        check(L.vk_set_column_info(self.h, ptr(batch.pref, C.c_int), None), self.h)

    def refill(self, slots, items, atom_ini, ignore=None):
        """Continuous batching (vk_refill): the columns of ``items`` (as for
        ColumnBatch) start in ``slots`` of this slotted handle; atom_ini
        [n][natom], ignore [n][ni] masks or None.  The handle's batch keeps
        the slot layout; its nz follows the new columns."""
        b = self.batch
        nb = ColumnBatch(items, self.ni)
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        ai = np.ascontiguousarray(atom_ini, dtype=float)
        ig = None if ignore is None else np.ascontiguousarray(ignore, dtype=np.int32)
        check(lib().vk_refill(self.h, len(slots), ptr(slots, C.c_int), ptr(nb.nz, C.c_int),
                              ptr(nb.k), ptr(nb.atm), ptr(nb.Dzz), ptr(nb.spf), ptr(nb.y),
                              ptr(nb.ymix), ptr(ai), ptr(nb.pref, C.c_int),
                              ptr(ig, C.c_int) if ig is not None else None), self.h)
        b.nz[slots] = nb.nz
        b.end = b.off[:-1] + b.nz

    def set_state(self, y, ymix):
        check(lib().vk_update_state(self.h, ptr(np.ascontiguousarray(y)),
                                    ptr(np.ascontiguousarray(ymix))), self.h)

    def set_atm(self, atm):
        check(lib().vk_update_atm(self.h, ptr(np.ascontiguousarray(atm))), self.h)

    def set_k(self, k):
        check(lib().vk_update_k(self.h, ptr(np.ascontiguousarray(k))), self.h)

    def attempt(self, dt, flags=capi.VK_F_MOLDIFF, want_k=False):
        """One Ros2 attempt per column: returns dict(sol, ymix, delta[, k1, k2])."""
        b = self.batch
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, float), (b.ncols,)))
        sol = np.empty((b.L, self.ni))
        ymix = np.empty((b.L, self.ni))
        delta = np.empty(b.ncols)
        k1 = np.empty((b.L, self.ni)) if want_k else None
        k2 = np.empty((b.L, self.ni)) if want_k else None
        check(lib().vk_ros2_attempt(self.h, ptr(dt), int(flags), ptr(sol), ptr(ymix),
                                    ptr(delta), ptr(k1), ptr(k2)), self.h)
        out = dict(sol=sol, ymix=ymix, delta=delta)
        if want_k:
            out.update(k1=k1, k2=k2)
        return out

    def chem_source(self, y):
        out = np.empty((self.batch.L, self.ni))
        check(lib().vk_chem_source(self.h, ptr(np.ascontiguousarray(y)), ptr(out)), self.h)
        return out

    def rhs(self, y=None, flags=capi.VK_F_MOLDIFF):
        """f(y) = chemistry + transport (vk_rhs) [L][ni]; y None: the handle's state."""
        out = np.empty((self.batch.L, self.ni))
        yp = ptr(np.ascontiguousarray(y)) if y is not None else None
        check(lib().vk_rhs(self.h, yp, int(flags), ptr(out)), self.h)
        return out

    def lhs(self):
        b = self.batch
        jv = np.empty((b.L, self.gnet.nnz))
        dA, dB, dC = (np.empty((b.L, self.ni)) for _ in range(3))
        check(lib().vk_get_lhs(self.h, ptr(jv), ptr(dA), ptr(dB), ptr(dC)), self.h)
        return jv, dA, dB, dC

    def timing(self):
        v = [C.c_double() for _ in range(4)]
        n = C.c_int()
        check(lib().vk_get_timing(self.h, *[C.byref(x) for x in v], C.byref(n)), self.h)
        return dict(rates=v[0].value, lu=v[1].value, solve=v[2].value, stage=v[3].value,
                    launches=n.value)

    # ------------------------------------------------------------- run mode
    def set_atom_ini(self, atom_ini):
        check(lib().vk_set_atom_ini(self.h, ptr(np.ascontiguousarray(atom_ini, dtype=float))), self.h)

    def set_conv_ignore(self, mask):
        """Species the steady-state test ignores: one mask [ni] for every
        column, or one per column [ncols][ni]."""
        m = np.ascontiguousarray(mask, dtype=np.int32)
        if m.ndim == 1:
            check(lib().vk_set_column_info(self.h, None, ptr(m, C.c_int)), self.h)
        else:
            check(lib().vk_set_conv_ignore(self.h, ptr(m, C.c_int)), self.h)

    def set_clock(self, dt=None, t=None, count=None):
        b = self.batch
        f = lambda a, dt_: None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, dt_), (b.ncols,)))
        dt, t, count = f(dt, float), f(t, float), f(count, np.int32)
        check(lib().vk_set_clock(self.h, ptr(dt), ptr(t), ptr(count, C.c_int)), self.h)

    def run(self, ctrl, max_steps=0, timeout_s=0.0, max_attempts=0):
        """vk_run (max_attempts > 0: vk_run_budget, the call also ends after
        that many attempts of the batch)."""
        if max_attempts > 0:
            check(lib().vk_run_budget(self.h, C.byref(ctrl), int(max_steps), int(max_attempts),
                                      float(timeout_s)), self.h)
        else:
            check(lib().vk_run(self.h, C.byref(ctrl), int(max_steps), float(timeout_s)), self.h)

    def state(self, out=None):
        """Device state copied to host arrays: new ones, or the (e.g. pinned)
        C-contiguous arrays of ``out`` (keys y, ymix, dt, t, count, end_case,
        delta; float64, counts int32)."""
        b = self.batch
        if out is None:
            out = dict(y=np.empty((b.L, self.ni)), ymix=np.empty((b.L, self.ni)),
                       dt=np.empty(b.ncols), t=np.empty(b.ncols), delta=np.empty(b.ncols),
                       count=np.empty(b.ncols, dtype=np.int32),
                       end_case=np.empty(b.ncols, dtype=np.int32))
        for k, n in (('y', b.L * self.ni), ('ymix', b.L * self.ni), ('dt', b.ncols),
                     ('t', b.ncols), ('delta', b.ncols), ('count', b.ncols), ('end_case', b.ncols)):
            a = out[k]
            want = np.int32 if k in ('count', 'end_case') else np.float64
            if a.dtype != want or a.size != n or not a.flags.c_contiguous:
                raise ValueError('state(out): %s must be C-contiguous %s of %d' % (k, want.__name__, n))
        check(lib().vk_get_state(self.h, ptr(out['y']), ptr(out['ymix']), ptr(out['dt']),
                                 ptr(out['t']), ptr(out['count'], C.c_int),
                                 ptr(out['end_case'], C.c_int), ptr(out['delta'])), self.h)
        return out

    def set_rate_params(self, net, use_lowT_limit_rates=False):
        """Upload the network's rate parameters for compute_k (Network.rate_params)
        and, with use_lowT_limit_rates, its low-temperature caps (Network.rate_caps)."""
        kind, rev, params, nasa9 = net.rate_params()
        check(lib().vk_set_rate_params(self.h, ptr(kind, C.c_int), ptr(rev, C.c_int),
                                       ptr(np.ascontiguousarray(params)), ptr(nasa9)), self.h)
        if use_lowT_limit_rates:
            ck, ct, cp = net.rate_caps()
            check(lib().vk_set_rate_caps(self.h, ptr(ck, C.c_int), ptr(ct),
                                         ptr(np.ascontiguousarray(cp))), self.h)
        else:
            check(lib().vk_set_rate_caps(self.h, None, None, None), self.h)

    def compute_k(self):
        """Rate constants of every layer from its temperature and M, on the device."""
        check(lib().vk_compute_k(self.h), self.h)

    def k(self):
        """Device rate constants, [L, nr]."""
        out = np.empty((self.batch.L, self.gnet.net.nr))
        check(lib().vk_get_k(self.h, ptr(out)), self.h)
        return out

    def photo_update(self, mask=None):
        """Radiative transfer from the current state (vk_photo_update) of all
        columns or those with mask != 0: J into the photolysis k slots; returns
        each column's actinic-flux change (kept by the run's steady-state test)."""
        ch = np.zeros(self.batch.ncols)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        check(lib().vk_photo_update(self.h, ptr(m, C.c_int), ptr(ch)), self.h)
        return ch

    def photo_get(self):
        """(tau [L + ncols, nbins], actinic flux [L, nbins], J [L, nch])."""
        nb, nch = self.photo_dims
        b = self.batch
        tau = np.empty((b.L + b.ncols, nb))
        af = np.empty((b.L, nb))
        J = np.empty((b.L, nch))
        check(lib().vk_photo_get(self.h, ptr(tau), ptr(af), ptr(J)), self.h)
        return tau, af, J

    def set_launch(self, kernel, ctas_per_sm=0, variant=-1):
        """Launch tuning of one per-column kernel (vk_set_launch): CTAs per SM
        (0: default) and, for capi.VK_TUNE_LU32, the register tiling (-1: by ni)."""
        check(lib().vk_set_launch(self.h, int(kernel), int(ctas_per_sm), int(variant)), self.h)

    def get_launch(self, kernel):
        """(ctas_per_sm, variant) set for a kernel (vk_get_launch)."""
        c, v = C.c_int(), C.c_int()
        check(lib().vk_get_launch(self.h, int(kernel), C.byref(c), C.byref(v)), self.h)
        return c.value, v.value

    def conv_stats(self):
        """(longdy, longdydt) of each column's last steady-state test."""
        b = self.batch
        ld, ldt = np.zeros(b.ncols), np.zeros(b.ncols)
        check(lib().vk_get_conv(self.h, ptr(ld), ptr(ldt)), self.h)
        return ld, ldt

    def refine_stats(self):
        """(most sweeps any column needed, columns redone in FP64) of the last attempt."""
        a, b = C.c_int(), C.c_int()
        check(lib().vk_get_refine_stats(self.h, C.byref(a), C.byref(b)), self.h)
        return a.value, b.value

    def set_route(self, dt0):
        """Mixed precision: FP64 from step size dt0 on (until a failed
        refinement lowers a column's limit); inf restores the default."""
        check(lib().vk_set_route(self.h, float(dt0)), self.h)

    def set_precision(self, precision, max_refine=6, refine_tol=1e-10):
        check(lib().vk_set_precision(self.h, int(precision), int(max_refine), float(refine_tol)), self.h)

    def counters(self):
        """[ncols][6]: attempts, delta / negativity / loss rejections, attempts
        redone in FP64 (mixed mode), accepted steps."""
        c = np.empty((self.batch.ncols, capi.NCOUNTERS), dtype=np.int32)
        check(lib().vk_get_counters(self.h, ptr(c, C.c_int)), self.h)
        return c


class Ros2Group:
    """Handles of several networks (any ni) run to steady state by one graph
    per replay (C-ABI ``vk_group_*``): each handle's attempts and control on
    its own stream, so the networks share the GPU.  Results per handle are
    those of ``Ros2Handle.run`` on that handle alone, bit for bit.  The group
    keeps its handles alive and is closed before them."""

    def __init__(self, handles):
        self.handles = list(handles)
        n = len(self.handles)
        arr = (C.c_void_p * n)(*[h.h for h in self.handles])
        g = C.c_void_p()
        check(lib().vk_group_create(arr, n, C.byref(g)))
        self.g = g

    def close(self):
        if getattr(self, 'g', None):
            lib().vk_group_destroy(self.g)
            self.g = None

    __del__ = close

    def run(self, ctrls, max_steps=0, timeout_s=0.0, max_attempts=0):
        """vk_group_run: ctrls is one VkCtrl for every handle, or a list of
        them in handle order."""
        n = len(self.handles)
        if isinstance(ctrls, capi.VkCtrl):
            ctrls = [ctrls] * n
        if len(ctrls) != n:
            raise ValueError('one control struct per handle: %d for %d handles' % (len(ctrls), n))
        arr = (capi.VkCtrl * n)(*ctrls)
        check(lib().vk_group_run(self.g, arr, int(max_steps), int(max_attempts), float(timeout_s)))

    def timing(self):
        """(device ms, kernels launched) of the last run."""
        ms, n = C.c_double(), C.c_int()
        check(lib().vk_group_timing(self.g, C.byref(ms), C.byref(n)))
        return ms.value, n.value


# --------------------------------------------------------------------------
# Drop-in solver for the reference: op.Ros2 with the step on the GPU.

def _flags_from_cfg(cfg):
    f = 0
    if getattr(cfg, 'use_moldiff', True):
        f |= capi.VK_F_MOLDIFF
    if getattr(cfg, 'use_topflux', False):
        f |= capi.VK_F_TOPFLUX
    if getattr(cfg, 'use_botflux', False):
        f |= capi.VK_F_BOTFLUX
    return f


def _unsupported(cfg):
    """Reference options this GPU step does not implement (raise, never fall back)."""
    bad = []
    for key in ('use_vm_mol', 'use_settling', 'use_condense', 'use_ion'):
        if getattr(cfg, key, False):
            bad.append(key)
    if getattr(cfg, 'use_fix_sp_bot', {}):
        bad.append('use_fix_sp_bot')
    if getattr(cfg, 'use_fix_H2He', False):        # turns use_fix_sp_bot on (op.py:2935-2941)
        bad.append('use_fix_H2He')
    if getattr(cfg, 'non_gas_sp', []):
        bad.append('non_gas_sp')
    if getattr(cfg, 'diff_esc', []) and not getattr(cfg, 'use_moldiff', True):
        # lhs_jac_no_mol's escape term (op.py:2102-2107); with molecular
        # diffusion the escape only enters through the top flux, as here
        bad.append('diff_esc with use_moldiff = False')
    return bad


class Ros2GPUMixin:
    """Overrides ``solver`` of the reference's ``op.Ros2`` (op.py:2860-3007).

    Same contract as the reference: reads var.y, var.ymix, var.dt, var.k and
    the atmosphere arrays, writes var.y = sol, var.ymix and para.delta, and
    returns (var, para).  clip / step_ok / step_reject / step_size stay the
    reference's own (inherited), so a run through ``op.Integration`` takes the
    same accept/reject decisions."""

    _vk_net_cls = None      # network.Network, set by make_ros2gpu
    _vk_cfg = None

    def _vk_setup(self, var, atm):
        cfg = self._vk_cfg
        bad = _unsupported(cfg)
        if bad:
            raise NotImplementedError('Ros2GPU does not implement: ' + ', '.join(bad))
        net = self._vk_net_cls.from_file(cfg.network, use_photo=cfg.use_photo)
        species = self._vk_species
        if list(net.species) != list(species):
            raise RuntimeError('species order of %s differs from chem_funs.spec_list' % cfg.network)
        self._vk_gnet = GPUNetwork(net, [a for a in cfg.atom_list])
        nz = var.y.shape[0]
        self._vk_h = Ros2Handle(self._vk_gnet, 1, nz)
        self._vk_nz = nz

    def _vk_pack(self, var, atm):
        nz, ni = var.y.shape
        k = np.array([var.k[i] for i in range(1, 2 * len(self._vk_gnet.net.reactions) + 1)])
        col = _AtmView(atm, ni)
        from .solver import ColumnBatch
        b = ColumnBatch([dict(col=col, k=k, y=var.y, ymix=var.ymix)], ni)
        return b

    def solver(self, var, atm, para):
        if getattr(self, '_vk_h', None) is None:
            self._vk_setup(var, atm)
        b = self._vk_pack(var, atm)
        self._vk_h.set_columns(b)
        out = self._vk_h.attempt(var.dt, _flags_from_cfg(self._vk_cfg))
        var.y = out['sol']
        var.ymix = out['ymix']
        para.delta = float(out['delta'][0])
        return var, para

    # ---- photochemistry: the reference calls compute_tau, compute_flux and
    # compute_J in that order (vulcan.py:172-174 before the loop,
    # op.py:826-828 inside it); the device does all three in compute_J
    # (vk_photo_update), on the tables the reference's own set-up left in var
    # (make_bins_read_cross, read_sflux).  The diffuse fluxes persist on the
    # device between calls, as var.dflux_u / var.dflux_d do in the reference.
    # Temperature-dependent cross sections (T_cross_sp) use the reference's
    # per-layer var.cross_T / var.cross_J_T.  Photoionisation keeps the
    # reference's own methods (the device path does not implement it).
    def _vk_photo_gpu(self):
        return not getattr(self._vk_cfg, 'use_ion', False)

    def compute_tau(self, var, atm):
        if not self._vk_photo_gpu():
            return super().compute_tau(var, atm)

    def compute_flux(self, var, atm):
        if not self._vk_photo_gpu():
            return super().compute_flux(var, atm)

    def compute_J(self, var, atm):
        if not self._vk_photo_gpu():
            return super().compute_J(var, atm)
        from . import photo
        cfg = self._vk_cfg
        if getattr(self, '_vk_h', None) is None:
            self._vk_setup(var, atm)
        h = self._vk_h
        h.set_columns(self._vk_pack(var, atm))
        net = self._vk_gnet.net
        if getattr(h, 'photo_dims', None) is None:
            chans = sorted(var.pho_rate_index)
            # absorbers in the order the reference's compute_tau sums them
            ps = var.photo_sp if isinstance(var.photo_sp, set) else set(var.photo_sp)
            absp = list(set.union(ps, getattr(var, 'ion_sp', set())))
            t = photo.PhotoTables(
                bins=np.asarray(var.bins, float), dbin1=float(var.dbin1), dbin2=float(var.dbin2),
                i12=int(var.sflux_din12_indx), sflux_top=np.asarray(var.sflux_top, float),
                absp_sp=absp, cross=np.array([var.cross[sp] for sp in absp]),
                scat_sp=list(cfg.scat_sp), cross_scat=np.array([var.cross_scat[sp] for sp in cfg.scat_sp]),
                ch_sp=[c[0] for c in chans], ch_br=[c[1] for c in chans],
                cross_J=np.array([var.cross_J[c] for c in chans]), sl_angle=float(cfg.sl_angle),
                edd=float(cfg.edd), f_diurnal=float(cfg.f_diurnal), flux_atol=float(cfg.flux_atol))
            photo.attach(h, t, net)
            self._vk_photo_chans = chans
            tsp = set(getattr(cfg, 'T_cross_sp', []))
            if tsp:
                photo.attach_cross_T(h, {sp: var.cross_T[sp] for sp in absp if sp in tsp},
                                     {c: var.cross_J_T[c] for c in chans if c[0] in tsp})
        change = h.photo_update()
        tau, aflux, J = h.photo_get()
        nz = var.y.shape[0]
        var.tau = tau[:nz + 1]
        if hasattr(var, 'aflux'):
            var.prev_aflux = var.aflux
        var.aflux = aflux
        var.sflux = var.sflux_top * np.exp(-1. * var.tau / np.cos(cfg.sl_angle))
        var.aflux_change = float(change[0])
        remove = set(getattr(cfg, 'remove_list', []))
        var.J_sp = {(sp, 0): np.zeros(nz) for sp in var.photo_sp}
        for ch, (sp, br) in enumerate(self._vk_photo_chans):
            var.J_sp[(sp, br)] = J[:, ch].copy()
            var.J_sp[(sp, 0)] += J[:, ch]
            i = var.pho_rate_index[(sp, br)]
            if i not in remove:
                var.k[i] = J[:, ch] * cfg.f_diurnal


class _AtmView:
    """Adapter: a reference AtmData object seen as a column.Column."""

    def __init__(self, atm, ni):
        self.nz = atm.Tco.size
        self.M, self.n_0, self.Tco = atm.M, atm.n_0, atm.Tco
        self.g, self.dzi, self.Kzz, self.vz = atm.g, atm.dzi, atm.Kzz, atm.vz
        self.Ti = getattr(atm, 'Ti', None)
        self.Hpi = getattr(atm, 'Hpi', None)
        self.Hp, self.pico = atm.Hp, atm.pico
        self.dz = getattr(atm, 'dz', None)
        self.Dzz, self.ms, self.alpha = atm.Dzz, atm.ms, atm.alpha
        self.top_flux, self.bot_flux, self.bot_vdep = atm.top_flux, atm.bot_flux, atm.bot_vdep
        self.pref_indx = int(getattr(atm, 'pref_indx', 0))


def make_ros2gpu(op_module, cfg_module, species):
    """Return ``Ros2GPU``: a subclass of the reference's ``op.Ros2`` whose
    ``solver`` runs on the GPU.  Register it as ``op.Ros2GPU`` and set
    ``vulcan_cfg.ode_solver = 'Ros2GPU'`` (vulcan.py:161-163 resolves the
    solver with getattr(op, vulcan_cfg.ode_solver))."""
    from .network import Network

    class Ros2GPU(Ros2GPUMixin, op_module.Ros2):
        _vk_net_cls = Network
        _vk_cfg = cfg_module
        _vk_species = list(species)

    return Ros2GPU
