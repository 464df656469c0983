"""Learned warm start: an MLP proposes a near-steady state for a new column.

Not part of the reference (its initial state is ``ini_mix``, build_atm.py:141;
``const_mix`` :192-198 is the fallback here).  The network maps per-layer
inputs -- log P, T, log Kzz, the column's elemental abundances, a 16-point
summary of the column's T-P profile and the layer's log10 thermochemical
equilibrium mixing ratios (eqchem.py) -- to the ni log10 mixing ratios at
steady state.  It is trained on steady states produced by this package's own
solver, with the hand-written BF16 kernels of vk_mlp.cu (forward, backward,
Adam; PyTorch only holds the device memory).

The proposal is projected onto the column's element totals (maximum-entropy
projection: mixing ratios summing to 1 in every layer, column totals equal
to those of ``const_mix``), so that plain Ros2 from the proposal conserves
the same element totals as from ``const_mix``.  Plain Ros2 then runs to the
reference's convergence test -- the solver, not the network, decides the
answer -- and a column that does not converge from its proposal can be rerun
from const_mix (fallback_items).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import check, lib

LOG_FLOOR = -30.0
N_TP = 16
N_BASE_FEATURES = 3 + 4 + N_TP


def column_features(spec, net, atom_list=('H', 'O', 'C', 'N', 'He')):
    """[nz, 23] input features of one column spec (see module docstring)."""
    pco, T = spec.pco, spec.Tco
    nz = pco.size
    logp = np.log10(pco / 1e6)
    logK = np.log10(np.mean(spec.Kzz))
    # elemental abundances (per H) of the constant-mixing start
    mix = spec.const_mix
    comp = {a: 0.0 for a in atom_list}
    for sp, x in mix.items():
        i = net.species.index(sp)
        for a in atom_list:
            comp[a] += net.compo[i, net.compo_atoms.index(a)] * x
    h = comp['H']
    ab = [np.log10(max(comp[a] / h, 1e-30)) for a in atom_list if a != 'H']
    grid = np.linspace(logp[0], logp[-1], N_TP)
    tp = np.interp(grid, logp[::-1], T[::-1]) / 1000.0
    f = np.empty((nz, 3 + len(ab) + N_TP))
    f[:, 0] = logp
    f[:, 1] = T / 1000.0
    f[:, 2] = logK
    f[:, 3:3 + len(ab)] = ab
    f[:, 3 + len(ab):] = tp[None, :]
    return f


def const_mix_abundances(spec, net, atom_list=('H', 'O', 'C', 'He', 'N')):
    """Element counts per molecule of the column's const_mix start."""
    comp = net.compo_for(list(atom_list))
    x0 = np.zeros(net.ni)
    for sp, v in spec.const_mix.items():
        x0[net.species.index(sp)] = v
    return (x0 / x0.sum()) @ comp


def eq_mix(spec, net, atom_list=('H', 'O', 'C', 'He', 'N')):
    """Thermochemical equilibrium of every layer of the column [nz, ni]."""
    from . import eqchem
    return eqchem.equilibrium(net, spec.Tco, spec.pco, const_mix_abundances(spec, net, atom_list),
                              list(atom_list))


def features_eq(spec, net, x_eq=None):
    """[nz, 23 + ni]: column_features plus the layer's log10 equilibrium
    mixing ratios (the steady state is equilibrium at depth and quenched
    above, so the network learns the departure from it)."""
    if x_eq is None:
        x_eq = eq_mix(spec, net)
    return np.concatenate([column_features(spec, net), log_targets(x_eq)], axis=1)


def log_targets(ymix):
    return np.log10(np.clip(ymix, 10.0 ** LOG_FLOOR, None))


def project_columns(xs, n0s, comp, atom_inis, iters=200, tol=1e-12):
    """Closest mixing ratios (in relative entropy) to each proposal x [nz, ni]
    with sum_i x[j, i] = 1 in every layer and the column element totals
    sum_j n0[j] sum_i comp[i, a] x[j, i] = atom_ini[a] (number densities
    summed over layers, like the reference's atom_ini, op.py:2474-2481).
    The totals must be those of a state whose layers sum to 1 (see
    start_totals): the reference's atom_ini of a const_mix start whose
    mixing ratios sum to more than 1 is not reachable under that constraint.

    The solution is x[j, i] = q[j, i] exp(comp[i] . lam) / Z_j(lam), each
    layer normalised exactly, where lam minimises the convex dual
        phi(lam) = sum_j w_j log Z_j(lam) - lam . A,   w_j = n0_j / sum n0,
    A = atom_ini / sum n0: Newton on lam (one small Hessian per column, the
    weighted covariance of the element counts) with Armijo backtracking, all
    columns at once (layers padded to the longest column).  Elements a column
    does not hold (A_a = 0) remove the species that contain them."""
    comp = np.asarray(comp, dtype=float)
    nc, ni = len(xs), comp.shape[0]
    K = comp.shape[1]
    nzs = np.array([x.shape[0] for x in xs])
    Z = int(nzs.max())
    lay = np.arange(Z)[None, :] < nzs[:, None]                      # [nc, Z]
    tot = np.array([n.sum() for n in n0s])
    w = np.zeros((nc, Z))
    logq = np.full((nc, Z, ni), -np.inf)
    for c in range(nc):
        w[c, :nzs[c]] = n0s[c] / tot[c]
        logq[c, :nzs[c]] = np.log(np.clip(xs[c], 1e-300, None))
    A = np.stack(atom_inis) / tot[:, None]                         # [nc, K]
    act = (A > 0) & (comp.sum(axis=0) > 0)[None, :]
    # species holding an element the column has none of cannot appear
    kill = ((comp[None, :, :] > 0) & ~act[:, None, :]).any(axis=2)   # [nc, ni]
    logq = np.where(kill[:, None, :], -np.inf, logq)
    logq[~lay] = 0.0                                                # padding layers: harmless
    T = np.where(act, A, 1.0)
    eye = np.eye(K)

    def state(lam, ix):
        lx = logq[ix] + np.einsum('ia,ca->ci', comp, lam * act[ix])[:, None, :]
        m = lx.max(axis=2, keepdims=True)
        e = np.exp(lx - m)
        zs = e.sum(axis=2)
        x = e / zs[:, :, None]
        logz = np.log(zs) + m[:, :, 0]
        ww = w[ix]
        phi = (ww * logz).sum(1) - (lam * A[ix] * act[ix]).sum(1)
        ef = x @ comp                                                # [n, Z, K]
        g = np.where(act[ix], np.einsum('cj,cja->ca', ww, ef) - A[ix], 0.0)
        return x, phi, g, ef

    def error(g, ix):
        return np.max(np.abs(g) / T[ix], axis=1)

    lam = np.zeros((nc, K))
    allix = np.arange(nc)
    x, phi, g, ef = state(lam, allix)
    done = np.zeros(nc, dtype=bool)
    for _ in range(iters):
        done |= error(g, allix) < tol
        if done.all():
            break
        ix = np.nonzero(~done)[0]
        xi, efi, wi = x[ix], ef[ix], w[ix]
        # Hessian: weighted covariance of the element counts per layer
        H = (np.einsum('cj,cji,ia,ib->cab', wi, xi, comp, comp, optimize=True)
             - np.einsum('cj,cja,cjb->cab', wi, efi, efi, optimize=True))
        H = np.where(act[ix][:, :, None] & act[ix][:, None, :], H, 0.0) + (~act[ix])[:, :, None] * eye
        H = H + (1e-14 * np.einsum('caa->c', H) / K + 1e-300)[:, None, None] * eye
        step = np.linalg.solve(H, g[ix][:, :, None])[:, :, 0] * act[ix]
        dec = (g[ix] * step).sum(1)
        t = np.ones(ix.size)
        acc = np.zeros(ix.size, dtype=bool)
        for _ in range(60):
            jx = np.nonzero(~acc)[0]
            cand = lam[ix[jx]] - t[jx, None] * step[jx]
            xc, pc, gc, ec = state(cand, ix[jx])
            ok = (pc <= phi[ix[jx]] - 1e-4 * t[jx] * dec[jx]) | (error(gc, ix[jx]) < 0.5 * error(g[ix[jx]], ix[jx]))
            sel = ix[jx[ok]]
            lam[sel], x[sel], phi[sel], g[sel], ef[sel] = cand[ok], xc[ok], pc[ok], gc[ok], ec[ok]
            acc[jx[ok]] = True
            if acc.all():
                break
            t = np.where(acc, t, 0.5 * t)
        done[ix[~acc]] = True                       # no decrease possible: at the floor
    return [x[c, :nzs[c]] for c in range(nc)]


def start_totals(item, comp):
    """Element totals of the normalised start n0 * ymix (what a run conserves
    after its first renormalisation y = n0 ymix, op.py:894), the projection
    target of a proposal for that column."""
    return (item['col'].n_0[:, None] * item['ymix'] @ comp).sum(axis=0)


def project_column(x, n0, comp, atom_ini, iters=100, tol=1e-12):
    """project_columns for one column."""
    return project_columns([x], [n0], comp, [np.asarray(atom_ini, dtype=float)], iters, tol)[0]


class MLP:
    """BF16 MLP (4 x 512, SiLU) trained with the vk_mlp_* kernels."""

    def __init__(self, d_in, d_out, width=512, depth=4, seed=0, device='cuda'):
        import torch
        self.torch = torch
        self.dims = [d_in] + [width] * depth + [d_out]
        g = torch.Generator().manual_seed(seed)
        self.W, self.Wb, self.b = [], [], []
        for k, n in zip(self.dims[:-1], self.dims[1:]):
            w = torch.randn(k, n, generator=g) * (1.0 / k) ** 0.5
            self.W.append(w.to(device).contiguous())
            self.Wb.append(self.W[-1].to(torch.bfloat16).contiguous())
            self.b.append(torch.zeros(n, device=device))
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step = 0
        self.device = device
        self.x_mean = self.x_std = self.y_mean = self.y_std = None

    # -------------------------------------------------------------- kernels
    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    def forward(self, X):
        """X: bf16 [B, d_in] -> (Zs, Hs); Zs[-1] is the FP32 output."""
        torch = self.torch
        L = lib()
        Zs, Hs = [], [X]
        h = X
        nl = len(self.W)
        B = X.shape[0]
        for l in range(nl):
            K, N = self.dims[l], self.dims[l + 1]
            Z = torch.empty(B, N, device=self.device)
            Hn = torch.empty(B, N, device=self.device, dtype=torch.bfloat16) if l < nl - 1 else None
            check(L.vk_mlp_forward(B, K, N, self._p(h), self._p(self.Wb[l]),
                                   C.cast(self._p(self.b[l]), C.POINTER(C.c_float)),
                                   C.cast(self._p(Z), C.POINTER(C.c_float)), self._p(Hn),
                                   1 if l < nl - 1 else 0, None))
            Zs.append(Z)
            if Hn is not None:
                Hs.append(Hn)
                h = Hn
        return Zs, Hs

    def backward(self, Zs, Hs, dout):
        """dout: FP32 gradient of the loss w.r.t. the output -> (dW, db)."""
        torch = self.torch
        L = lib()
        nl = len(self.W)
        B = dout.shape[0]
        dW = [None] * nl
        db = [None] * nl
        dH = dout.contiguous()
        fp = lambda t: C.cast(self._p(t), C.POINTER(C.c_float)) if t is not None else None
        for l in range(nl - 1, -1, -1):
            K, N = self.dims[l], self.dims[l + 1]
            dZs = torch.empty(B, N, device=self.device, dtype=torch.bfloat16)
            dW[l] = torch.empty(K, N, device=self.device)
            db[l] = torch.empty(N, device=self.device)
            dX = torch.empty(B, K, device=self.device) if l > 0 else None
            check(L.vk_mlp_backward(B, K, N, self._p(Hs[l]), self._p(self.Wb[l]), fp(Zs[l]), fp(dH),
                                    1 if l < nl - 1 else 0, self._p(dZs), fp(dW[l]), fp(db[l]),
                                    fp(dX), None))
            dH = dX
        return dW, db

    def adam(self, dW, db, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        L = lib()
        self.step += 1
        fp = lambda t: C.cast(self._p(t), C.POINTER(C.c_float))
        for l in range(len(self.W)):
            check(L.vk_mlp_adam(self.W[l].numel(), fp(self.W[l]), self._p(self.Wb[l]), fp(dW[l]),
                                fp(self.mW[l]), fp(self.vW[l]), lr, b1, b2, eps, self.step, None))
            check(L.vk_mlp_adam(self.b[l].numel(), fp(self.b[l]), None, fp(db[l]), fp(self.mb[l]),
                                fp(self.vb[l]), lr, b1, b2, eps, self.step, None))

    # ------------------------------------------------------------ training
    def fit(self, X, Y, epochs=30, batch=4096, lr=1e-3, seed=0, log=None):
        """X [S, d_in], Y [S, d_out] (numpy); standardised internally."""
        torch = self.torch
        self.x_mean, self.x_std = X.mean(0), X.std(0) + 1e-6
        self.y_mean, self.y_std = Y.mean(0), Y.std(0) + 1e-3
        Xs = torch.tensor((X - self.x_mean) / self.x_std, dtype=torch.float32, device=self.device)
        Ys = torch.tensor((Y - self.y_mean) / self.y_std, dtype=torch.float32, device=self.device)
        Xb = Xs.to(torch.bfloat16)
        S = X.shape[0]
        rng = np.random.default_rng(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.tensor(rng.permutation(S), device=self.device)
            tot = 0.0
            lr_ep = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))
            for s0 in range(0, S - batch + 1, batch):
                idx = perm[s0:s0 + batch]
                xb = Xb[idx].contiguous()
                yb = Ys[idx]
                Zs, Hs = self.forward(xb)
                diff = Zs[-1] - yb
                loss = float((diff * diff).mean())
                dout = (2.0 / diff.numel()) * diff
                dW, db = self.backward(Zs, Hs, dout)
                self.adam(dW, db, lr=lr_ep)
                tot += loss
            hist.append(tot / max(1, S // batch))
            if log:
                log('epoch %d loss %.5f' % (ep, hist[-1]))
        return hist

    def predict(self, X):
        torch = self.torch
        Xs = torch.tensor((X - self.x_mean) / self.x_std, dtype=torch.float32, device=self.device)
        Zs, _ = self.forward(Xs.to(torch.bfloat16).contiguous())
        return Zs[-1].cpu().numpy() * self.y_std + self.y_mean

    def save(self, path):
        d = {'dims': np.array(self.dims), 'x_mean': self.x_mean, 'x_std': self.x_std,
             'y_mean': self.y_mean, 'y_std': self.y_std}
        for l in range(len(self.W)):
            d['W%d' % l] = self.W[l].cpu().numpy()
            d['b%d' % l] = self.b[l].cpu().numpy()
        np.savez_compressed(path, **d)

    @classmethod
    def load(cls, path, device='cuda'):
        import torch
        d = np.load(path)
        dims = [int(v) for v in d['dims']]
        m = cls(dims[0], dims[-1], width=dims[1], depth=len(dims) - 2, device=device)
        for l in range(len(m.W)):
            m.W[l] = torch.tensor(d['W%d' % l], device=device)
            m.Wb[l] = m.W[l].to(torch.bfloat16).contiguous()
            m.b[l] = torch.tensor(d['b%d' % l], device=device)
        m.x_mean, m.x_std, m.y_mean, m.y_std = d['x_mean'], d['x_std'], d['y_mean'], d['y_std']
        return m


_EQ_NET = None


def _eq_init(net):
    global _EQ_NET
    _EQ_NET = net


def _eq_job(spec):
    return eq_mix(spec, _EQ_NET)


def eq_mix_many(specs, net, workers=None):
    """eq_mix of many columns on the host cores (a spawned process pool: the
    Gibbs minimisation is CPU work, ~0.06 s a column)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os
    workers = workers or min(16, os.cpu_count() or 1, len(specs))
    if workers <= 1 or len(specs) < 8:
        return [eq_mix(sp, net) for sp in specs]
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context('spawn'),
                                initializer=_eq_init, initargs=(net,)) as ex:
        return list(ex.map(_eq_job, specs, chunksize=max(1, len(specs) // (4 * workers))))


def propose(model, specs, net, items, atom_list=('H', 'O', 'C', 'He', 'N')):
    """Warm-start states for column items (from batch.build_items): returns a
    list of (y, ymix), each proposal projected onto its column's element
    totals (those of the const_mix start, which the run then conserves)."""
    comp = net.compo_for(list(atom_list)).astype(float)
    with_eq = model.dims[0] > N_BASE_FEATURES
    if with_eq:
        xeq = eq_mix_many(specs, net)
        feats = [features_eq(sp, net, x) for sp, x in zip(specs, xeq)]
    else:
        feats = [column_features(sp, net) for sp in specs]
    logx = model.predict(np.concatenate(feats))
    off = np.concatenate([[0], np.cumsum([f.shape[0] for f in feats])])
    xs = [10.0 ** np.clip(logx[off[c]:off[c + 1]], LOG_FLOOR, 0.0) for c in range(len(specs))]
    n0s = [it['col'].n_0 for it in items]
    xs = project_columns(xs, n0s, comp, [start_totals(it, comp) for it in items])
    return [(n0[:, None] * x, x) for n0, x in zip(n0s, xs)]


def rhs_residual(h, y, n0, batch, flags=None):
    """Residual of a state under the Ros2 system: mean over a column's layers
    of max_i |f_i(y)| / (|y_i| + 1e-10 n_0), f = chemistry + transport
    (vk_rhs) -- the rate (s^-1) at which the state still moves; zero at the
    steady state.  One value per column."""
    from . import capi
    f = h.rhs(y, capi.VK_F_MOLDIFF if flags is None else flags)
    r = np.abs(f) / (np.abs(y) + 1e-10 * n0[:, None])
    per_layer = r.max(axis=1)
    return np.array([per_layer[batch.off[c]:batch.off[c + 1]].mean() for c in range(batch.ncols)])


# --------------------------------------------------------------------------
# Pipeline: steady states from the solver -> training -> warm-started runs.

def _run_to_steady(net, specs, items, atoms, precision, count_max, timeout_s, chunk=500):
    """Integrate a batch to steady state on the device; returns the state dict."""
    from . import batch as bmod, capi, configs
    from .solver import ctrl_from
    h, b = bmod.make_batch_handle(net, items, atoms, precision=precision)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = count_max
    import time
    t0 = time.perf_counter()
    while True:
        try:
            h.run(ctrl, max_steps=chunk, timeout_s=timeout_s)
        except capi.VkError as e:
            if e.code != capi.VK_ETIMEOUT:
                raise
        st = h.state()
        if (st['end_case'] != 0).all() or time.perf_counter() - t0 > timeout_s:
            break
    st['wall_s'] = time.perf_counter() - t0
    st['counters'] = h.counters()
    st['batch'] = b
    h.close()
    return st


def generate(net, seeds, ncols, atoms, count_max=4000, timeout_s=900, precision=1, log=print):
    """Run seeded batches to steady state; return (features, targets, column
    id) of the converged columns (one sample per layer)."""
    from . import batch as bmod, configs
    Xs, Ys, Cs = [], [], []
    for seed in seeds:
        specs = configs.config2_columns(ncols=ncols, seed=seed)
        items = bmod.build_items(specs, net)
        st = _run_to_steady(net, specs, items, atoms, precision, count_max, timeout_s)
        b = st['batch']
        conv = st['end_case'] == 1
        for c in np.nonzero(conv)[0]:
            ym = st['ymix'][b.off[c]:b.off[c + 1]]
            Xs.append(features_eq(specs[c], net))
            Ys.append(log_targets(ym))
            Cs.append(np.full(ym.shape[0], seed * 100000 + c))
        log('seed %d: %d/%d converged, median steps %s, %.1f s'
            % (seed, conv.sum(), ncols, np.median(st['count'][conv]) if conv.any() else None,
               st['wall_s']))
    return np.concatenate(Xs), np.concatenate(Ys), np.concatenate(Cs)


def generate_stream(net, specs, atoms, model=None, budget_s=600.0, count_max=3000,
                    route_dt0=1e-6, nslots=512, log=print):
    """Steady states for training from a stream of columns (continuous
    batching, batch.run_stream): every column starts from the model's judged
    proposal (const_mix where there is no model or the judge rejects it) and
    runs the reference's convergence test; returns (features, targets, column
    index) of the columns that converged within budget_s seconds.  The
    solver, not the model, decides each target."""
    import time
    from . import batch as bmod, configs
    from .solver import ctrl_from
    t0 = time.perf_counter()
    items_const = bmod.build_items(specs, net)
    xeq = eq_mix_many(specs, net)
    if model is not None:
        items, used = judged_items(model, specs, net, items_const, atoms, 1)
    else:
        items, used = items_const, np.zeros(len(specs), dtype=bool)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = count_max
    left = budget_s - (time.perf_counter() - t0)
    res, wall = bmod.run_stream(net, items, atoms, nslots=min(nslots, len(items)), ctrl=ctrl,
                                precision=1, slot_cap=int(max(sp.pco.size for sp in specs)),
                                budget_s=max(left, 1.0), keep_state=True, chunk_attempts=24,
                                route_dt0=route_dt0 if model is not None else None)
    Xs, Ys, Cs = [], [], []
    for i in sorted(res):
        if res[i]['end_case'] != 1:
            continue
        Xs.append(features_eq(specs[i], net, xeq[i]))
        Ys.append(log_targets(res[i]['ymix']))
        Cs.append(np.full(res[i]['ymix'].shape[0], i))
    log('stream: %d columns, %d ended, %d converged (%d from proposals) in %.0f s'
        % (len(specs), len(res), len(Xs), int(sum(used[i] for i in res if res[i]['end_case'] == 1)),
           time.perf_counter() - t0))
    return np.concatenate(Xs), np.concatenate(Ys), np.concatenate(Cs)


def warm_items(model, specs, net, items, atoms, precision=1):
    """Items started from the projected MLP proposal (element totals those
    of the normalised const_mix start; atom_ini stays the reference's, so the
    run's conservation check reads as from const_mix); returns (items,
    used_mask).
    The solver judges the proposal: its step control and convergence test are
    the reference's, and a column that does not converge from it can be rerun
    from const_mix (fallback_items)."""
    prop = propose(model, specs, net, items, atom_list=atoms)
    out = [dict(it, y=y, ymix=x) for it, (y, x) in zip(items, prop)]
    return out, np.ones(len(items), dtype=bool)


def judge_proposals(h, batch, items_warm, items_const, flags=None):
    """The solver's judge of the learned start: a column keeps its proposal
    only where it does not raise the residual of the Ros2 system
    (rhs_residual) above that of the const_mix start; elsewhere the
    const_mix state goes back into the handle.  Returns (items, used mask)."""
    n0 = np.concatenate([it['col'].n_0 for it in items_const])
    yw = np.concatenate([it['y'] for it in items_warm])
    yc = np.concatenate([it['y'] for it in items_const])
    used = rhs_residual(h, yw, n0, batch, flags) <= rhs_residual(h, yc, n0, batch, flags)
    items = [iw if u else ic for iw, ic, u in zip(items_warm, items_const, used)]
    if not used.all():
        h.set_state(np.concatenate([it['y'] for it in items]),
                    np.concatenate([it['ymix'] for it in items]))
    return items, used


def judged_items(model, specs, net, items_const, atoms, precision=1, chunk=512):
    """Learned starts for a list of columns, each kept only where it does not
    raise the residual of the Ros2 system (judge_proposals), judged in
    handles of `chunk` columns; returns (items, used mask)."""
    from . import batch as bmod
    warm, _ = warm_items(model, specs, net, items_const, atoms, precision)
    out, used = [], []
    for a in range(0, len(items_const), chunk):
        h, b = bmod.make_batch_handle(net, warm[a:a + chunk], atoms, precision)
        it, u = judge_proposals(h, b, warm[a:a + chunk], items_const[a:a + chunk])
        h.close()
        out += it
        used.append(u)
    return out, np.concatenate(used)


def eq_items(specs, net, items, atoms):
    """Items started from thermochemical equilibrium (the reference's
    ini_mix = 'EQ' seam), projected onto the normalised const_mix start's
    element totals."""
    comp = net.compo_for(list(atoms)).astype(float)
    xs = [eq_mix(sp, net, atoms) for sp in specs]
    n0s = [it['col'].n_0 for it in items]
    xs = project_columns(xs, n0s, comp, [start_totals(it, comp) for it in items])
    return [dict(it, y=n0[:, None] * x, ymix=x) for it, n0, x in zip(items, n0s, xs)]


def fallback_items(items_const, end_case):
    """const_mix items of the columns whose warm-started run did not converge."""
    return [it for it, e in zip(items_const, end_case) if e != 1]


def main(argv=None):
    import argparse
    import json
    import os
    from .network import Network
    ap = argparse.ArgumentParser(description='learned warm start: generate / train / evaluate')
    ap.add_argument('cmd', choices=['generate', 'generate-stream', 'train'])
    ap.add_argument('--net', required=True, help='compiled network .npz or network text file')
    ap.add_argument('--seeds', default='10,11')
    ap.add_argument('--ncols', type=int, default=512)
    ap.add_argument('--data', default='warmstart_data.npz')
    ap.add_argument('--model', default='warmstart_model.npz')
    ap.add_argument('--epochs', type=int, default=100)
    ap.add_argument('--lr', type=float, default=1e-3)
    ap.add_argument('--batch', type=int, default=4096)
    ap.add_argument('--width', type=int, default=512)
    ap.add_argument('--depth', type=int, default=4)
    ap.add_argument('--count-max', type=int, default=4000)
    ap.add_argument('--timeout', type=float, default=900)
    ap.add_argument('--budget', type=float, default=600,
                    help='generate-stream: wall seconds for the whole stream')
    ap.add_argument('--proposals', default=None,
                    help='generate-stream: start the columns from this model\'s judged proposals')
    a = ap.parse_args(argv)
    net = Network.from_npz(a.net) if a.net.endswith('.npz') else Network.from_file(a.net)
    atoms = ['H', 'O', 'C', 'He', 'N']
    if a.cmd == 'generate-stream':
        from . import configs
        seeds = [int(s) for s in a.seeds.split(',')]
        specs = [sp for sd in seeds for sp in configs.config2_columns(ncols=a.ncols, seed=sd)]
        model = MLP.load(a.proposals) if a.proposals else None
        X, Y, cid = generate_stream(net, specs, atoms, model, budget_s=a.budget,
                                    count_max=min(a.count_max, 3000))
        # column ids unique across seeds: seed * 100000 + index within its seed
        cid = np.array([seeds[c // a.ncols] * 100000 + c % a.ncols for c in cid])
        np.savez_compressed(a.data, X=X.astype(np.float32), Y=Y.astype(np.float32), col=cid)
        print(json.dumps({'samples': int(X.shape[0]), 'columns': int(np.unique(cid).size),
                          'data': os.path.abspath(a.data)}))
    elif a.cmd == 'generate':
        X, Y, cid = generate(net, [int(s) for s in a.seeds.split(',')], a.ncols, atoms,
                             count_max=a.count_max, timeout_s=a.timeout)
        np.savez_compressed(a.data, X=X.astype(np.float32), Y=Y.astype(np.float32), col=cid)
        print(json.dumps({'samples': int(X.shape[0]), 'data': os.path.abspath(a.data)}))
    else:
        parts = [np.load(f) for f in a.data.split(',')]      # several generate outputs
        X = np.concatenate([d['X'] for d in parts]).astype(np.float64)
        Y = np.concatenate([d['Y'] for d in parts]).astype(np.float64)
        cid = np.concatenate([d['col'] for d in parts])
        cols = np.unique(cid)
        val = np.isin(cid, cols[::10])               # every tenth column held out
        m = MLP(X.shape[1], Y.shape[1], width=a.width, depth=a.depth)
        hist = m.fit(X[~val], Y[~val], epochs=a.epochs, batch=a.batch, lr=a.lr, log=print)
        err = np.abs(m.predict(X[val]) - Y[val])     # dex
        m.save(a.model)
        print(json.dumps({'samples': int(X.shape[0]), 'columns': int(cols.size),
                          'loss_first': hist[0], 'loss_last': hist[-1],
                          'val_dex_mean': float(err.mean()), 'val_dex_p99': float(np.percentile(err, 99)),
                          'val_dex_mean_ymix_gt_1e-10': float(err[Y[val] > -10].mean())}))


if __name__ == '__main__':
    main()
