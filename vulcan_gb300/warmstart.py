"""Learned warm start: an MLP proposes a near-steady state for a new column.

Not part of the reference (its initial state is ``ini_mix``, build_atm.py:141;
``const_mix`` :192-198 is the fallback here).  The network maps per-layer
inputs -- log P, T, log Kzz, the column's elemental abundances and a
16-point summary of the column's T-P profile -- to the ni log10 mixing ratios
at steady state.  It is trained on steady states produced by this package's
own solver, with the hand-written BF16 kernels of vk_mlp.cu (forward,
backward, Adam; PyTorch only holds the device memory).

The proposal is projected onto the column's elemental composition
(generalised iterative scaling per layer, mixing ratios summing to 1), so that
plain Ros2 from the proposal conserves the same element totals as from
``const_mix`` and converges to the same steady state.  Plain Ros2 then runs
to the reference's convergence test; a column whose proposal has a larger
chemical residual than the const_mix start falls back to const_mix.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import column as colmod
from .capi import check, lib

LOG_FLOOR = -30.0
N_TP = 16


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


def log_targets(ymix):
    return np.log10(np.clip(ymix, 10.0 ** LOG_FLOOR, None))


def project_elements(x, compo, target, iters=100, tol=1e-12):
    """Closest mixing ratios (in relative entropy) to the proposal x [nz, ni]
    with sum_i x = 1 and element ratios sum_i compo[i,a] x_i = target[a]:
    x_i = q_i exp(sum_k lambda_k F_ik), Newton on the multipliers lambda of
    each layer (F = element counts plus a column of ones)."""
    act = (target > 0) & (compo.sum(axis=0) > 0)
    F = np.concatenate([compo[:, act], np.ones((compo.shape[0], 1))], axis=1)
    T = np.concatenate([target[act], [1.0]])
    nz, K = x.shape[0], F.shape[1]
    logq = np.log(np.clip(x, 1e-300, None))
    logq -= logq.max(axis=1, keepdims=True)
    lam = np.zeros((nz, K))

    def evalf(lm):
        lx = logq + lm @ F.T
        xx = np.exp(np.clip(lx, -745.0, 700.0))
        phi = xx.sum(axis=1) - lm @ T           # convex dual objective
        return xx, xx @ F - T[None, :], phi

    xx, g, phi = evalf(lam)
    for _ in range(iters):
        err = np.max(np.abs(g) / T[None, :], axis=1)
        todo = err >= tol
        if not todo.any():
            break
        Hm = np.einsum('zi,ik,il->zkl', xx, F, F)
        d = np.einsum('zkk->zk', Hm)
        Hm = Hm + (1e-12 * d + 1e-250)[:, :, None] * np.eye(K)[None]
        step = np.linalg.solve(Hm, g[:, :, None])[:, :, 0]
        dec = np.einsum('zk,zk->z', g, step)      # directional decrease
        t = np.ones(nz)
        acc = ~todo
        lam_n, xn, gn, phin = lam.copy(), xx.copy(), g.copy(), phi.copy()
        for _ in range(40):                        # Armijo backtracking per layer
            cand = lam - t[:, None] * step
            xc, gc, pc = evalf(cand)
            ok = (~acc) & (pc <= phi - 1e-4 * t * dec)
            lam_n[ok], xn[ok], gn[ok], phin[ok] = cand[ok], xc[ok], gc[ok], pc[ok]
            acc |= ok
            if acc.all():
                break
            t = np.where(acc, t, 0.5 * t)
        lam, xx, g, phi = lam_n, xn, gn, phin
    return xx


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


def propose(model, specs, net, items):
    """Warm-start states for column items (from batch.build_items): returns
    a list of (y, ymix, used_warm) with the proposal projected onto each
    column's elemental composition."""
    out = []
    atoms = net.compo_atoms
    comp = net.compo.astype(float)
    for spec, it in zip(specs, items):
        f = column_features(spec, net)
        logx = model.predict(f)
        x = 10.0 ** np.clip(logx, LOG_FLOOR, 0.0)
        ymix0 = it['ymix']
        target = ymix0[0] @ comp                        # element ratios of the const_mix start
        x = project_elements(x, comp, target)
        y = it['col'].n_0[:, None] * x
        out.append((y, x))
    del atoms
    return out


def chem_residual(h, y, n0, batch):
    """Mean over layers of max_i |chemical source| / n_0 (s^-1) per column."""
    src = h.chem_source(np.ascontiguousarray(y))
    r = np.abs(src) / n0[:, None]
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
    """Run seeded batches to steady state; return (features, targets) of the
    converged columns (one sample per layer)."""
    from . import batch as bmod, configs
    Xs, Ys = [], []
    for seed in seeds:
        specs = configs.config2_columns(ncols=ncols, seed=seed)
        items = bmod.build_items(specs, net)
        st = _run_to_steady(net, specs, items, atoms, precision, count_max, timeout_s)
        b = st['batch']
        conv = st['end_case'] == 1
        for c in np.nonzero(conv)[0]:
            ym = st['ymix'][b.off[c]:b.off[c + 1]]
            Xs.append(column_features(specs[c], net))
            Ys.append(log_targets(ym))
        log('seed %d: %d/%d converged, median steps %s, %.1f s'
            % (seed, conv.sum(), ncols, np.median(st['count'][conv]) if conv.any() else None,
               st['wall_s']))
    return np.concatenate(Xs), np.concatenate(Ys)


def warm_items(model, specs, net, items, atoms, precision=1):
    """Items started from the projected MLP proposal where its chemical
    residual is below that of the const_mix start; returns (items, used_mask)."""
    from . import batch as bmod
    from . import column as cm
    prop = propose(model, specs, net, items)
    h, b = bmod.make_batch_handle(net, items, atoms, precision=precision)
    n0 = np.concatenate([it['col'].n_0 for it in items])
    r_const = chem_residual(h, np.concatenate([it['y'] for it in items]), n0, b)
    r_warm = chem_residual(h, np.concatenate([p[0] for p in prop]), n0, b)
    h.close()
    used = r_warm < r_const
    out = []
    for it, (y, x), u, sp in zip(items, prop, used, specs):
        if u:
            it = dict(it, y=y, ymix=x, atom_ini=cm.atom_totals(net, y, sp.atom_list))
        out.append(it)
    return out, used


def main(argv=None):
    import argparse
    import json
    import os
    from .network import Network
    ap = argparse.ArgumentParser(description='learned warm start: generate / train / evaluate')
    ap.add_argument('cmd', choices=['generate', 'train'])
    ap.add_argument('--net', required=True, help='compiled network .npz or network text file')
    ap.add_argument('--seeds', default='10,11')
    ap.add_argument('--ncols', type=int, default=512)
    ap.add_argument('--data', default='warmstart_data.npz')
    ap.add_argument('--model', default='warmstart_model.npz')
    ap.add_argument('--epochs', type=int, default=40)
    ap.add_argument('--count-max', type=int, default=4000)
    ap.add_argument('--timeout', type=float, default=900)
    a = ap.parse_args(argv)
    net = Network.from_npz(a.net) if a.net.endswith('.npz') else Network.from_file(a.net)
    atoms = ['H', 'O', 'C', 'He', 'N']
    if a.cmd == 'generate':
        X, Y = generate(net, [int(s) for s in a.seeds.split(',')], a.ncols, atoms,
                        count_max=a.count_max, timeout_s=a.timeout)
        np.savez_compressed(a.data, X=X, Y=Y)
        print(json.dumps({'samples': int(X.shape[0]), 'data': os.path.abspath(a.data)}))
    else:
        d = np.load(a.data)
        m = MLP(d['X'].shape[1], d['Y'].shape[1])
        hist = m.fit(d['X'], d['Y'], epochs=a.epochs, log=print)
        m.save(a.model)
        print(json.dumps({'samples': int(d['X'].shape[0]), 'loss_first': hist[0], 'loss_last': hist[-1]}))


if __name__ == '__main__':
    main()
