"""Thermochemical equilibrium of every layer (ideal gas, no condensates).

The reference's ``ini_mix = 'EQ'`` start (build_atm.py:78-164) calls FastChem;
this is an independent restatement of the same physics with the network's own
Gibbs data (the NASA-9 g/RT the reverse rates use, network.py ``gibbs_RT``):
minimise  G = sum_i n_i (g_i(T) + ln(P / P0) + ln(n_i / N))  subject to the
element abundances.  Its stationary point is the element-potential form

    x_i = exp(-c_i + F_i . lam),   c_i = g_i(T) + ln(P / P0),

with sum_i x_i = 1 and the element abundances.  Solved in mole numbers by the
published Gordon & McBride iteration (NASA RP-1311, 1994: Newton on the
element potentials and ln N with the species corrections eliminated, step
damping on the major and minor species), every layer at once.
"""
from __future__ import annotations

import numpy as np

P0 = 1.0e6                      # 1 bar in dyn cm^-2 (the reference's gibbs corr)


def equilibrium(net, T, P, abund, atom_list, iters=400, tol=5e-10):
    """Equilibrium mole fractions [nz, ni] at temperatures T [nz] (K),
    pressures P [nz] (dyn cm^-2) and element abundances ``abund`` (relative
    numbers per element of atom_list, any scale)."""
    T = np.asarray(T, dtype=float)
    P = np.asarray(P, dtype=float)
    Fall = net.compo_for(list(atom_list)).astype(float)
    b = np.asarray(abund, dtype=float)
    act = (b > 0) & (Fall.sum(axis=0) > 0)
    # species that contain an absent element cannot form
    keep = np.all(Fall[:, ~act] == 0, axis=1)
    F = Fall[keep][:, act]
    b = b[act] / (b[act].sum() / 2.0)          # ~ element counts per molecule
    nz, ns, K = T.size, F.shape[0], F.shape[1]
    c = (net.gibbs_RT(T).T + np.log(P / P0)[:, None])[:, keep]     # [nz, ns]
    ln_n = np.full((nz, ns), np.log(1.0 / ns))
    ln_N = np.zeros(nz)
    size = np.log(1e-8)
    for _ in range(iters):
        n = np.exp(ln_n)
        N = np.exp(ln_N)
        mu = c + ln_n - ln_N[:, None]                             # mu_j / RT
        nF = n[:, :, None] * F[None, :, :]                        # [nz, ns, K]
        M = np.zeros((nz, K + 1, K + 1))
        M[:, :K, :K] = np.einsum('zjk,jl->zkl', nF, F, optimize=True)
        M[:, :K, K] = nF.sum(1)
        M[:, K, :K] = nF.sum(1)
        M[:, K, K] = n.sum(1) - N
        rhs = np.empty((nz, K + 1))
        rhs[:, :K] = b[None, :] - nF.sum(1) + np.einsum('zjk,zj->zk', nF, mu)
        rhs[:, K] = N - n.sum(1) + (n * mu).sum(1)
        sol = np.linalg.solve(M, rhs[:, :, None])[:, :, 0]
        pi, dlnN = sol[:, :K], sol[:, K]
        dln = -mu + pi @ F.T + dlnN[:, None]                      # [nz, ns]
        # damping (Gordon & McBride): major species move at most 2 in ln,
        # minor ones are not pushed above a 1e-4 mole-fraction size ratio
        rel = ln_n - ln_N[:, None]
        major = rel > size
        big = np.maximum(5.0 * np.abs(dlnN), np.max(np.where(major, np.abs(dln), 0.0), axis=1))
        lam1 = 2.0 / np.maximum(big, 1e-300)
        up = (~major) & (dln > 0)
        with np.errstate(divide='ignore', invalid='ignore'):
            l2 = np.abs((-rel - 9.2103) / (dln - dlnN[:, None]))
        lam2 = np.min(np.where(up, l2, np.inf), axis=1)
        lam = np.minimum(1.0, np.minimum(lam1, lam2))
        ln_n = np.maximum(ln_n + lam[:, None] * dln, -700.0)
        ln_N = ln_N + lam * dlnN
        conv = (np.max(np.exp(ln_n) * np.abs(dln), axis=1) / np.exp(ln_n).sum(1) < tol) & \
               (np.abs(dlnN) < tol)
        if conv.all():
            break
    x = np.zeros((nz, Fall.shape[0]))
    x[:, keep] = np.exp(ln_n)
    return x / x.sum(axis=1, keepdims=True)
