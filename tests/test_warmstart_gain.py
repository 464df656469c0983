"""What the trained warm-start network gains over the starts without it, on
steady states it was not trained on (tests/golden/warmstart_holdout.npz:
held-out columns of the committed model's training set, steady states from
this package's solver): its proposal against the thermochemical-equilibrium
start and the reference's const_mix start, in dex of the steady-state mixing
ratios above 1e-10.  The run-level gain (steps and columns per hour to the
reference's convergence test) is measured by ``bench.py --converge``."""
import os

import numpy as np

from conftest import GOLDEN, REPO

WEIGHTS = os.path.join(REPO, 'vulcan_gb300', 'warmstart_weights.npz')
N_BASE = 23


def _forward(w, X):
    """FP32/FP64 restatement of the network (SiLU hidden layers, standardised
    inputs and outputs) -- the device runs it in BF16 with FP32 accumulation."""
    dims = [int(v) for v in w['dims']]
    h = (X - w['x_mean']) / w['x_std']
    nl = len(dims) - 1
    for layer in range(nl):
        z = h @ w['W%d' % layer] + w['b%d' % layer]
        h = z / (1.0 + np.exp(-z)) if layer < nl - 1 else z
    return h * w['y_std'] + w['y_mean']


def _data():
    d = np.load(os.path.join(GOLDEN, 'warmstart_holdout.npz'))
    return d['X'].astype(float), d['Y'].astype(float), d['col']


def _const_mix_log(col_ids, ni):
    """log10 mixing ratios of the const_mix start of each held-out column
    (seeded config-2 columns; id = seed * 100000 + index)."""
    from vulcan_gb300 import configs
    from helpers import network
    net = network('c2')
    out = []
    for c in col_ids:
        seed, idx = divmod(int(c), 100000)
        spec = configs.config2_columns(ncols=512, seed=seed)[idx]
        x0 = np.zeros(ni)
        for sp, v in spec.const_mix.items():
            x0[net.species.index(sp)] = v
        out.append(np.log10(np.clip(x0 / x0.sum(), 1e-30, None)))
    return np.array(out)


def _errors(P, X, Y, col):
    m = Y > -10
    e_mlp = float(np.abs(P - Y)[m].mean())
    e_eq = float(np.abs(X[:, N_BASE:] - Y)[m].mean())
    cm = _const_mix_log(np.unique(col), Y.shape[1])
    idx = np.searchsorted(np.unique(col), col)
    e_cm = float(np.abs(cm[idx] - Y)[m].mean())
    return e_mlp, e_eq, e_cm


def test_network_beats_equilibrium_and_const_mix_starts():
    w = np.load(WEIGHTS)
    X, Y, col = _data()
    assert X.shape[1] == int(w['dims'][0]) and len(np.unique(col)) >= 6
    e_mlp, e_eq, e_cm = _errors(_forward(w, X), X, Y, col)
    # measured: 0.09 dex against 2.5 (equilibrium) and 13 (const_mix)
    assert e_mlp < 0.2
    assert e_mlp < 0.3 * e_eq < e_cm
    # and column by column
    for c in np.unique(col):
        r = col == c
        a, b, _ = _errors(_forward(w, X[r]), X[r], Y[r], col[r])
        assert a < b, c
