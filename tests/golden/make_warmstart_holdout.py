"""Held-out steady states for the learned-warm-start gain test.

Reads the outputs of ``python -m vulcan_gb300.warmstart generate`` that the
committed model was trained on (the same list ``train --data`` takes), takes
the held-out columns exactly as ``train`` does (every tenth of the sorted
column ids of all files), and keeps the first --ncols of them from files
whose features include the equilibrium mixing ratios.  Writes X (features),
Y (log10 steady-state mixing ratios from this package's solver) and the
column ids.

Usage:  python tests/golden/make_warmstart_holdout.py --data a.npz,b.npz
"""
import argparse
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--data', required=True)
    ap.add_argument('--ncols', type=int, default=6)
    ap.add_argument('--n-features', type=int, default=92)
    ap.add_argument('--out', default=os.path.join(HERE, 'warmstart_holdout.npz'))
    a = ap.parse_args()
    parts = [np.load(f) for f in a.data.split(',')]
    cols = np.unique(np.concatenate([d['col'] for d in parts]))
    held = cols[::10]
    X, Y, C = [], [], []
    for d in parts:
        if d['X'].shape[1] != a.n_features:
            continue
        for c in np.unique(d['col'][np.isin(d['col'], held)]):
            if len(C) and len(np.unique(np.concatenate(C))) >= a.ncols:
                break
            r = d['col'] == c
            X.append(d['X'][r]), Y.append(d['Y'][r]), C.append(d['col'][r])
    np.savez_compressed(a.out, X=np.concatenate(X).astype(np.float32),
                        Y=np.concatenate(Y).astype(np.float32), col=np.concatenate(C))
    print('wrote', a.out, len(np.unique(np.concatenate(C))), 'columns')


if __name__ == '__main__':
    main()
