"""Config 0 at every step: the CHO thermo column (nz = 100) integrated for
500 Ros2 steps from the reference's initial state, every attempt compared.

The oracle (pinned to the reference: its first 150 steps reproduce the
reference's attempt count and dt sequence, tests/test_oracle.py) runs the
whole 500-step loop of the reference -- accept/reject, step size,
update_mu_dz every 100 steps, renormalisation -- and records the inputs of
every attempt (state, step size, the geometry in force).  The device then
solves all of those attempts at once, one column per attempt, and each
result must match the oracle's: 1e-10 in the floor metric (mixing ratios
below 1e-10 absolute) and delta to 1e-6 where dt < 1e-2 s, else 10x the
spread the reference's own banded solve shows when its Jacobian moves at the
rounding level (the conditioning floor, tests/helpers.py).
"""
import numpy as np
import pytest

from helpers import base_atm, column_from_golden, floor_err, golden, network, oracle_net
from oracle import ros2 as O

pytestmark = pytest.mark.gpu

NSTEPS = 500


@pytest.fixture(scope='module')
def attempts():
    """Every attempt of the oracle's 500-step c0 loop: (y, ymix, dt, atm, result)."""
    g = golden('c0')
    on = oracle_net('c0', g)
    atm0 = base_atm(g)
    st = O.ColState(y=g['y_ini'].copy(), ymix=g['ymix_ini'].copy(), dt=1e-10,
                    atom_ini=g['atom_ini'].copy(), atom_loss=np.zeros(len(g['atom_ini'])))
    cur = {'atm': atm0}
    rec = []

    def on_attempt(y, ymix, dt, res):
        rec.append((y.copy(), ymix.copy(), float(dt), cur['atm'], res))

    def on_step(s, atm):
        cur['atm'] = atm

    O.integrate(on, st, g['k'], atm0, O.Flags(), O.Tol(), 2140., 1.138 * 7.1492E9,
                int(g['pref_indx']), max_steps=NSTEPS, solve='banded',
                on_step=on_step, on_attempt=on_attempt)
    assert st.count == NSTEPS
    return g, on, rec


def _floor(on, g, y, ymix, dt, atm, r0, samples=2, eps=4e-16):
    e = d = 0.0
    for seed in range(samples):
        r = O.ros2_attempt(on, y, ymix, dt, g['k'], atm, O.Flags(), O.Tol(), 'banded',
                           perturb=(eps, seed))
        e = max(e, floor_err(r.sol, r0.sol, g['n_0']))
        d = max(d, abs(r.delta / r0.delta - 1) if r0.delta else 0.0)
    return e, d


@pytest.mark.parametrize('precision', [0, 1])
def test_every_attempt_of_500_steps(attempts, precision):
    from vulcan_gb300 import _build
    from vulcan_gb300.solver import ColumnBatch, GPUNetwork, Ros2Handle
    _build.build()
    g, on, rec = attempts
    net = network('c0')
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    items = []
    for y, ymix, dt, atm, _ in rec:
        col = column_from_golden(g)
        col.dzi, col.Hpi = atm['dzi'].copy(), atm['Hpi'].copy()
        col.g, col.Hp = atm['g'].copy(), atm['Hp'].copy()
        items.append(dict(col=col, k=g['k'], y=y, ymix=ymix))
    b = ColumnBatch(items, net.ni)
    h = Ros2Handle(gn, len(items), b.L, precision)
    h.set_columns(b)
    out = h.attempt(np.array([r[2] for r in rec]))
    sols = b.split(out['sol'])
    h.close()
    worst = 0.0
    for n, (y, ymix, dt, atm, r0) in enumerate(rec):
        tol_s, tol_d = 1e-10, 1e-6
        if dt >= 1e-2:
            e_f, d_f = _floor(on, g, y, ymix, dt, atm, r0)
            tol_s, tol_d = max(tol_s, 10 * e_f), max(tol_d, 10 * d_f)
        e = floor_err(sols[n], r0.sol, g['n_0'])
        worst = max(worst, e)
        assert e <= tol_s, (n, dt, e, tol_s)
        if r0.delta:
            assert abs(out['delta'][n] / r0.delta - 1) <= tol_d, (n, dt)
    print('c0, %d attempts over %d steps: worst floor-metric error %.2e' % (len(rec), NSTEPS, worst))
