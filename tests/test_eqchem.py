"""Thermochemical equilibrium (Gibbs minimisation with the network's NASA-9
data): element balance, normalisation, and the textbook limits."""
import numpy as np

from helpers import network
from vulcan_gb300 import configs, eqchem

ATOMS = ['H', 'O', 'C', 'He', 'N']


def _abund(net, met=1.0, c_to_o=None):
    mix = configs.solar_mix(met=met, c_to_o=c_to_o, with_n=True)
    x0 = np.zeros(net.ni)
    for sp, v in mix.items():
        x0[net.species.index(sp)] = v
    return x0 @ net.compo_for(ATOMS)


def test_element_ratios_and_normalisation():
    net = network('c2')
    comp = net.compo_for(ATOMS)
    for met, co in ((1.0, None), (100.0, 1.2), (0.1, 0.3)):
        b = _abund(net, met, co)
        T = np.linspace(500, 3000, 30)
        P = np.logspace(9, 0, 30)
        x = eqchem.equilibrium(net, T, P, b, ATOMS)
        np.testing.assert_allclose(x.sum(axis=1), 1.0, rtol=1e-12)
        el = x @ comp
        np.testing.assert_allclose(el / el[:, :1], np.broadcast_to(b / b[0], el.shape), rtol=1e-8)


def test_textbook_limits():
    """Cool and dense: CH4, H2O, NH3 carry C, O, N; hot and thin: atomic H."""
    net = network('c2')
    sp = net.species.index
    x = eqchem.equilibrium(net, [500.0, 3000.0], [1e9, 1e0], _abund(net), ATOMS)
    assert x[0, sp('CH4')] > 100 * x[0, sp('CO')]
    assert x[0, sp('NH3')] > x[0, sp('N2')]
    assert x[0, sp('H2')] > 0.8
    assert x[1, sp('H')] > 10 * x[1, sp('H2')]
    assert x[1, sp('CO')] > 100 * x[1, sp('CH4')]


def test_minimises_gibbs_energy():
    """Random feasible perturbations (element-conserving) raise G."""
    net = network('c2')
    comp = net.compo_for(ATOMS)
    T, P = np.array([1500.0]), np.array([1e6])
    x = eqchem.equilibrium(net, T, P, _abund(net), ATOMS)[0]
    c = net.gibbs_RT(T)[:, 0] + np.log(P[0] / eqchem.P0)

    def G(n):
        m = n > 0
        return float(np.sum(n[m] * (c[m] + np.log(n[m] / n.sum()))))

    rng = np.random.default_rng(0)
    big = np.nonzero(x > 1e-12)[0]
    # element-conserving directions among the non-trace species
    _, sv, vt = np.linalg.svd(comp[big].T)
    null = vt[np.sum(sv > 1e-10):]
    g0 = G(x)
    for _ in range(20):
        d = np.zeros_like(x)
        d[big] = null.T @ rng.normal(size=null.shape[0])
        step = 1e-3 * np.min(x[big] / (np.abs(d[big]) + 1e-300))
        assert G(x + step * d) >= g0 - 1e-12 * abs(g0)


def test_matches_the_reference_fastchem():
    """The equilibrium start against the reference's own FastChem (fixture
    golden_eq: five columns of the 512-column workload, FastChem built from
    the reference's sources and run the way its ini_fc runs it, with the
    same NASA-9 data): every network species above 1e-10 within 1e-3 dex
    (FastChem iterates to 1e-4 relative) -- except the two FastChem lists
    twice (CH2_1, C4H2: two data sets under one name, both present in its
    equilibrium, where the network has one)."""
    import os
    from conftest import GOLDEN
    from helpers import network
    from vulcan_gb300 import eqchem
    g = np.load(os.path.join(GOLDEN, 'golden_eq.npz'))
    net = network('c2')
    atoms = [str(a) for a in g['atoms']]
    assert g['have'].all()
    worst = 0.0
    for c in g['columns']:
        ref = g['x_%d' % c]
        x = eqchem.equilibrium(net, g['tco_%d' % c], g['pco_%d' % c], g['abund_%d' % c], atoms)
        m = (ref > 1e-10) & ~g['dup'][None, :]
        err = np.abs(np.log10(np.maximum(x[m], 1e-300)) - np.log10(ref[m]))
        worst = max(worst, float(err.max()))
    assert worst < 1e-3, worst
    assert sorted(net.species[i] for i in np.nonzero(g['dup'])[0]) == ['C4H2', 'CH2_1']
