"""Synthetic 150-species stress network (ni = 150, 1200 reversible reactions,
60 frozen photolysis channels, nz = 200): generator checks on the CPU; the
oracle and the device tables' gather form against the reference's own run on
this network (fixture c4s: its code generator, rate set-up and Ros2 attempts);
on the GPU the chemistry and whole Ros2 attempts against the oracle."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, atm_from_column, floor_err, item_floor
from oracle import ros2 as O
from vulcan_gb300 import batch, configs, synthnet
from vulcan_gb300.network import Network

ATOMS = ['H', 'O', 'C', 'He', 'N']


BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), '_build', 'tests')


@pytest.fixture(scope='module')
def syn():
    d = os.path.join(BUILD, 'syn150')
    path = synthnet.generate(d)
    net = Network.from_file(path, use_photo=True)
    npz = os.path.join(str(d), 'net.npz')
    net.to_npz(npz)
    return path, net, npz


def test_sizes_and_element_balance(syn):
    path, net, _ = syn
    assert net.ni == 150
    kinds = [r.kind for r in net.reactions]
    assert kinds.count('photo') == 60
    rev = [r for r in net.reactions if r.kind != 'photo' and r.text != 'He -> He']
    assert len(rev) == 1200
    assert sum(r.kind == 'falloff' for r in rev) == 180
    comp = net.compo_for(ATOMS)
    si = {s: k for k, s in enumerate(net.species)}
    for r in net.reactions:
        a = sum(nu * comp[si[s]] for nu, s in r.reac if s != 'M')
        b = sum(nu * comp[si[s]] for nu, s in r.prod if s != 'M')
        np.testing.assert_array_equal(a, b, err_msg=r.text)


def test_deterministic(syn):
    p2 = synthnet.generate(os.path.join(BUILD, 'syn150_again'))
    assert open(p2).read() == open(syn[0]).read()


def test_compiles_for_device_tables(syn):
    from vulcan_gb300.solver import GPUNetwork
    g = GPUNetwork(syn[1], ATOMS)
    rows, cols = g.jac_pattern()
    assert 150 <= len(rows) <= 150 * 150


def _column(net, nz):
    specs = configs.config4_columns(sorted(net.photo_index()), ncols=2, nz=nz)
    items = batch.build_items(specs, net)
    for sp, it in zip(specs, items):
        pidx = net.photo_index()
        for key in sp.photo_J:
            assert it['k'][pidx[key] - 1].max() > 0
    return specs, items


@pytest.mark.gpu
def test_chem_source_matches_oracle(syn):
    from vulcan_gb300 import _build
    _build.build()
    path, net, npz = syn
    specs, items = _column(net, 40)
    h, b = batch.make_batch_handle(net, items, ATOMS)
    on = O.OracleNet.from_npz(npz, ATOMS)
    rng = np.random.default_rng(0)
    y = np.concatenate([it['y'] * (1 + 0.5 * rng.random(it['y'].shape)) + 1e3 for it in items])
    src = h.chem_source(y)
    for c, it in enumerate(items):
        sl = slice(b.off[c], b.off[c + 1])
        ref = O.chemdf(on, y[sl], it['col'].M, it['k'])
        scale = np.abs(ref).max(axis=1, keepdims=True)
        assert np.max(np.abs(src[sl] - ref) / scale) <= 1e-12
    h.close()


@pytest.mark.gpu
@pytest.mark.parametrize('precision', [0, 1])
def test_attempt_matches_oracle(syn, precision):
    from vulcan_gb300 import _build
    _build.build()
    path, net, npz = syn
    specs, items = _column(net, 30)
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=precision)
    on = O.OracleNet.from_npz(npz, ATOMS)
    for dt in (1e-10, 1e-6):
        sol = h.attempt(np.full(b.ncols, dt))['sol']
        for c, it in enumerate(items):
            sl = slice(b.off[c], b.off[c + 1])
            r, fl = item_floor(on, it, dt)
            # these first attempts from const_mix are rejected steps (delta ~ 1):
            # 1e-10 where the step is well conditioned, else 10x its floor
            assert floor_err(sol[sl], r.sol, it['col'].n_0) <= max(1e-10, 10 * fl), (dt, c, fl)
    h.close()


def _lhs_check(net, items, npz, precision=0):
    from vulcan_gb300.solver import GPUNetwork
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=precision)
    on = O.OracleNet.from_npz(npz, ATOMS)
    h.attempt(np.full(b.ncols, 1e-10))
    jv, dA, dB, dC = h.lhs()
    rows, cols = GPUNetwork(net, ATOMS).jac_pattern()
    it = items[0]
    nz = it['col'].nz
    J = O.neg_jac_blocks(on, it['y'], it['col'].M, it['k'])
    for l in (0, 1, nz // 2, nz - 1):
        ref = J[l][rows, cols]
        assert np.max(np.abs(jv[l] - ref)) <= 1e-13 * np.abs(J[l]).max(), 'layer %d' % l
    A, B, C, Ai, Bi, Ci = O.diff_coeffs(it['y'], atm_from_column(it['col']), O.Flags())
    for got, e, m, sl in ((dA, A, Ai, slice(None)), (dB, B, Bi, slice(0, -1)),
                          (dC, C, Ci, slice(1, None))):
        ref = e[:, None] + m
        mag = np.abs(e[:, None]) + np.abs(m)
        assert np.all(np.abs(got[:nz][sl] - ref[sl]) <= 1e-13 * mag[sl])
    h.close()


@pytest.mark.gpu
def test_lhs_matches_oracle(syn):
    """Sparse -J and transport coefficients of the 150-species network."""
    from vulcan_gb300 import _build
    _build.build()
    path, net, npz = syn
    specs, items = _column(net, 30)
    _lhs_check(net, items[:1], npz)


@pytest.mark.gpu
@pytest.mark.parametrize('precision', [0, 1])
def test_attempt_matches_oracle_ncho_items(precision):
    """The same item -> oracle path on an NCHO-thermo column (ni = 69): the
    seeded set-up (batch.build_items) against the oracle at small dt."""
    from vulcan_gb300 import _build
    _build.build()
    net = Network.from_npz(os.path.join(GOLDEN, 'net_NCHO_thermo.npz'))
    specs = configs.config2_columns(ncols=2, seed=7, nz_range=(40, 60))
    items = batch.build_items(specs, net)
    npz = os.path.join(GOLDEN, 'net_NCHO_thermo.npz')
    on = O.OracleNet.from_npz(npz, ATOMS)
    h, b = batch.make_batch_handle(net, items, ATOMS, precision=precision)
    for dt in (1e-10, 1e-6):
        sol = h.attempt(np.full(b.ncols, dt))['sol']
        for c, it in enumerate(items):
            sl = slice(b.off[c], b.off[c + 1])
            r, fl = item_floor(on, it, dt)
            assert floor_err(sol[sl], r.sol, it['col'].n_0) <= max(1e-10, 10 * fl), (dt, c, fl)
    h.close()


def test_species_missing_from_composition_file_is_named(tmp_path):
    """A network species absent from all_compose.txt stops the set-up with
    its name (the reference fails there too, at compo_row.index)."""
    import shutil
    from vulcan_gb300.network import Network
    src = synthnet.generate(str(tmp_path / 'syn'))
    d = os.path.dirname(src)
    comp = os.path.join(d, 'all_compose.txt')
    lines = open(comp).read().splitlines()
    victim = lines[5].split()[0]
    with open(comp, 'w') as f:
        f.write('\n'.join(ln for ln in lines if ln.split()[:1] != [victim]) + '\n')
    with pytest.raises(ValueError, match=victim):
        Network.from_file(src, use_photo=True)
    shutil.rmtree(d)


# ---- pinned to the reference itself: fixture c4s, recorded by running the
# unmodified reference (its own code generator, rate set-up and Ros2 loop) on
# the generator's files installed into a copy (tests/golden/make_golden.py)

def test_reference_fixture_is_this_generator(syn):
    """The network the reference ran is the one this generator writes: the
    same species in the reference's own order, the same rate slots."""
    from helpers import golden, network
    g = golden('c4s')
    net = network('c4s')
    assert [str(s) for s in g['spec_list']] == list(net.species) == list(syn[1].species)
    assert int(g['nr']) == net.nr == syn[1].nr
    assert [r.text for r in net.reactions] == [r.text for r in syn[1].reactions]


def test_oracle_chemistry_matches_reference_c4s():
    """chemdf bit for bit, -J within 1e-14 of the block scale with the same
    sparsity as the reference's sympy Jacobian (150 species, 2522 rate slots)."""
    from helpers import golden, oracle_net
    g = golden('c4s')
    on = oracle_net('c4s', g)
    np.testing.assert_array_equal(O.chemdf(on, g['y_ini'], g['M'], g['k']), g['chemdf0'])
    J = O.neg_jac_blocks(on, g['y_ini'], g['M'], g['k'])
    for i, l in enumerate(g['negjac_layers']):
        ref = g['negjac_blocks'][i]
        assert np.max(np.abs(J[l] - ref)) <= 1e-14 * np.abs(ref).max()
        assert np.all((J[l] != 0) == (ref != 0))


@pytest.mark.parametrize('n', range(5))
def test_oracle_attempts_match_reference_c4s(n):
    """Recorded Ros2 attempts (accepted and rejected, from const_mix) on the
    150-species network: the banded (the reference's LAPACK solve) and the
    block-Thomas restatements within 1e-10."""
    from helpers import attempt_atm, golden, oracle_net
    g = golden('c4s')
    on = oracle_net('c4s', g)
    args = (on, g['att_y'][n], g['att_ymix'][n], float(g['att_dt'][n]), g['k'],
            attempt_atm(g, n), O.Flags(), O.Tol())
    for solve in ('banded', 'block'):
        r = O.ros2_attempt(*args, solve)
        assert floor_err(r.sol, g['att_sol'][n], g['n_0']) <= 1e-10, solve
        assert abs(r.delta / g['att_delta'][n] - 1) <= 1e-6, solve


def test_gather_form_matches_reference_c4s():
    """The device tables' host evaluation (vk_network_eval_host: the rate
    kernel's gather form, operations and order) on every layer of the
    recorded start: chemdf bit for bit, -J within 1e-14."""
    import ctypes as C
    from helpers import golden, network
    from vulcan_gb300 import _build, capi
    from vulcan_gb300.solver import GPUNetwork
    _build.build()
    g = golden('c4s')
    net = network('c4s')
    gn = GPUNetwork(net, ATOMS)
    rows, cols = gn.jac_pattern()
    lib = capi.lib()
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    for l in range(g['y_ini'].shape[0]):
        y = np.ascontiguousarray(g['y_ini'][l])
        k = np.ascontiguousarray(g['k'][:, l])
        f, jv = np.zeros(net.ni), np.zeros(gn.nnz)
        assert lib.vk_network_eval_host(gn.handle, p(y), p(k), float(g['M'][l]), p(f), p(jv)) == 0
        np.testing.assert_array_equal(f, g['chemdf0'][l])
        if l in g['negjac_layers']:
            ref = g['negjac_blocks'][list(g['negjac_layers']).index(l)]
            J = np.zeros((net.ni, net.ni))
            J[rows, cols] = jv
            assert np.abs(J - ref).max() <= 1e-14 * np.abs(ref).max()
