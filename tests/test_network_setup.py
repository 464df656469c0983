"""Network compiler, rate constants and column set-up vs the reference's own values."""
import numpy as np
import pytest

from helpers import column_from_golden, golden, network
from vulcan_gb300 import column as C
from vulcan_gb300 import configs

# Ros2-attempt fixtures on five more shipped networks (CHO photo, the full
# NCHO and SNCHO networks, the Jupiter network with condensation species,
# TiSNCHO), recorded from the reference with seeded J
A_TAGS = ['a_CHO_photo', 'a_NCHO_full_photo', 'a_NCHO_photo_lowT_Jupiter', 'a_SNCHO_full_photo',
          'a_TiSNCHO_photo']


@pytest.mark.parametrize('tag', ['c0', 'c1', 'c2'] + A_TAGS)
def test_species_order_and_nr(tag):
    g = golden(tag)
    net = network(tag)
    assert net.species == [str(s) for s in g['spec_list']]
    assert net.nr == int(g['nr'])


@pytest.mark.parametrize('tag', ['c0', 'c1', 'c2'] + A_TAGS)
def test_rate_constants_bit_exact(tag):
    """k (forward Arrhenius / fall-off / special, reverse via NASA-9 Gibbs)."""
    g = golden(tag)
    net = network(tag)
    with np.errstate(over='ignore'):
        k = net.rate_constants(g['Tco'], g['M'])
    if 'photo_sp' in g:
        pidx = net.photo_index()
        for sp, br in zip(g['photo_sp'], g['photo_br']):
            i = pidx[(str(sp), int(br))]
            assert np.all(k[i - 1] == 0)           # placeholder before J is injected
            k[i - 1] = g['k'][i - 1]
    np.testing.assert_array_equal(k, g['k'])


@pytest.mark.parametrize('tag', ['c0', 'c2', 'c0n2', 'c0o2', 'c0co2', 'c0rocky', 'c0nomol'] + A_TAGS)
def test_column_setup_bit_exact(tag):
    """pico, M, n_0, mu, g, Hp, dz, dzi, Ti, Hpi, Dzz, ms, alpha as the
    reference's f_pico / f_mu_dz / mol_diff built them, for the H2 base gas
    and the N2, O2 and CO2 ones (c0n2, c0o2, c0co2), a rocky surface, and
    without molecular diffusion (no interface T or Hp then)."""
    g = golden(tag)
    net = network(tag)
    base = str(g.get('atm_base', 'H2'))
    rocky = bool(g.get('rocky', False))
    mol = bool(g.get('use_moldiff', True))
    col = C.build_column(net, g['pco'], g['Tco'], g['Kzz'], gs=configs.GS, Rp=configs.RP,
                         rocky=rocky, atm_base=base, use_moldiff=mol, ymix0=g['ymix_ini'])
    assert col.pref_indx == int(g['pref_indx'])
    for key in ('pico', 'M', 'n_0', 'mu', 'g', 'Hp', 'dz', 'dzi', 'Ti', 'Hpi', 'Dzz', 'ms', 'alpha'):
        if not mol and key in ('Ti', 'Hpi'):
            assert getattr(col, key) is None and not np.any(g[key])
            continue
        np.testing.assert_array_equal(getattr(col, key), g[key], err_msg=key)


def test_initial_state_and_atoms():
    g = golden('c0')
    net = network('c0')
    mix = dict(zip([str(s) for s in g['const_mix_sp']], g['const_mix_x']))
    y, ymix = C.const_mix_state(net, g['n_0'], mix)
    np.testing.assert_array_equal(y, g['y_ini'])
    np.testing.assert_allclose(ymix, g['ymix_ini'], rtol=1e-15, atol=0)
    at = C.atom_totals(net, y, [str(a) for a in g['atom_list']])
    np.testing.assert_allclose(at, g['atom_ini'], rtol=1e-14)


def test_config_generators_match_fixture_inputs():
    g = golden('c0')
    spec = configs.config0()
    np.testing.assert_array_equal(spec.Tco, g['Tco'])
    np.testing.assert_array_equal(spec.Kzz, g['Kzz'])


def test_pair_tables():
    net = network('c0')
    t = net.pair_tables()
    assert t['fwd_ptr'].size == net.npair + 1
    # 'H + H + M -> H2 + M' merges to H^2 with one M on each side
    p = [r.text for r in net.reactions].index('H + H + M -> H2 + M')
    h = net.species.index('H')
    f0, f1 = t['fwd_ptr'][p], t['fwd_ptr'][p + 1]
    assert list(t['fwd_sp'][f0:f1]) == [h] and list(t['fwd_nu'][f0:f1]) == [2]
    assert t['fwd_m'][p] == 1 and t['rev_m'][p] == 1


def test_network_roundtrip(tmp_path):
    net = network('c1')
    path = tmp_path / 'n.npz'
    net.to_npz(path)
    n2 = type(net).from_npz(path)
    assert n2.species == net.species
    assert [r.text for r in n2.reactions] == [r.text for r in net.reactions]
    T = np.linspace(500, 3000, 7)
    np.testing.assert_array_equal(n2.rate_constants(T, T * 1e15), net.rate_constants(T, T * 1e15))


def test_column_helper_consistent():
    g = golden('c0')
    col = column_from_golden(g)
    assert col.nz == g['pco'].size


def test_low_temperature_caps_bit_exact():
    """use_lowT_limit_rates: the reference's read_rate, lim_lowT_rates,
    rev_rate on a 150-450 K column (fixture lowT); the three capped forward
    rates and their reverses, every other rate unchanged."""
    g = golden('lowT')
    net = network('c2')
    k = net.rate_constants(g['Tco'], g['M'], use_lowT_limit_rates=True)
    np.testing.assert_array_equal(k, g['k'])
    plain = net.rate_constants(g['Tco'], g['M'])
    np.testing.assert_array_equal(plain[0::2], g['k_plain'])
    capped = np.nonzero(np.any(k != plain, axis=1))[0]
    texts = {net.reactions[p].text for p in set(capped // 2)}
    assert texts == {'H + CH3 + M -> CH4 + M', 'H + C2H4 + M -> C2H5 + M',
                     'H + C2H5 + M -> C2H6 + M'}
    kind, t_max, params = net.rate_caps()
    assert int((kind > 0).sum()) == 3 and set(t_max[kind > 0]) == {277.5, 300., 200.}


def test_remove_list_bit_exact():
    """remove_list = [5, 12, 101] (two forward rates, one reverse rate): the
    reference's rev_rate / remove_rate zero exactly those slots; a removed
    forward rate keeps its reverse (fixture rmlist)."""
    g = golden('rmlist')
    net = network('c2')
    k = net.rate_constants(g['Tco'], g['M'], remove_list=[5, 12, 101])
    np.testing.assert_array_equal(k, g['k'])
    for i in (5, 12, 101):
        assert np.all(k[i - 1] == 0)
    assert np.all(k[5] > 0) and np.all(k[101] > 0)    # reverses of 5 and 101


def test_sulfur_network_rate_constants_bit_exact():
    """The SNCHO photochemical network (89 species, 1 150 rate slots): the
    reference's read_rate / lim_lowT_rates / rev_rate on a 40-layer column
    (fixture snchok); photolysis slots are zero placeholders in both until J
    is computed."""
    import os
    from conftest import GOLDEN
    from vulcan_gb300.network import Network
    g = golden('snchok')
    net = Network.from_npz(os.path.join(GOLDEN, 'net_SNCHO_photo.npz'))
    assert net.ni == 89 and net.nr == 1150
    k = net.rate_constants(g['Tco'], g['M'], use_lowT_limit_rates=True)
    np.testing.assert_array_equal(k, g['k'])


def test_sulfur_network_chemical_source_bit_exact():
    """The oracle's chemistry source on the sulfur network equals the
    reference's generated chemdf at a seeded positive state (fixture snchok)."""
    import os
    from conftest import GOLDEN
    from oracle import ros2 as O
    g = golden('snchok')
    on = O.OracleNet.from_npz(os.path.join(GOLDEN, 'net_SNCHO_photo.npz'),
                              ['H', 'O', 'C', 'He', 'N', 'S'])
    np.testing.assert_array_equal(O.chemdf(on, g['y_rand'], g['M'], g['k']), g['chemdf_rand'])


def test_sulfur_network_jacobian_blocks():
    """The oracle's chemistry Jacobian on the sulfur network against the
    reference's sympy-generated neg_symjac at the same state: the same
    sparsity, values within 1e-14 of the block scale (fixture snchok)."""
    import os
    from conftest import GOLDEN
    from oracle import ros2 as O
    g = golden('snchok')
    on = O.OracleNet.from_npz(os.path.join(GOLDEN, 'net_SNCHO_photo.npz'),
                              ['H', 'O', 'C', 'He', 'N', 'S'])
    J = O.neg_jac_blocks(on, g['y_rand'], g['M'], g['k'])
    for i, l in enumerate(g['negjac_layers']):
        ref = g['negjac_blocks'][i]
        assert np.max(np.abs(J[l] - ref)) <= 1e-14 * np.abs(ref).max()
        assert np.all((J[l] != 0) == (ref != 0))
