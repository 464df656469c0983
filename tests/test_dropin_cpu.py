"""Drop-in host logic that needs no GPU: which reference options Ros2GPU
refuses (loudly, before any device work) and which it accepts."""
import types

import pytest

from vulcan_gb300.solver import _unsupported, make_ros2gpu


def _cfg(**kw):
    base = dict(network=None, use_photo=False, atom_list=['H', 'O', 'C', 'He'],
                use_moldiff=True, use_topflux=False, use_botflux=False, diff_esc=['H'],
                use_fix_sp_bot={}, non_gas_sp=[])
    base.update(kw)
    return types.SimpleNamespace(**base)


def test_reference_defaults_accepted():
    """The reference's vulcan_cfg defaults (molecular diffusion, H escape
    through the top flux) and the flux options run on the device."""
    assert _unsupported(_cfg()) == []
    assert _unsupported(_cfg(use_topflux=True, use_botflux=True)) == []
    assert _unsupported(_cfg(use_moldiff=False, diff_esc=[])) == []


@pytest.mark.parametrize('kw,name', [
    (dict(use_condense=True), 'use_condense'),
    (dict(use_settling=True), 'use_settling'),
    (dict(use_ion=True), 'use_ion'),
    (dict(use_vm_mol=True), 'use_vm_mol'),
    (dict(use_fix_sp_bot={'H2O': 1e-3}), 'use_fix_sp_bot'),
    (dict(use_fix_H2He=True), 'use_fix_H2He'),
    (dict(non_gas_sp=['H2O_l_s']), 'non_gas_sp'),
    (dict(use_moldiff=False), 'diff_esc with use_moldiff = False'),
])
def test_unimplemented_options_raise(kw, name):
    cfg = _cfg(**kw)
    assert name in _unsupported(cfg)

    class FakeRos2:
        pass

    cls = make_ros2gpu(types.SimpleNamespace(Ros2=FakeRos2), cfg, ['H', 'H2'])
    var = types.SimpleNamespace(y=None)
    with pytest.raises(NotImplementedError, match=name.split()[0]):
        cls().solver(var, None, None)


def test_dropin_packs_transport_options():
    """Ros2GPU hands the reference's atm fluxes, deposition velocities and
    vz to the device and turns use_moldiff / use_topflux / use_botflux into
    the attempt flags (host side of fixtures c0bc and c0vz)."""
    import numpy as np
    from helpers import column_from_golden, golden, network
    from vulcan_gb300 import capi
    from vulcan_gb300.solver import GPUNetwork, _flags_from_cfg
    for tag in ('c0bc', 'c0vz'):
        g = golden(tag)
        net = network(tag)
        cfg = _cfg(use_topflux=bool(g['use_topflux']), use_botflux=bool(g['use_botflux']),
                   atom_list=[str(a) for a in g['atom_list']])
        f = _flags_from_cfg(cfg)
        assert f & capi.VK_F_MOLDIFF
        assert bool(f & capi.VK_F_TOPFLUX) == bool(g['use_topflux'])
        assert bool(f & capi.VK_F_BOTFLUX) == bool(g['use_botflux'])

        class FakeRos2:
            pass

        cls = make_ros2gpu(types.SimpleNamespace(Ros2=FakeRos2), cfg, net.species)
        s = cls()
        s._vk_gnet = GPUNetwork(net, cfg.atom_list)       # host-side tables only
        col = column_from_golden(g, 1)
        col.top_flux = g['att_top_flux'][1].copy()
        col.bot_flux, col.bot_vdep = g['bot_flux'].copy(), g['bot_vdep'].copy()
        atm = types.SimpleNamespace(**{k: getattr(col, k) for k in (
            'M', 'n_0', 'Tco', 'g', 'dzi', 'Kzz', 'vz', 'Ti', 'Hpi', 'Hp', 'pico', 'dz', 'Dzz',
            'ms', 'alpha', 'top_flux', 'bot_flux', 'bot_vdep', 'pref_indx')})
        var = types.SimpleNamespace(y=g['att_y'][1], ymix=g['att_ymix'][1],
                                    k={i: g['k'][i - 1] for i in range(1, net.nr + 1)})
        b = s._vk_pack(var, atm)
        np.testing.assert_array_equal(b.spf[0, capi.SP_TOPFLUX], col.top_flux)
        np.testing.assert_array_equal(b.spf[0, capi.SP_BOTFLUX], col.bot_flux)
        np.testing.assert_array_equal(b.spf[0, capi.SP_BOTVDEP], col.bot_vdep)
        np.testing.assert_array_equal(b.atm[:-1, capi.ATM_VZ], g['vz'])
        np.testing.assert_array_equal(b.k, g['k'].T)


def test_batch_api_takes_the_transport_and_setup_options():
    """ColumnSpec's top / bottom fluxes, deposition velocities, vz, base gas
    and rocky flag reach the batch arrays, and run_batch's cfg turns
    use_moldiff / use_topflux / use_botflux into the run's flags."""
    import dataclasses
    import numpy as np
    from helpers import golden, network
    from vulcan_gb300 import batch, capi, configs
    from vulcan_gb300.solver import ColumnBatch, ctrl_from
    net = network('c0')
    g = golden('c0bc')
    sp = configs.config0()
    vz = 100.0 * np.cos(np.linspace(0, np.pi, sp.pco.size - 1))
    sp = dataclasses.replace(sp, top_flux={'CO2': 1e12, 'H2O': 4e11},
                             bot_flux={'CH4': (1e14, 0.0), 'CO': (0.0, 1e-2), 'H2O': (2e14, 1e-3)},
                             vz=vz, atm_base='N2')
    it = batch.build_items([sp], net)[0]
    b = ColumnBatch([it], net.ni)
    i = net.species.index
    assert b.spf[0, capi.SP_TOPFLUX, i('CO2')] == 1e12
    assert b.spf[0, capi.SP_BOTVDEP, i('CO')] == 1e-2 and b.spf[0, capi.SP_BOTFLUX, i('H2O')] == 2e14
    # the same boundary arrays as the reference's BC_flux read from the same values
    np.testing.assert_array_equal(b.spf[0, capi.SP_TOPFLUX], g['top_flux'])
    np.testing.assert_array_equal(b.spf[0, capi.SP_BOTFLUX], g['bot_flux'])
    np.testing.assert_array_equal(b.spf[0, capi.SP_BOTVDEP], g['bot_vdep'])
    np.testing.assert_array_equal(b.atm[:-1, capi.ATM_VZ], vz)
    assert it['col'].atm_base == 'N2'
    assert ctrl_from(None).flags == capi.VK_F_MOLDIFF
    assert ctrl_from({'use_topflux': True, 'use_botflux': True}).flags == \
        capi.VK_F_MOLDIFF | capi.VK_F_TOPFLUX | capi.VK_F_BOTFLUX
    assert ctrl_from(types.SimpleNamespace(use_moldiff=False)).flags == 0
    assert ctrl_from({'rtol': 0.1}, flags=capi.VK_F_BOTFLUX).flags == capi.VK_F_BOTFLUX
