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
