"""The device radiative transfer on other parameters and networks (c1rtA: zenith
angle 60 deg, Eddington coefficient 0.669, f_diurnal 0.5, 2 nm bins, the bin
switch beyond the bins so that J sums with index -1; c3rt: the sulfur
network): against the oracle and, for c1rtA,
through the drop-in, against the reference's records.  Tolerances as for the
drop-in on c1rt (actinic flux 1e-10: the deep layers' flux is exp(-tau/mu)
of a large optical depth)."""
import numpy as np
import pytest

from test_photo import _attach, _dropin, _fixture, _oracle_call, _rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('tag,column', [('c1rtA', 'c1'), ('c3rt', 'c3s')])
def test_device_matches_oracle_on_other_parameters(tag, column):
    """c1rtA on the NCHO column; c3rt: the 89-species sulfur network's
    radiative transfer (37 absorbers, 60 channels) on the c3s column."""
    from test_gpu_parity import make_handle
    from vulcan_gb300 import _build
    _build.build()
    d = _fixture(tag)
    g, net, gn, h, b = make_handle(column)
    np.testing.assert_array_equal(g['Tco'], d['Tco'])
    np.testing.assert_allclose(g['dz'], d['rec0_dz'], rtol=1e-14)
    _attach(h, d, net)
    nz, nb = d['rec0_y'].shape[0], len(d['bins'])
    du, dd = np.zeros((nz + 1, nb)), np.zeros((nz + 1, nb))
    prev = None
    for rec in range(2):
        h.set_state(d['rec0_y'], d['rec0_ymix'])
        change = h.photo_update()
        tau_d, af_d, J_d = h.photo_get()
        tau, af, J, ch = _oracle_call(d, d['rec0_y'], d['rec0_ymix'], d['rec0_dz'], du, dd, prev)
        prev = af
        assert _rel(tau_d[:nz + 1], tau) < 1e-13
        assert _rel(af_d, af, 1e-30) < 1e-10
        assert _rel(J_d.T, J) < 1e-10
        if rec:
            assert abs(change[0] / ch - 1) < 1e-9
        k = h.k()
        for c, ki in enumerate(d['ch_kindex']):
            np.testing.assert_allclose(k[:, int(ki) - 1], float(d['f_diurnal']) * J_d[:, c],
                                       rtol=1e-15)
    h.close()


def test_dropin_matches_reference_on_other_parameters():
    from helpers import golden, network
    from vulcan_gb300 import _build
    _build.build()
    d = _fixture('c1rtA')
    s, var, atm, chans, calls = _dropin(d, network('c1'), golden('c1'))
    for rec in ('rec0', 'rec1'):
        for f in (s.compute_tau, s.compute_flux, s.compute_J):
            f(var, atm)
        assert _rel(var.aflux, d[rec + '_aflux'], 1e-30) < 1e-10
        J = np.array([var.J_sp[c] for c in chans])
        assert _rel(J, d[rec + '_J']) < 1e-10
        for c, ki in var.pho_rate_index.items():
            np.testing.assert_array_equal(var.k[ki], var.J_sp[c] * 0.5)
    assert abs(var.aflux_change / float(d['rec1_aflux_change']) - 1) < 1e-9
    assert calls == []
    s._vk_h.close()
