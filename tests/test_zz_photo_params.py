"""The device radiative transfer on other parameters (fixture c1rtA: zenith
angle 60 deg, Eddington coefficient 0.669, f_diurnal 0.5, 2 nm bins, the bin
switch beyond the bins so that J sums with index -1): against the oracle and,
through the drop-in, against the reference's records.  Tolerances as for the
drop-in on c1rt (actinic flux 1e-10: the deep layers' flux is exp(-tau/mu)
of a large optical depth)."""
import numpy as np
import pytest

from test_photo import _attach, _dropin, _fixture, _oracle_call, _rel

pytestmark = pytest.mark.gpu


def test_device_matches_oracle_on_other_parameters():
    from test_gpu_parity import make_handle
    from vulcan_gb300 import _build
    _build.build()
    d = _fixture('c1rtA')
    assert int(d['sflux_din12_indx']) == -1
    g, net, gn, h, b = make_handle('c1')
    np.testing.assert_array_equal(g['Tco'], d['Tco'])
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
            np.testing.assert_allclose(k[:, int(ki) - 1], 0.5 * J_d[:, c], rtol=1e-15)
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
