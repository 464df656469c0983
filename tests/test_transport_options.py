"""Device attempts with the reference's transport options against the
attempts it recorded: constant top and bottom fluxes with deposition
velocities and H escape through the top flux, with molecular diffusion
(fixture c0bc) and without it (c0nomol), and vertical advection changing sign
with height (c0vz).  The oracle reproduces the same fixtures
(tests/test_oracle.py)."""
import pytest

from helpers import column_from_golden, floor_err, golden, network

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


@pytest.mark.parametrize('precision', [0, 1])
@pytest.mark.parametrize('tag', ['c0bc', 'c0nomol', 'c0vz'])
def test_attempts_with_transport_options(tag, precision):
    from vulcan_gb300 import capi
    from vulcan_gb300.solver import ColumnBatch, GPUNetwork, Ros2Handle
    g = golden(tag)
    net = network(tag)
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    flags = 0
    for key, bit in (('use_moldiff', capi.VK_F_MOLDIFF), ('use_topflux', capi.VK_F_TOPFLUX),
                     ('use_botflux', capi.VK_F_BOTFLUX)):
        if bool(g[key]):
            flags |= bit
    items = []
    for n in range(len(g['att_index'])):
        col = column_from_golden(g, n)
        col.top_flux = g['att_top_flux'][n].copy()
        col.bot_flux, col.bot_vdep = g['bot_flux'].copy(), g['bot_vdep'].copy()
        items.append(dict(col=col, k=g['k'], y=g['att_y'][n], ymix=g['att_ymix'][n]))
    b = ColumnBatch(items, net.ni)
    h = Ros2Handle(gn, len(items), b.L, precision)
    h.set_columns(b)
    out = h.attempt(g['att_dt'], flags)
    sols = b.split(out['sol'])
    for n in range(len(items)):
        assert floor_err(sols[n], g['att_sol'][n], g['n_0']) <= 1e-10, n
        assert abs(out['delta'][n] / g['att_delta'][n] - 1) <= 1e-6, n
    h.close()
