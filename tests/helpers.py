"""Shared helpers: golden fixtures -> oracle inputs and GPU column batches."""
import os

import numpy as np

from conftest import GOLDEN
from oracle import ros2 as O
from vulcan_gb300 import column as C
from vulcan_gb300 import configs
from vulcan_gb300.network import Network

NETS = {'c0': 'net_CHO_thermo.npz', 'c1': 'net_NCHO_photo.npz', 'c2': 'net_NCHO_thermo.npz',
        'c2long': 'net_NCHO_thermo.npz', 'c2conv': 'net_NCHO_thermo.npz',
        'c2tight': 'net_NCHO_thermo.npz', 'c2slow': 'net_NCHO_thermo.npz',
        'c0bc': 'net_CHO_thermo.npz', 'c0nomol': 'net_CHO_thermo.npz',
        'c0vz': 'net_CHO_thermo.npz', 'c0n2': 'net_CHO_thermo.npz',
        'c0o2': 'net_CHO_thermo.npz', 'c0co2': 'net_CHO_thermo.npz',
        'c0rocky': 'net_CHO_thermo.npz', 'c3s': 'net_SNCHO_photo.npz',
        'c4s': 'net_SYN150_photo.npz',
        'a_CHO_photo': 'net_CHO_photo.npz', 'a_NCHO_full_photo': 'net_NCHO_full_photo.npz',
        'a_NCHO_photo_lowT_Jupiter': 'net_NCHO_photo_lowT_Jupiter.npz',
        'a_SNCHO_full_photo': 'net_SNCHO_full_photo.npz', 'a_TiSNCHO_photo': 'net_TiSNCHO_photo.npz'}


def golden(tag):
    return dict(np.load(os.path.join(GOLDEN, 'golden_%s.npz' % tag), allow_pickle=False))


def network(tag):
    return Network.from_npz(os.path.join(GOLDEN, NETS[tag]))


def oracle_net(tag, g):
    return O.OracleNet.from_npz(os.path.join(GOLDEN, NETS[tag]), [str(a) for a in g['atom_list']])


def base_atm(g):
    ni = g['ms'].size
    return dict(M=g['M'], n_0=g['n_0'], Tco=g['Tco'], Kzz=g['Kzz'], vz=g['vz'], Dzz=g['Dzz'],
                Ti=g['Ti'], ms=g['ms'], alpha=g['alpha'], pico=g['pico'], dzi=g['dzi'],
                Hpi=g['Hpi'], g=g['g'], Hp=g['Hp'], dz=g['dz'], zco=g['zco'],
                top_flux=g.get('top_flux', np.zeros(ni)), bot_flux=g.get('bot_flux', np.zeros(ni)),
                bot_vdep=g.get('bot_vdep', np.zeros(ni)))


def attempt_atm(g, n):
    a = dict(base_atm(g), dzi=g['att_dzi'][n], Hpi=g['att_Hpi'][n], g=g['att_g'][n],
             Hp=g['att_Hp'][n])
    if 'att_top_flux' in g:           # diffusion-limited escape updates the top fluxes
        a['top_flux'] = g['att_top_flux'][n]
    return a


def fixture_flags(g):
    """Transport options a fixture was recorded with (the reference's
    defaults where the fixture predates the keys)."""
    return O.Flags(use_moldiff=bool(g.get('use_moldiff', True)),
                   use_topflux=bool(g.get('use_topflux', False)),
                   use_botflux=bool(g.get('use_botflux', False)))


def column_from_golden(g, n=None):
    """column.Column with the reference's set-up arrays (attempt n's dynamic ones)."""
    net_ymix = g['ymix_ini']
    col = C.Column(pco=g['pco'], Tco=g['Tco'], Kzz=g['Kzz'], vz=g['vz'], gs=configs.GS,
                   Rp=configs.RP, rocky=False, use_moldiff=True)
    col.pico, col.M, col.n_0 = g['pico'], g['M'], g['n_0']
    col.g, col.Hp, col.dz, col.zco = g['g'].copy(), g['Hp'].copy(), g['dz'].copy(), g['zco'].copy()
    col.dzi, col.Ti, col.Hpi = g['dzi'].copy(), g['Ti'], g['Hpi'].copy()
    col.Dzz, col.ms, col.alpha = g['Dzz'], g['ms'], g['alpha']
    col.pref_indx = int(g['pref_indx'])
    ni = g['ms'].size
    col.top_flux, col.bot_flux, col.bot_vdep = np.zeros(ni), np.zeros(ni), np.zeros(ni)
    if n is not None:
        col.dzi, col.Hpi = g['att_dzi'][n].copy(), g['att_Hpi'][n].copy()
        col.g, col.Hp = g['att_g'][n].copy(), g['att_Hp'][n].copy()
    del net_ymix
    return col


def floor_err(a, b, n0, floor=1e-10):
    """max |a-b| / (|b| + floor * n_0): relative error with a mixing-ratio floor."""
    return float(np.max(np.abs(a - b) / (np.abs(b) + floor * n0[:, None])))


def reference_floor(tag, g, n, samples=3, eps=4e-16):
    """Conditioning floor of one recorded attempt: how far the reference's own
    algorithm (LAPACK banded solve) moves when its Jacobian changes at the
    rounding level -- the analytic Jacobian, and that Jacobian with every
    entry scaled by (1 + eps u), u ~ U(-1,1), for a few seeds.  Returns the
    largest (floor-metric error of sol, relative error of delta) vs the
    recorded reference attempt."""
    on = oracle_net(tag, g)
    args = (on, g['att_y'][n], g['att_ymix'][n], float(g['att_dt'][n]), g['k'],
            attempt_atm(g, n), O.Flags(), O.Tol(), 'banded')
    e = d = 0.0
    for s in [None] + [(eps, seed) for seed in range(samples)]:
        r = O.ros2_attempt(*args, perturb=s)
        e = max(e, floor_err(r.sol, g['att_sol'][n], g['n_0']))
        d = max(d, abs(r.delta / g['att_delta'][n] - 1))
    return e, d


def step_tolerance(e_floor, d_floor):
    """Per-attempt tolerances: 1e-10 (floor metric) and 1e-6 (delta) where the
    step is well conditioned, else 10x the reference's own conditioning floor."""
    return max(1e-10, 10 * e_floor), max(1e-6, 10 * d_floor)


def atm_from_column(col):
    """Oracle atmosphere dict of a column.Column (set-up arrays as built)."""
    keys = ('M', 'n_0', 'Tco', 'Kzz', 'vz', 'Dzz', 'Ti', 'ms', 'alpha', 'pico', 'dzi', 'Hpi',
            'g', 'Hp', 'dz', 'zco', 'top_flux', 'bot_flux', 'bot_vdep')
    return {k: getattr(col, k) for k in keys}


def item_floor(on, it, dt, samples=3, eps=4e-16):
    """Conditioning floor of an attempt from a column item (batch.build_items):
    the oracle's result and its spread when the Jacobian changes at the
    rounding level (see reference_floor).  Returns (oracle result, floor)."""
    args = (on, it['y'], it['ymix'], dt, it['k'], atm_from_column(it['col']), O.Flags(),
            O.Tol(), 'banded')
    r0 = O.ros2_attempt(*args)
    e = 0.0
    for seed in range(samples):
        r = O.ros2_attempt(*args, perturb=(eps, seed))
        e = max(e, floor_err(r.sol, r0.sol, it['col'].n_0))
    return r0, e
