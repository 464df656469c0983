"""Seeded synthetic workloads (no public dataset is involved).

* ``c0``: CHO thermo network, nz=100, P log-spaced 1e3 bar -> 1e-8 bar,
  T linear in log P from 2500 K (bottom) to 1000 K (top), Kzz = 1e9 cm^2/s,
  constant mixing ratios H2 0.85, He 0.145, C and O carried by CH4/CO/H2O at
  C/H = 2.7e-4, O/H = 4.9e-4; dt starts at 1e-10 s.
* ``c1``: NCHO photo network, nz=150, same T-P shape with a seeded +-200 K
  Gaussian-process perturbation, Kzz log-linear 1e7 -> 1e10 cm^2/s, frozen
  photolysis rates log10 J_top ~ U[-12,-3] s^-1 attenuated by exp(-tau),
  tau log-linear in P reaching 50 at 1 bar.
* ``c2``: batch of columns on the NCHO thermo network, nz ~ U{60..200},
  T_bot ~ U[1200,3000] K, T_top ~ U[500,1500] K, log10 Kzz ~ U[5,10],
  metallicity log-uniform 0.1-100x solar, C/O ~ U[0.3,1.2].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

P_B, P_T = 1e9, 1e-2                    # dyn cm^-2 (1e3 bar, 1e-8 bar)
GS, RP = 2140., 1.138 * 7.1492E9        # HD 189733b-like gravity and radius
SOLAR_CH, SOLAR_OH, SOLAR_NH = 2.7e-4, 4.9e-4, 6.76e-5

# Solver knobs: the reference's defaults (vulcan_cfg.py:128-159).
SOLVER_DEFAULTS = dict(
    dttry=1.E-10, trun_min=1e2, runtime=1.E22, dt_min=1.E-14, dt_max=1.E22 * 1e-5,
    dt_var_max=2., dt_var_min=0.5, count_min=120, count_max=int(3E4),
    atol=1.E-1, mtol=1.E-22, mtol_conv=1.E-20, pos_cut=0., nega_cut=-1.,
    loss_eps=1e-1, yconv_cri=0.01, slope_cri=1.e-4, yconv_min=0.1, flux_cri=0.1,
    rtol=0.25, st_factor=0.5, conv_step=500, update_frq=100)


@dataclass
class ColumnSpec:
    """Inputs of one synthetic column before the atmosphere set-up."""
    network: str            # network file name (thermo/<name>)
    use_photo: bool
    pco: np.ndarray
    Tco: np.ndarray
    Kzz: np.ndarray         # [nz-1]
    const_mix: dict
    atom_list: list
    conver_ignore: list
    photo_J: dict = None    # {(sp, branch): J[nz]} frozen photolysis rates
    # the reference's transport and set-up options (vulcan_cfg names):
    top_flux: dict = None   # {sp: flux} constant top flux (BC_top file), cm^-2 s^-1
    bot_flux: dict = None   # {sp: (flux, v_dep)} bottom flux and deposition (BC_bot file)
    vz: np.ndarray = None   # [nz-1] vertical advection (cm/s, + upward)
    use_moldiff: bool = True
    atm_base: str = 'H2'
    rocky: bool = False


def log_p_grid(nz):
    return np.logspace(np.log10(P_B), np.log10(P_T), nz)


def linear_logp_T(pco, T_bot, T_top):
    x = (np.log10(pco[0]) - np.log10(pco)) / (np.log10(pco[0]) - np.log10(pco[-1]))
    return T_bot + (T_top - T_bot) * x


def solar_mix(met=1.0, c_to_o=None, with_n=False):
    """Constant mixing ratios: H2 0.85, He 0.145, C/O/N split over molecules."""
    h = 2 * 0.85
    o = SOLAR_OH * met * h
    c = (SOLAR_CH * met * h) if c_to_o is None else c_to_o * o
    co = 0.5 * min(c, o)
    mix = {'H2': 0.85, 'He': 0.145, 'CO': co, 'CH4': c - co, 'H2O': o - co}
    if with_n:
        n = SOLAR_NH * met * h
        mix['NH3'] = 0.5 * n
        mix['N2'] = 0.25 * n
    return mix


def config0(nz=100):
    pco = log_p_grid(nz)
    return ColumnSpec(network='CHO_thermo_network.txt', use_photo=False, pco=pco,
                      Tco=linear_logp_T(pco, 2500., 1000.),
                      Kzz=np.full(nz - 1, 1e9), const_mix=solar_mix(),
                      atom_list=['H', 'O', 'C', 'He'], conver_ignore=[])


def _gp_perturbation(rng, x, amp, length):
    d = x[:, None] - x[None, :]
    cov = amp ** 2 * np.exp(-0.5 * (d / length) ** 2) + 1e-9 * np.eye(x.size)
    L = np.linalg.cholesky(cov)
    return np.clip(L @ rng.standard_normal(x.size), -2 * amp, 2 * amp)


def photo_J_profile(rng, pco, channels):
    """Frozen J(z) = J_top exp(-tau), tau = 50 (P / 1 bar), per channel."""
    tau = 50.0 * (pco / 1e6)
    att = np.exp(-tau)
    return {ch: 10.0 ** rng.uniform(-12, -3) * att for ch in channels}


def config1(photo_channels, nz=150, seed=1):
    rng = np.random.default_rng(seed)
    pco = log_p_grid(nz)
    T = linear_logp_T(pco, 2500., 1000.)
    T = T + _gp_perturbation(rng, np.log10(pco), 100.0, 1.5)
    pico_inner = np.sqrt(pco[1:] * pco[:-1])
    x = (np.log10(pco[0]) - np.log10(pico_inner)) / (np.log10(pco[0]) - np.log10(pco[-1]))
    Kzz = 10.0 ** (7.0 + 3.0 * x)
    return ColumnSpec(network='NCHO_photo_network.txt', use_photo=True, pco=pco,
                      Tco=T, Kzz=Kzz, const_mix=solar_mix(with_n=True),
                      atom_list=['H', 'O', 'C', 'He', 'N'],
                      conver_ignore=['HC3N'],
                      photo_J=photo_J_profile(rng, pco, photo_channels))


def config2_columns(ncols=512, seed=2, nz_range=(60, 200)):
    """Seeded parameters of a batch of uneven columns (NCHO thermo)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(ncols):
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        T_bot = rng.uniform(1200., 3000.)
        T_top = rng.uniform(500., 1500.)
        logK = rng.uniform(5., 10.)
        met = 10.0 ** rng.uniform(-1., 2.)
        c_to_o = rng.uniform(0.3, 1.2)
        pco = log_p_grid(nz)
        specs.append(ColumnSpec(
            network='NCHO_thermo_network.txt', use_photo=False, pco=pco,
            Tco=linear_logp_T(pco, T_bot, T_top), Kzz=np.full(nz - 1, 10.0 ** logK),
            const_mix=solar_mix(met=met, c_to_o=c_to_o, with_n=True),
            atom_list=['H', 'O', 'C', 'He', 'N'], conver_ignore=['HC3N']))
    return specs


def config4_columns(photo_channels, ncols=128, seed=4, nz=200,
                    network='SYN150_network.txt'):
    """Seeded columns on the synthetic 150-species stress network
    (synthnet.generate): nz = 200, T/Kzz/metallicity drawn like the uneven
    NCHO batch, frozen J on its 60 photolysis channels."""
    rng = np.random.default_rng(seed)
    specs = []
    pco = log_p_grid(nz)
    for _ in range(ncols):
        T_bot = rng.uniform(1200., 3000.)
        T_top = rng.uniform(500., 1500.)
        logK = rng.uniform(5., 10.)
        met = 10.0 ** rng.uniform(-1., 2.)
        c_to_o = rng.uniform(0.3, 1.2)
        specs.append(ColumnSpec(
            network=network, use_photo=True, pco=pco,
            Tco=linear_logp_T(pco, T_bot, T_top), Kzz=np.full(nz - 1, 10.0 ** logK),
            const_mix=solar_mix(met=met, c_to_o=c_to_o, with_n=True),
            atom_list=['H', 'O', 'C', 'He', 'N'], conver_ignore=[],
            photo_J=photo_J_profile(rng, pco, photo_channels)))
    return specs
