"""One atmospheric column: the FP64 set-up arrays the Ros2 step consumes.

Restates the reference's atmosphere builder for the fields that feed the
transport operator and Jacobian:
  * pressure interfaces ``pico``            build_atm.py:310-325 (Atm.f_pico)
  * M = n_0 = p/(kT)                        build_atm.py:475-476
  * mean molecular weight, g(z), Hp, dz, dzi, zco, Ti, Hpi
                                            build_atm.py:515-615 (mean_mass, f_mu_dz)
                                            op.py:944-984 (Integration.update_mu_dz)
  * molecular diffusion Dzz, thermal diffusion alpha, masses ms
                                            build_atm.py:660-741 (Atm.mol_diff)
  * constant-mixing-ratio start             build_atm.py:192-198, 262-272
  * element totals                          build_atm.py:283-291 (ele_sum)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .network import KB, NAVO


@dataclass
class Column:
    pco: np.ndarray
    Tco: np.ndarray
    Kzz: np.ndarray                 # [nz-1] at interfaces
    vz: np.ndarray                  # [nz-1]
    gs: float
    Rp: float
    rocky: bool
    use_moldiff: bool
    atm_base: str = 'H2'
    pico: np.ndarray = None
    M: np.ndarray = None
    n_0: np.ndarray = None
    mu: np.ndarray = None
    g: np.ndarray = None
    Hp: np.ndarray = None
    dz: np.ndarray = None
    zco: np.ndarray = None
    dzi: np.ndarray = None
    Ti: np.ndarray = None
    Hpi: np.ndarray = None
    Dzz: np.ndarray = None          # [nz-1, ni]
    Dzz_cen: np.ndarray = None      # [nz, ni] the same at layer centres (written to .vul)
    ms: np.ndarray = None           # [ni]
    alpha: np.ndarray = None        # [ni]
    pref_indx: int = 0
    top_flux: np.ndarray = None
    bot_flux: np.ndarray = None
    bot_vdep: np.ndarray = None
    extra: dict = field(default_factory=dict)

    @property
    def nz(self):
        return self.pco.size


def f_pico(pco):
    """Interface pressures: geometric means, extrapolated at both ends."""
    pi = np.sqrt(pco * np.roll(pco, 1))
    pi[0] = pco[0] ** 1.5 * pco[1] ** (-0.5)
    return np.append(pi, pco[-1] ** 1.5 * pco[-2] ** (-0.5))


def mean_mass(mass, ymix):
    """mu(z) = sum_i m_i ymix_i, accumulated species by species."""
    mu = np.zeros(ymix.shape[0])
    for i in range(ymix.shape[1]):
        mu += mass[i] * ymix[:, i]
    return mu


def mu_dz(col: Column, mass, ymix):
    """Gravity, scale height and grid spacing from the current ymix.

    Same recurrence as f_mu_dz / update_mu_dz: g = gs at the 1-bar interface
    index (gas giants with P_b >= 1 bar), g ~ (Rp/(Rp+z))^2 away from it,
    dz = Hp ln(pico_i/pico_{i+1}), zco accumulated upward (and downward below
    the reference level)."""
    nz = col.nz
    Tco, pico = col.Tco, col.pico
    mu = mean_mass(mass, ymix)
    g = col.g if col.g is not None else np.zeros(nz)
    Hp = col.Hp if col.Hp is not None else np.empty(nz)
    dz = col.dz if col.dz is not None else np.zeros(nz)
    zco = col.zco if col.zco is not None else np.zeros(nz + 1)
    pref = col.pref_indx
    for i in range(pref, nz):
        if i == pref:
            g[i] = col.gs
            Hp[i] = KB * Tco[i] / (mu[i] / NAVO * col.gs)
        else:
            g[i] = col.gs * (col.Rp / (col.Rp + zco[i])) ** 2
            Hp[i] = KB * Tco[i] / (mu[i] / NAVO * g[i])
        dz[i] = Hp[i] * np.log(pico[i] / pico[i + 1])
        zco[i + 1] = zco[i] + dz[i]
    if pref != 0:
        for i in range(pref - 1, -1, -1):
            g[i] = col.gs * (col.Rp / (col.Rp + zco[i + 1])) ** 2
            Hp[i] = KB * Tco[i] / (mu[i] / NAVO * g[i])
            dz[i] = Hp[i] * np.log(pico[i] / pico[i + 1])
            zco[i] = zco[i + 1] - dz[i]
    dzi = 0.5 * (dz + np.roll(dz, 1))
    col.mu, col.g, col.Hp, col.dz, col.zco = mu, g, Hp, dz, zco
    col.dzi = dzi[1:].copy()
    if col.use_moldiff:
        Ti = 0.5 * (Tco + np.roll(Tco, -1))
        col.Ti = Ti[:-1].copy()
        Hpi = 0.5 * (Hp + np.roll(Hp, -1))
        col.Hpi = Hpi[:-1].copy()
    return col


def mol_diff(col: Column, species, mass):
    """Dzz at interfaces and thermal-diffusion factors (atm_base H2/N2/O2/CO2)."""
    ni = len(species)
    Tco, n_0 = col.Tco, col.n_0
    Tco_i = np.delete((Tco + np.roll(Tco, 1)) * 0.5, 0)
    n0_i = np.delete((n_0 + np.roll(n_0, 1)) * 0.5, 0)
    alpha = np.zeros(ni)
    Dzz = np.zeros((col.nz - 1, ni))
    Dzz_cen = np.zeros((col.nz, ni))
    col.ms = np.array(mass, dtype=np.float64)
    if not col.use_moldiff:
        col.Dzz, col.Dzz_cen, col.alpha = Dzz, Dzz_cen, alpha
        return col
    base = col.atm_base
    if base == 'H2':
        gen = lambda T, n, mi: 2.2965E17 * T ** 0.765 / n * (16.04 / mi * (mi + 2.016) / 18.059) ** 0.5
        if 'H' in species:
            alpha[species.index('H')] = -0.1
        if 'He' in species:
            alpha[species.index('He')] = 0.145
        for k, sp in enumerate(species):
            if mass[k] > 4.:
                alpha[k] = 0.25
    else:
        params = {'N2': (7.34E16, 0.75, 16.04, 28.014, 44.054),
                  'O2': (7.51E16, 0.759, 16.04, 32., 48.04),
                  'CO2': (2.15E17, 0.750, 2.016, 44.001, 46.017)}
        if base not in params:
            raise IOError('Unknown atm_base ' + base)
        a, b, mref, mb, mt = params[base]
        gen = lambda T, n, mi: a * T ** b / n * (mref / mi * (mi + mb) / mt) ** 0.5
        for sp, v in (('H', -0.25), ('H2', -0.25), ('He', -0.25), ('Ar', 0.17)):
            if sp in species:
                alpha[species.index(sp)] = v
    for k in range(ni):
        Dzz[:, k] = gen(Tco_i, n0_i, mass[k])
        Dzz_cen[:, k] = gen(Tco, n_0, mass[k])
    col.Dzz, col.Dzz_cen, col.alpha = Dzz, Dzz_cen, alpha
    return col


def build_column(net, pco, Tco, Kzz, gs=2140., Rp=1.138 * 7.1492E9, rocky=False,
                 use_moldiff=True, atm_base='H2', vz=None, ymix0=None):
    """Assemble a Column from pressure/temperature/Kzz and an initial ymix."""
    pco = np.asarray(pco, dtype=np.float64)
    nz = pco.size
    col = Column(pco=pco, Tco=np.asarray(Tco, dtype=np.float64),
                 Kzz=np.asarray(Kzz, dtype=np.float64),
                 vz=np.zeros(nz - 1) if vz is None else np.asarray(vz, np.float64),
                 gs=gs, Rp=Rp, rocky=rocky, use_moldiff=use_moldiff,
                 atm_base=atm_base)
    col.pico = f_pico(pco)
    col.M = pco / (KB * col.Tco)
    col.n_0 = col.M.copy()
    if not rocky and pco[0] >= 1e6:
        col.pref_indx = min(range(nz + 1), key=lambda i: abs(np.log10(col.pico[i]) - 6.))
    else:
        col.pref_indx = 0
    ni = net.ni
    col.top_flux = np.zeros(ni)
    col.bot_flux = np.zeros(ni)
    col.bot_vdep = np.zeros(ni)
    if ymix0 is not None:
        mu_dz(col, net.mass, ymix0)
    mol_diff(col, net.species, net.mass)
    return col


def const_mix_state(net, n_0, const_mix):
    """y = n_0 * x for the listed species, ymix = y / sum(y)."""
    nz = n_0.size
    y = np.zeros((nz, net.ni))
    for sp, x in const_mix.items():
        y[:, net.species.index(sp)] = n_0 * x
    ymix = y / np.sum(y, axis=1).reshape((-1, 1))
    return y, ymix


def atom_totals(net, y, atom_list):
    """Column totals of each element: sum_i n_a(i) sum_z y[z, i]."""
    comp = net.compo_for(atom_list)
    return np.array([np.sum([comp[i, a] * y[:, i] for i in range(net.ni)])
                     for a in range(len(atom_list))])
