"""Generate golden fixtures by running the reference VULCAN itself.

Test infrastructure only: run where the reference source is at hand (its
path from ``--ref`` or the VULCAN_REFERENCE environment variable); the GPU
machine only reads the committed ``tests/golden/*.npz``.

For each workload it
  1. copies the reference tree to a temporary directory (the reference's code
     generator rewrites its network file in place, so it never runs on the
     original), adds a matplotlib stub and appends overrides to vulcan_cfg.py;
  2. runs the reference's own ``make_chem_funs.py`` (its numpy-2 crash in
     check_conserv comes after chem_funs.py is complete and is tolerated);
  3. runs the reference's set-up sequence (vulcan.py order) with the seeded
     synthetic temperature / Kzz / mixing ratios / frozen J injected, then the
     reference's own ``op.Integration`` loop with a recording ``op.Ros2``
     subclass that captures every Ros2 attempt's inputs and outputs
     (y, ymix, dt, k1, k2, sol, delta) plus the per-step trajectory;
  4. stores the compiled network (our parser's tables) beside the reference's
     own view of it (species order, nr) and the atmosphere arrays.

Workloads:
  c0, c1, c2, c2long, c2conv, c2tight, c2slow, c3s   Ros2 attempts and
      trajectories (c3s on the 89-species sulfur network);
  c0bc, c0nomol, c0vz   transport options (top / bottom fluxes, deposition,
      H escape, no molecular diffusion, vertical advection) with the
      reference's transport RHS and LHS blocks;
  c0n2, c0o2, c0co2, c0rocky   column set-up with another base gas for
      molecular diffusion, rocky surface;
  c1rt, c1rtT, c1rtA, c3rt   the reference's radiative transfer
      (T-independent and T-dependent cross sections, other parameters, the
      sulfur network);
  lowT, rmlist, snchok   rate constants (low-temperature caps, reactions
      removed, the sulfur network);
  c4s   Ros2 attempts on the seeded 150-species synthetic network
      (vulcan_gb300.synthnet, installed into the copy), 20 layers;
  n_<network>   every shipped network the reference can set up: rate
      constants, chemdf at a seeded state with seeded J, -J blocks;
  a_<network>   Ros2 attempts on five more shipped networks (seeded J).

Usage:  python tests/golden/make_golden.py [tag ...] [--ref <VULCAN tree>]
        python tests/golden/make_golden.py --setup-only c1rt c1rtT
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import textwrap

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from vulcan_gb300 import configs  # noqa: E402
from vulcan_gb300.network import Network  # noqa: E402

# Which attempts go into the committed fixture (all attempts are recorded).
KEEP = {'c0': (0, 1, 2, 3, 5, 8, 13, 40, 99, 100, 101, 150, 250, 499),
        'c1': (0, 1, 2, 10, 29),
        'c2': (0, 1, 2, 10, 29),
        'c2long': (400, 800, 1200, 1600, 1999),
        'c2conv': (0,),
        'c2tight': (0,),
        'c2slow': (0,),
        'c1rt': (0,),
        'c1rtT': (0,),
        'c1rtA': (0,),
        'c3rt': (0,),
        'lowT': (0,),
        'c0bc': (0, 1, 2, 10, 29),
        'c0nomol': (0, 1, 2, 10, 29),
        'c0vz': (0, 1, 2, 10, 29),
        'rmlist': (0,),
        'snchok': (0,),
        'c3s': (0, 1, 2, 5, 9),
        'c0n2': (0,), 'c0o2': (0,), 'c0co2': (0,), 'c0rocky': (0,),
        'c0vul': (0,),
        'c4s': (0, 1, 2, 5, 9)}
NSTEPS = {'c0': 500, 'c1': 30, 'c2': 30, 'c2long': 2000, 'c2conv': 4000, 'c2tight': 12000,
          'c2slow': 4000, 'c1rt': 110, 'c1rtT': 110, 'c1rtA': 2, 'c3rt': 2, 'lowT': 1, 'c0bc': 30,
          'c0nomol': 30, 'c0vz': 30, 'rmlist': 1, 'snchok': 1, 'c3s': 10, 'c0n2': 2, 'c0o2': 2, 'c0co2': 2,
          'c0rocky': 2, 'c0vul': 20, 'c4s': 10}
# convergence criterion tightened from the reference defaults (yconv_cri 0.01,
# yconv_min 0.1): a steady state determined to ~1e-3 that another integrator
# must reproduce, whatever path it takes there
EXTRA_CFG = {'c2tight': 'yconv_cri = 0.001\nyconv_min = 0.001\n',
             # radiative transfer on, on 1 nm bins below 240 nm (2 nm above) to keep
             # the fixture small; everything else the reference's defaults
             'c1rt': 'dbin1 = 1.0\n',
             # the same with temperature-dependent cross sections for the three
             # species the reference ships T tables for in this network
             'c1rtT': "dbin1 = 1.0\nT_cross_sp = ['CO2', 'H2O', 'NH3']\n"}
# boundary options on the c0 column: constant top and bottom fluxes with
# deposition velocities, diffusion-limited escape of H (update_phi_esc), with
# and without molecular diffusion (the no-moldiff Jacobian's escape term is
# not part of the device path, so c0nomol leaves diff_esc empty)
BC_CFG = ("use_topflux = True\nuse_botflux = True\n"
          "top_BC_flux_file = 'atm/BC_top_golden.txt'\n"
          "bot_BC_flux_file = 'atm/BC_bot_golden.txt'\n")
EXTRA_CFG['c0bc'] = BC_CFG + "diff_esc = ['H']\n"
EXTRA_CFG['c0nomol'] = BC_CFG + "use_moldiff = False\n"
# fluxes large enough to stand out in the transport terms they enter
BC_FILES = {'atm/BC_top_golden.txt': '#species flux [cm-2 s-1]\nCO2  1.0E+12\nH2O  4.0E+11\n',
            'atm/BC_bot_golden.txt': ('#species flux [cm-2 s-1]   v_dep [cm s-1]\n'
                                      'CH4  1.0E+14  0.\nCO  0.  1.0E-02\nH2O  2.0E+14  1.0E-03\n')}
BC_TAGS = ('c0bc', 'c0nomol')
# vertical advection: a vz profile that changes sign (upwind branches both
# ways), injected like T and Kzz
EXTRA_CFG['c0vz'] = 'use_vz = True\n'
# column set-up variants: molecular-diffusion base gas, rocky surface
for _t, _base in (('c0n2', 'N2'), ('c0o2', 'O2'), ('c0co2', 'CO2')):
    EXTRA_CFG[_t] = "atm_base = '%s'\n" % _base
EXTRA_CFG['c0rocky'] = 'rocky = True\n'
VZ_TAGS = ('c0vz',)
# other radiative-transfer parameters: zenith angle 60 deg, Eddington
# coefficient 0.669, f_diurnal 0.5, and dbin_12trans beyond the bins (the
# reference then sums J with index -1, build_atm.py:647, op.py:2770-2774)
EXTRA_CFG['c1rtA'] = ('dbin1 = 2.0\nsl_angle = 60. / 180. * 3.14159\nedd = 0.669\n'
                      'f_diurnal = 0.5\ndbin_12trans = 900.\n')
# the sulfur network's radiative transfer (37 absorbers, 60 channels)
EXTRA_CFG['c3rt'] = 'dbin1 = 2.0\n'
PHOTO_TAGS = ('c1rt', 'c1rtT', 'c1rtA', 'c3rt')
# every network file the reference ships that its own set-up can use (two
# cannot: SNCHO_photo_network_2025 names a species without a NASA-9 file,
# SNCHO_photo_network_C3 species missing from all_compose.txt): rate
# constants, the generated chemistry source at a seeded positive state with
# seeded J in the photolysis slots, and -J blocks (rate driver, 8 layers)
NET_FILES = ('CHO_photo_network.txt', 'CHO_photo_network_lowT.txt', 'CHO_thermo_network.txt',
             'NCHO_earth_photo_network.txt', 'NCHO_full_photo_network.txt',
             'NCHO_photo_network.txt', 'NCHO_photo_network_lowT.txt',
             'NCHO_photo_network_lowT_Jupiter.txt', 'NCHO_photo_oxidising_network.txt',
             'NCHO_thermo_network.txt', 'SNCHO_DMS_photo_network_Tsai2024.txt',
             'SNCHO_full_photo_network.txt', 'SNCHO_photo_network.txt',
             'SNCHO_photo_network_2024.txt', 'TiSNCHO_photo_network.txt')
NET_TAGS = {'n_' + f.replace('_network', '').replace('.txt', ''): f for f in NET_FILES}
for _t in NET_TAGS:
    KEEP[_t], NSTEPS[_t] = (0,), 1
# Ros2 attempts (10 steps of a 20-layer column, seeded J) on shipped networks
# beyond the c0 / c1 / c2 / c3s ones: the largest of each family, the
# titanium one and the one with condensation species
ATT_TAGS = {'a_' + f.replace('_network', '').replace('.txt', ''): f
            for f in ('CHO_photo_network.txt', 'NCHO_full_photo_network.txt',
                      'NCHO_photo_network_lowT_Jupiter.txt', 'SNCHO_full_photo_network.txt',
                      'TiSNCHO_photo_network.txt')}
for _t in ATT_TAGS:
    KEEP[_t], NSTEPS[_t] = (0, 1, 2, 5, 9), 10


def family_mix(fname):
    """A start with the family's main carriers of each element."""
    mix = {'H2': 0.85, 'He': 0.145, 'H2O': 1e-3, 'CH4': 5e-4}
    if 'NCHO' in fname:
        mix['NH3'] = 1e-4
    if 'SNCHO' in fname:
        mix['H2S'] = 3e-5
    if fname.startswith('TiSNCHO'):
        mix['TiO'] = 1e-8
        mix['VO'] = 1e-9
    return mix


def net_atoms(fname):
    """The elements of a shipped network family."""
    if fname.startswith('TiSNCHO'):
        return ['H', 'O', 'C', 'He', 'N', 'S', 'Ti', 'V']
    if fname.startswith('SNCHO'):
        return ['H', 'O', 'C', 'He', 'N', 'S']
    if fname.startswith('NCHO'):
        return ['H', 'O', 'C', 'He', 'N']
    return ['H', 'O', 'C', 'He']


# the seeded 150-species synthetic network (vulcan_gb300.synthnet: network
# file, NASA-9 files and composition table in the reference's formats,
# installed into the temporary copy) on a 20-layer column with frozen J on
# its 60 photolysis channels
SYN_TAGS = ('c4s',)
# rate constants only (no integration): read_rate, lim_lowT_rates, rev_rate
RATE_TAGS = ('lowT', 'rmlist', 'snchok')
# the sulfur network with its photolysis slots (rate constants only)
RATE_PHOTO_TAGS = ('snchok',)
# remove_list: two forward rates and one reverse rate taken out
EXTRA_CFG['rmlist'] = 'remove_list = [5, 12, 101]\n'

DRIVER = r'''
import os, sys, time, json
import numpy as np
sys.path.insert(0, os.getcwd())
sys.path.insert(0, os.path.join(os.getcwd(), '_mplstub'))
import scipy.linalg
_orig = scipy.linalg.solve_banded
SB = []
def _sb(*a, **kw):
    x = _orig(*a, **kw)
    SB.append(np.array(x, copy=True))
    return x
scipy.linalg.solve_banded = _sb
import vulcan_cfg
import store, build_atm, op, chem_funs
from phy_const import kb
inp = np.load('golden_inputs.npz', allow_pickle=True)
meta = json.load(open('golden_meta.json'))

var = store.Variables(); atm = store.AtmData(); para = store.Parameters()
para.start_time = time.time()
make_atm = build_atm.Atm()
output = op.Output()
atm = make_atm.f_pico(atm)
atm = make_atm.load_TPK(atm)
atm.Tco = inp['Tco'].copy()
atm.M = atm.pco / (kb * atm.Tco)
atm.n_0 = atm.M.copy()
atm.Kzz = inp['Kzz'].copy()
if 'vz' in inp.files:
    atm.vz = inp['vz'].copy()
rate = op.ReadRate()
var = rate.read_rate(var, atm)
var = rate.rev_rate(var, atm)
var = rate.remove_rate(var)
ini = build_atm.InitialAbun()
var = ini.ini_y(var, atm)
var = ini.ele_sum(var)
atm = make_atm.f_mu_dz(var, atm, output)
make_atm.mol_diff(atm)
make_atm.BC_flux(atm)
NZ = len(atm.pco)
if not vulcan_cfg.use_moldiff:         # no interface T / Hp without molecular diffusion
    atm.Ti, atm.Hpi = np.zeros(NZ - 1), np.zeros(NZ - 1)
for key, J in zip(meta['photo_keys'], inp['photo_J']):
    var.k[var.pho_rate_index[(key[0], int(key[1]))]] = J.copy()
nr = chem_funs.nr
K = np.array([var.k[i] for i in range(1, nr + 1)])
setup = dict(pico=atm.pico, M=atm.M, n_0=atm.n_0, mu=atm.mu, g=atm.g.copy(),
             Hp=atm.Hp.copy(), dz=atm.dz.copy(), zco=atm.zco.copy(), dzi=atm.dzi,
             Ti=atm.Ti, Hpi=atm.Hpi, Dzz=atm.Dzz, ms=atm.ms, alpha=atm.alpha,
             Kzz=atm.Kzz, vz=atm.vz, Tco=atm.Tco, pco=atm.pco, k=K,
             y_ini=var.y.copy(), ymix_ini=var.ymix.copy(),
             atom_ini=np.array([var.atom_ini[a] for a in vulcan_cfg.atom_list]),
             pref_indx=atm.pref_indx, top_flux=atm.top_flux.copy(), bot_flux=atm.bot_flux.copy(),
             bot_vdep=atm.bot_vdep.copy(), use_moldiff=bool(vulcan_cfg.use_moldiff),
             use_topflux=bool(vulcan_cfg.use_topflux), use_botflux=bool(vulcan_cfg.use_botflux),
             diff_esc=np.array(list(vulcan_cfg.diff_esc), dtype='U8'),
             atm_base=str(vulcan_cfg.atm_base), rocky=bool(vulcan_cfg.rocky))
# chemistry pins at the initial state
setup['chemdf0'] = chem_funs.chemdf(var.y, atm.M, var.k)
ATT, STEPS = [], []

class RecRos2(op.Ros2):
    def solver(self, v, a, p):
        snap = dict(y=v.y.copy(), ymix=v.ymix.copy(), dt=float(v.dt),
                    dzi=a.dzi.copy(), Hpi=a.Hpi.copy(), g=a.g.copy(), Hp=a.Hp.copy(),
                    count=int(p.count), t=float(v.t), top_flux=a.top_flux.copy())
        del SB[:]
        v, p = op.Ros2.solver(self, v, a, p)
        snap.update(k1=SB[0], k2=SB[1], sol=v.y.copy(), delta=float(p.delta))
        ATT.append(snap)
        return v, p
    def clip(self, v, p, a, **kw):
        v, p = op.Ros2.clip(self, v, p, a, **kw)
        ATT[-1]['y_clip'] = v.y.copy()
        ATT[-1]['atom_loss'] = np.array([v.atom_loss[x] for x in vulcan_cfg.atom_list])
        ATT[-1]['ok'] = bool(self.step_ok(v, p))
        return v, p
    def step_size(self, v, p, **kw):
        STEPS.append(dict(count=int(p.count), t=float(v.t), dt_used=float(v.dt),
                          delta=float(p.delta), y=v.y.copy(), natt=len(ATT)))
        v = op.Ros2.step_size(self, v, p, **kw)
        STEPS[-1]['dt_next'] = float(v.dt)
        return v

solver = RecRos2()
if vulcan_cfg.use_topflux or vulcan_cfg.use_botflux or not vulcan_cfg.use_moldiff or np.any(atm.vz):
    # the reference's own transport RHS and LHS at the initial state, with the
    # functions its Ros2.solver picks for these options (op.py:2870-2888); the
    # LHS with every rate constant zero and dt = 1e10 s, so that its blocks are
    # the transport Jacobian (the chemistry part is pinned by negjac_blocks)
    mol = vulcan_cfg.use_moldiff
    setup['diffdf0'] = (solver.diffdf if mol else solver.diffdf_no_mol)(var.y, atm)
    k_keep, dt_keep = var.k, var.dt
    var.k = {i: np.zeros_like(v) for i, v in var.k.items()}
    var.dt = 1e10
    lhs = (solver.lhs_jac_tot if mol else solver.lhs_jac_no_mol)(var, atm)
    var.k, var.dt = k_keep, dt_keep
    ni_, nz_ = chem_funs.ni, len(atm.pco)
    lays = [0, 1, nz_ // 2, nz_ - 1]
    setup['lhs_layers'] = np.array(lays)
    setup['lhs_D'] = np.array([lhs[l*ni_:(l+1)*ni_, l*ni_:(l+1)*ni_] for l in lays])
    setup['lhs_U'] = np.array([np.diag(lhs[l*ni_:(l+1)*ni_, (l+1)*ni_:(l+2)*ni_])
                               if l < nz_ - 1 else np.zeros(ni_) for l in lays])
    setup['lhs_L'] = np.array([np.diag(lhs[l*ni_:(l+1)*ni_, (l-1)*ni_:l*ni_])
                               if l > 0 else np.zeros(ni_) for l in lays])
    setup['lhs_dt'] = 1e10
    del lhs
integ = op.Integration(solver, output)
solver.naming_solver(para)
# chemistry Jacobian pins (a few diagonal blocks of neg_symjac at the start)
ni = chem_funs.ni
J0 = chem_funs.neg_symjac(var.y, atm.M, var.k)
lays = [0, 1, len(atm.pco) // 2, len(atm.pco) - 1]
setup['negjac_layers'] = np.array(lays)
setup['negjac_blocks'] = np.array([J0[l*ni:(l+1)*ni, l*ni:(l+1)*ni] for l in lays])
del J0
t0 = time.time()
integ(var, atm, para, make_atm)
wall = time.time() - t0
keep = meta['keep']
att_keys = ['y', 'ymix', 'dt', 'dzi', 'Hpi', 'g', 'Hp', 'count', 't', 'k1', 'k2',
            'sol', 'delta', 'y_clip', 'atom_loss', 'ok', 'top_flux']
out = dict(setup)
sel = [i for i in keep if i < len(ATT)]
out['att_index'] = np.array(sel)
for key in att_keys:
    out['att_' + key] = np.array([ATT[i][key] for i in sel])
out['traj_count'] = np.array([s['count'] for s in STEPS])
out['traj_t'] = np.array([s['t'] for s in STEPS])
out['traj_dt_used'] = np.array([s['dt_used'] for s in STEPS])
out['traj_dt_next'] = np.array([s['dt_next'] for s in STEPS])
out['traj_delta'] = np.array([s['delta'] for s in STEPS])
out['traj_natt'] = np.array([s['natt'] for s in STEPS])
out['att_all_delta'] = np.array([a['delta'] for a in ATT])
out['att_all_ok'] = np.array([a['ok'] for a in ATT])
out['att_all_dt'] = np.array([a['dt'] for a in ATT])
ysteps = [s for s in (0, 1, 99, 100, 101, 199, 299, 399, 499) if s < len(STEPS)]
out['ystep_index'] = np.array(ysteps)
out['ystep_y'] = np.array([STEPS[s]['y'] for s in ysteps])
out['final_y'] = STEPS[-1]['y']
out['final_ymix'] = var.ymix.copy()
out['final_t'] = STEPS[-1]['t']
out['final_count'] = STEPS[-1]['count']
out['spec_list'] = np.array(chem_funs.spec_list)
out['nr'] = nr
out['end_case'] = para.end_case
out['wall_s'] = wall
out['n_attempts'] = len(ATT)
np.savez_compressed('golden_out.npz', **out)
if meta.get('save_vul'):                 # the reference's own .vul (op.Output.save_out)
    output.save_out(var, atm, para, os.getcwd())
# full record for local deep checks (not committed)
np.savez_compressed('golden_full.npz',
    **{('a%d_' % i) + k: np.asarray(ATT[i][k]) for i in range(len(ATT)) for k in att_keys})
print('attempts', len(ATT), 'steps', len(STEPS), 'wall', wall)
'''

PHOTO_DRIVER = r'''
import os, sys, time, json
import numpy as np
sys.path.insert(0, os.getcwd())
sys.path.insert(0, os.path.join(os.getcwd(), '_mplstub'))
import vulcan_cfg
import store, build_atm, op, chem_funs
from phy_const import kb
inp = np.load('golden_inputs.npz', allow_pickle=True)

var = store.Variables(); atm = store.AtmData(); para = store.Parameters()
para.start_time = time.time()
make_atm = build_atm.Atm()
output = op.Output()
atm = make_atm.f_pico(atm)
atm = make_atm.load_TPK(atm)
atm.Tco = inp['Tco'].copy()
atm.M = atm.pco / (kb * atm.Tco)
atm.n_0 = atm.M.copy()
atm.Kzz = inp['Kzz'].copy()
if 'vz' in inp.files:
    atm.vz = inp['vz'].copy()
rate = op.ReadRate()
var = rate.read_rate(var, atm)
var = rate.rev_rate(var, atm)
var = rate.remove_rate(var)
ini = build_atm.InitialAbun()
var = ini.ini_y(var, atm)
var = ini.ele_sum(var)
atm = make_atm.f_mu_dz(var, atm, output)
make_atm.mol_diff(atm)
make_atm.BC_flux(atm)
REC = []
CH = sorted(var.pho_rate_index)                 # (species, branch) channels

class RecRos2(op.Ros2):
    def compute_J(self, v, a):
        op.Ros2.compute_J(self, v, a)
        REC.append(dict(y=v.y.copy(), ymix=v.ymix.copy(), tau=v.tau.copy(), aflux=v.aflux.copy(),
                        dflux_u=v.dflux_u.copy(), dflux_d=v.dflux_d.copy(),
                        sflux=v.sflux.copy(), aflux_change=float(v.aflux_change),
                        J=np.array([v.J_sp[c] for c in CH]), dz=a.dz.copy(),
                        count=int(para.count)))

solver = RecRos2()
rate.make_bins_read_cross(var, atm)
make_atm.read_sflux(var, atm)
solver.compute_tau(var, atm)
solver.compute_flux(var, atm)
solver.compute_J(var, atm)
var = rate.remove_rate(var)
absp = sorted(set.union(var.photo_sp, var.ion_sp))
out = dict(bins=var.bins, dbin1=var.dbin1, dbin2=var.dbin2,
           sflux_din12_indx=var.sflux_din12_indx, sflux_top=var.sflux_top,
           absp_sp=np.array(absp), photo_sp=np.array(sorted(var.photo_sp)),
           cross=np.array([var.cross[s] for s in absp]),
           scat_sp=np.array(vulcan_cfg.scat_sp),
           cross_scat=np.array([var.cross_scat[s] for s in vulcan_cfg.scat_sp]),
           ch_sp=np.array([c[0] for c in CH]), ch_br=np.array([c[1] for c in CH]),
           ch_kindex=np.array([var.pho_rate_index[c] for c in CH]),
           cross_J=np.array([var.cross_J[c] for c in CH]),
           sl_angle=vulcan_cfg.sl_angle, edd=vulcan_cfg.edd, f_diurnal=vulcan_cfg.f_diurnal,
           dbin_12trans=vulcan_cfg.dbin_12trans, network=str(vulcan_cfg.network),
           flux_atol=vulcan_cfg.flux_atol, spec_list=np.array(chem_funs.spec_list),
           pco=atm.pco, Tco=atm.Tco, M=atm.M, n_0=atm.n_0)
TSP = list(vulcan_cfg.T_cross_sp)
if TSP:
    TCH = [c for c in CH if c[0] in TSP]
    out.update(T_cross_sp=np.array(TSP), cross_T=np.array([var.cross_T[s] for s in TSP]),
               chT_sp=np.array([c[0] for c in TCH]), chT_br=np.array([c[1] for c in TCH]),
               cross_J_T=np.array([var.cross_J_T[c] for c in TCH]))
integ = op.Integration(solver, output)
solver.naming_solver(para)
integ(var, atm, para, make_atm)
for i, r in enumerate(REC):
    for k, v in r.items():
        out['rec%d_%s' % (i, k)] = np.asarray(v)
out['n_rec'] = len(REC)
np.savez_compressed('golden_out.npz', **out)
print('photo records', len(REC), 'nbins', len(var.bins), 'counts', [r['count'] for r in REC])
'''

RATE_DRIVER = r'''
import os, sys, json
import numpy as np
sys.path.insert(0, os.getcwd())
sys.path.insert(0, os.path.join(os.getcwd(), '_mplstub'))
import vulcan_cfg
import store, build_atm, op, chem_funs
from phy_const import kb
inp = np.load('golden_inputs.npz', allow_pickle=True)
var = store.Variables(); atm = store.AtmData()
make_atm = build_atm.Atm()
atm = make_atm.f_pico(atm)
atm = make_atm.load_TPK(atm)
atm.Tco = inp['Tco'].copy()
atm.M = atm.pco / (kb * atm.Tco)
atm.n_0 = atm.M.copy()
rate = op.ReadRate()
var = rate.read_rate(var, atm)
k_plain = np.array([np.array(var.k[i], dtype=float) for i in range(1, chem_funs.nr + 1, 2)])   # forward
var = rate.lim_lowT_rates(var, atm)
var = rate.rev_rate(var, atm)
var = rate.remove_rate(var)
meta = json.load(open('golden_meta.json'))
for key, J in zip(meta['photo_keys'], inp['photo_J']):     # seeded J (photolysis networks)
    var.k[var.pho_rate_index[(key[0], int(key[1]))]] = J.copy()
K = np.array([var.k[i] for i in range(1, chem_funs.nr + 1)])
# the generated chemistry source at a seeded positive state (term-order pin)
Y = 10.0 ** np.random.default_rng(7).uniform(0.0, 18.0, (atm.Tco.size, chem_funs.ni))
ni = chem_funs.ni
J0 = chem_funs.neg_symjac(Y, atm.M, var.k)
lays = [0, atm.Tco.size // 2]
np.savez_compressed('golden_out.npz', Tco=atm.Tco, M=atm.M, pco=atm.pco, k_plain=k_plain,
                    k=K, y_rand=Y, chemdf_rand=chem_funs.chemdf(Y, atm.M, var.k),
                    spec_list=np.array(chem_funs.spec_list), nr=chem_funs.nr,
                    negjac_layers=np.array(lays),
                    negjac_blocks=np.array([J0[l*ni:(l+1)*ni, l*ni:(l+1)*ni] for l in lays]))
print('rate constants', chem_funs.nr, 'layers', atm.Tco.size)
'''

MPL_STUB = {
    '__init__.py': 'use = lambda *a, **k: None\n',
    'pyplot.py': textwrap.dedent('''
        def __getattr__(name):
            def _f(*a, **k):
                return None
            return _f
        '''),
    'legend.py': textwrap.dedent('''
        def __getattr__(name):
            def _f(*a, **k):
                return None
            return _f
        '''),
}


def cfg_overrides(spec, nz, count_max, use_photo, extra=''):
    mix = {k: float(v) for k, v in spec.const_mix.items()}
    return textwrap.dedent(f'''
        # ---- overrides appended by the golden-fixture generator ----
        network = 'thermo/{spec.network}'
        use_photo = {use_photo}
        atom_list = {spec.atom_list!r}
        nz = {nz}
        P_b = {configs.P_B!r}
        P_t = {configs.P_T!r}
        atm_type = 'isothermal'
        Tiso = 1500.
        Kzz_prof = 'const'
        const_Kzz = 1e9
        use_Kzz = True
        use_moldiff = True
        use_vz = False
        use_vm_mol = False
        atm_base = 'H2'
        rocky = False
        gs = {configs.GS!r}
        Rp = {configs.RP!r}
        ini_mix = 'const_mix'
        const_mix = {mix!r}
        diff_esc = []
        use_topflux = False
        use_botflux = False
        use_fix_sp_bot = {{}}
        use_condense = False
        use_settling = False
        use_ion = False
        remove_list = []
        use_lowT_limit_rates = False
        use_live_plot = False
        use_live_flux = False
        use_plot_end = False
        use_plot_evo = False
        use_save_movie = False
        plot_TP = False
        use_print_prog = False
        use_print_delta = False
        use_adapt_rtol = False
        conver_ignore = {spec.conver_ignore!r}
        count_max = {count_max}
        out_name = 'golden.vul'
        ''') + extra


def install_synthetic(dst, syn_dir):
    """The synthetic network's files in the reference copy: the network into
    thermo/, its NASA-9 files into thermo/NASA9/ (replacing the real ones of
    the species it shares names with), its composition table as
    thermo/all_compose.txt."""
    thermo = os.path.join(dst, 'thermo')
    for f in os.listdir(syn_dir):
        if f.endswith('_network.txt'):
            shutil.copy(os.path.join(syn_dir, f), os.path.join(thermo, f))
    shutil.copy(os.path.join(syn_dir, 'all_compose.txt'), os.path.join(thermo, 'all_compose.txt'))
    for f in os.listdir(os.path.join(syn_dir, 'NASA9')):
        shutil.copy(os.path.join(syn_dir, 'NASA9', f), os.path.join(thermo, 'NASA9', f))


def run_reference(ref_root, tag, spec, nsteps, keep, workdir, syn_dir=None):
    nz = spec.pco.size
    dst = os.path.join(workdir, 'vref_' + tag)
    shutil.copytree(ref_root, dst, ignore=shutil.ignore_patterns('output', 'plot', '.DS_Store'))
    os.chmod(dst, 0o755)
    for root, dirs, files in os.walk(dst):
        for d in dirs:
            os.chmod(os.path.join(root, d), 0o755)
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
    if syn_dir:
        install_synthetic(dst, syn_dir)
    if tag in BC_TAGS:
        for name, text in BC_FILES.items():
            with open(os.path.join(dst, name), 'w') as f:
                f.write(text)
    stub = os.path.join(dst, '_mplstub', 'matplotlib')
    os.makedirs(stub)
    for name, src in MPL_STUB.items():
        with open(os.path.join(stub, name), 'w') as f:
            f.write(src)
    with open(os.path.join(ref_root, 'vulcan_cfg.py')) as f:
        base_cfg = f.read()
    env = dict(os.environ, PYTHONPATH=os.path.join(dst, '_mplstub'), OMP_NUM_THREADS='1')
    # code generation (photo reactions included when the workload has J rates)
    with open(os.path.join(dst, 'vulcan_cfg.py'), 'w') as f:
        f.write(base_cfg + cfg_overrides(spec, nz, nsteps - 1, spec.use_photo, EXTRA_CFG.get(tag, '')))
    subprocess.run([sys.executable, 'make_chem_funs.py'], cwd=dst, env=env,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    with open(os.path.join(dst, 'chem_funs.py')) as f:
        if 'def neg_symjac' not in f.read():
            raise RuntimeError('reference code generation failed for ' + tag)
    # run time: photochemistry (radiative transfer) off, J frozen in k -- except
    # for the radiative-transfer fixtures, which record the reference's own J
    with open(os.path.join(dst, 'vulcan_cfg.py'), 'w') as f:
        f.write(base_cfg + cfg_overrides(spec, nz, nsteps - 1,
                                         tag in PHOTO_TAGS or tag in RATE_PHOTO_TAGS
                                         or (tag in NET_TAGS and spec.use_photo),
                                         EXTRA_CFG.get(tag, '')))
    keys = sorted(spec.photo_J) if spec.photo_J else []
    extra_in = {}
    if tag in VZ_TAGS:     # cm/s on the nz-1 interfaces: +100 below, -100 above
        x = np.linspace(0., 1., nz - 1)
        extra_in['vz'] = 100. * np.cos(np.pi * x)
    np.savez(os.path.join(dst, 'golden_inputs.npz'), Tco=spec.Tco, Kzz=spec.Kzz,
             photo_J=np.array([spec.photo_J[k] for k in keys]) if keys else np.zeros((0, nz)),
             **extra_in)
    with open(os.path.join(dst, 'golden_meta.json'), 'w') as f:
        json.dump({'photo_keys': [[k[0], k[1]] for k in keys], 'keep': list(keep),
                   'save_vul': tag == 'c0vul'}, f)
    with open(os.path.join(dst, 'golden_driver.py'), 'w') as f:
        f.write(PHOTO_DRIVER if tag in PHOTO_TAGS
                else RATE_DRIVER if tag in RATE_TAGS or tag in NET_TAGS else DRIVER)
    r = subprocess.run([sys.executable, 'golden_driver.py'], cwd=dst, env=env,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('reference run failed:\n' + r.stdout[-3000:] + r.stderr[-3000:])
    print(r.stdout.strip().splitlines()[-1])
    return dst


def photo_setup_check(d, ref_root):
    """Largest relative differences between the reference's binned tables
    (recorded) and this package's restatement (vulcan_gb300.photo) from the
    same files -- stored in the fixture so the CPU tests pin the restatement
    without the reference's data files."""
    from vulcan_gb300 import photo
    name = os.path.basename(str(d['network'])) if 'network' in d else 'NCHO_photo_network.txt'
    net = Network.from_file(os.path.join(ref_root, 'thermo', name), use_photo=True)
    t = photo.PhotoTables.from_reference_files(
        net, ref_root, 'atm/stellar_flux/sflux-HD189_Moses11.txt', 0.805, 0.03142,
        float(d['sl_angle']), dbin1=float(d['dbin1']), dbin2=float(d['dbin2']),
        dbin_12trans=float(d['dbin_12trans']) if 'dbin_12trans' in d else 240.0)
    rel = lambda a, b: float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    same = (len(t.bins) == len(d['bins']) and t.i12 == int(d['sflux_din12_indx'])
            and t.absp_sp == [str(s) for s in d['absp_sp']]
            and t.ch_sp == [str(s) for s in d['ch_sp']])
    out = {'setup_same_layout': same,
           'setup_rel_bins': rel(t.bins, d['bins']) if same else np.inf,
           'setup_rel_cross': rel(t.cross, d['cross']) if same else np.inf,
           'setup_rel_cross_J': rel(t.cross_J, d['cross_J']) if same else np.inf,
           'setup_rel_cross_scat': rel(t.cross_scat, d['cross_scat']) if same else np.inf,
           'setup_rel_sflux_top': rel(t.sflux_top, d['sflux_top']) if same else np.inf}
    if 'T_cross_sp' in d and same:
        # the per-layer tables of photo.TCross for the recorded temperatures
        tsp = [str(s) for s in d['T_cross_sp']]
        ct, cj = photo.TCross.from_reference_files(t, ref_root, tsp).for_column(d['Tco'])
        out['setup_rel_cross_T'] = max(rel(ct[sp], d['cross_T'][i]) for i, sp in enumerate(tsp))
        out['setup_rel_cross_J_T'] = max(
            rel(cj[(str(sp), int(br))], d['cross_J_T'][i])
            for i, (sp, br) in enumerate(zip(d['chT_sp'], d['chT_br'])))
    return out


def slim_photo(d):
    """Drop what the tests do not read: the direct beam and the downward
    diffuse flux of every record, the upward diffuse flux after the second
    record, and the state of the second record (the integrator's first update
    runs on the set-up call's state)."""
    out = {}
    for key, v in d.items():
        if key.startswith('rec') and '_' in key:
            i, name = key[3:].split('_', 1)
            i = int(i)
            if name in ('sflux', 'dflux_d') or (name == 'dflux_u' and i > 1):
                continue
            if i == 1 and name in ('y', 'ymix', 'tau', 'dz'):
                if not np.array_equal(v, d['rec0_' + name]):
                    raise RuntimeError('the first update ran on another state: ' + key)
                continue
        out[key] = v
    return out


def make(tag, ref_root, workdir, full_dir=None):
    syn_dir = None                        # synthetic network files (SYN_TAGS)
    if tag in ('c0', 'c0bc', 'c0nomol', 'c0vz', 'c0n2', 'c0o2', 'c0co2', 'c0rocky', 'c0vul'):
        spec = configs.config0()
    elif tag in ('c2', 'c2long', 'c2conv', 'c2tight'):
        spec = configs.config2_columns(ncols=1, seed=2)[0]
    elif tag == 'c2slow':
        # a column of the 512-column batch that has not converged after 4000 steps
        # on the device (nz = 62, T 1602 -> 1303 K, Kzz 6.9e6)
        spec = configs.config2_columns(ncols=512, seed=2)[60]
    elif tag in ('c3s', 'c3rt'):
        # the sulfur network (SNCHO, photolysis slots present with J = 0) on a
        # 40-layer column with H2S in the start
        import dataclasses
        spec = dataclasses.replace(configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0],
                                   network='SNCHO_photo_network.txt', use_photo=True,
                                   atom_list=['H', 'O', 'C', 'He', 'N', 'S'],
                                   const_mix={'H2': 0.85, 'He': 0.145, 'H2O': 1e-3, 'CH4': 5e-4,
                                              'NH3': 1e-4, 'H2S': 3e-5},
                                   conver_ignore=[])
        snet = Network.from_file(os.path.join(ref_root, 'thermo', spec.network), use_photo=True)
        spec.photo_J = {key: np.zeros(spec.pco.size) for key in sorted(snet.photo_index())}
    elif tag == 'snchok':
        import dataclasses
        spec = dataclasses.replace(configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0],
                                   network='SNCHO_photo_network.txt', use_photo=True,
                                   atom_list=['H', 'O', 'C', 'He', 'N', 'S'])
    elif tag == 'rmlist':
        spec = configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0]
    elif tag == 'lowT':
        # a cold column (150 -> 450 K) crossing the three low-temperature caps
        spec = configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0]
        spec.Tco = configs.linear_logp_T(spec.pco, 450., 150.)
    elif tag in NET_TAGS:
        import dataclasses
        fname = NET_TAGS[tag]
        photo_net = 'photo' in fname
        spec = dataclasses.replace(configs.config2_columns(ncols=1, seed=2, nz_range=(8, 8))[0],
                                   network=fname, use_photo=photo_net, atom_list=net_atoms(fname),
                                   const_mix={'H2': 0.9, 'He': 0.1}, conver_ignore=[])
        if photo_net:
            pnet = Network.from_file(os.path.join(ref_root, 'thermo', fname), use_photo=True)
            spec.photo_J = configs.photo_J_profile(np.random.default_rng(3), spec.pco,
                                                   sorted(pnet.photo_index()))
    elif tag in ATT_TAGS:
        import dataclasses
        fname = ATT_TAGS[tag]
        spec = dataclasses.replace(configs.config2_columns(ncols=1, seed=2, nz_range=(20, 20))[0],
                                   network=fname, use_photo=True, atom_list=net_atoms(fname),
                                   const_mix=family_mix(fname), conver_ignore=[])
        pnet = Network.from_file(os.path.join(ref_root, 'thermo', fname), use_photo=True)
        spec.photo_J = configs.photo_J_profile(np.random.default_rng(5), spec.pco,
                                               sorted(pnet.photo_index()))
    elif tag in SYN_TAGS:
        from vulcan_gb300 import synthnet
        syn_dir = os.path.join(workdir, 'syn150')
        snet = Network.from_file(synthnet.generate(syn_dir), use_photo=True)
        spec = configs.config4_columns(sorted(snet.photo_index()), ncols=1, nz=20)[0]
    elif tag in ('c1', 'c1rt', 'c1rtT', 'c1rtA'):
        net = Network.from_file(os.path.join(ref_root, 'thermo', 'NCHO_photo_network.txt'),
                                use_photo=True)
        spec = configs.config1(sorted(net.photo_index()))
    else:
        raise ValueError(tag)
    net = Network.from_file(os.path.join(syn_dir or os.path.join(ref_root, 'thermo'), spec.network),
                            use_photo=spec.use_photo)
    dst = run_reference(ref_root, tag, spec, NSTEPS[tag], KEEP[tag], workdir, syn_dir)
    d = dict(np.load(os.path.join(dst, 'golden_out.npz'), allow_pickle=False))
    if tag in NET_TAGS:
        if spec.photo_J:
            keys = sorted(spec.photo_J)
            d['photo_sp'] = np.array([k[0] for k in keys])
            d['photo_br'] = np.array([k[1] for k in keys])
        d['atom_list'] = np.array(spec.atom_list)
        out = os.path.join(HERE, 'golden_%s.npz' % tag)
        np.savez_compressed(out, **d)
        net.to_npz(os.path.join(HERE, 'net_%s.npz' % tag[2:]))
        print('wrote', out, os.path.getsize(out) // 1024, 'KiB')
        return
    if tag in RATE_TAGS:
        out = os.path.join(HERE, 'golden_%s.npz' % tag)
        np.savez_compressed(out, **d)
        net.to_npz(os.path.join(HERE, 'net_%s.npz' % spec.network.replace('_network.txt', '')))
        print('wrote', out, os.path.getsize(out) // 1024, 'KiB')
        return
    if tag in PHOTO_TAGS:
        d = slim_photo(d)
        d.update(photo_setup_check(d, ref_root))
        out = os.path.join(HERE, 'golden_%s.npz' % tag)
        np.savez_compressed(out, **d)
        print('wrote', out, os.path.getsize(out) // 1024, 'KiB')
        return
    if tag == 'c0vul':
        # the file the reference wrote (protocol-4 pickle of var_save, vars(atm),
        # vars(para)) next to the state it was written from
        src = os.path.join(dst, 'output', 'golden.vul')
        shutil.copy(src, os.path.join(HERE, 'golden_c0vul.vul'))
        np.savez_compressed(os.path.join(HERE, 'golden_c0vul.npz'), final_y=d['final_y'],
                            final_ymix=d['final_ymix'], final_t=d['final_t'],
                            final_count=d['final_count'], end_case=d['end_case'], k=d['k'],
                            y_ini=d['y_ini'], atom_list=np.array(spec.atom_list))
        print('wrote', os.path.join(HERE, 'golden_c0vul.vul'),
              os.path.getsize(os.path.join(HERE, 'golden_c0vul.vul')) // 1024, 'KiB')
        return
    d['atom_list'] = np.array(spec.atom_list)
    d['conver_ignore'] = np.array(spec.conver_ignore, dtype='U16')
    d['const_mix_sp'] = np.array(list(spec.const_mix))
    d['const_mix_x'] = np.array(list(spec.const_mix.values()))
    if spec.photo_J:
        keys = sorted(spec.photo_J)
        d['photo_sp'] = np.array([k[0] for k in keys])
        d['photo_br'] = np.array([k[1] for k in keys])
    out = os.path.join(HERE, 'golden_%s.npz' % tag)
    np.savez_compressed(out, **d)
    if tag in ATT_TAGS:                   # the same tables as the n_ fixture of the network
        net.to_npz(os.path.join(HERE, 'net_%s.npz' % tag[2:]))
        print('wrote', out, os.path.getsize(out) // 1024, 'KiB')
        return
    net.to_npz(os.path.join(HERE, 'net_%s.npz' % (
        spec.network.replace('_network.txt', '')
        + ('_photo' if spec.use_photo and 'photo' not in spec.network else ''))))
    if full_dir and tag not in ('c2conv', 'c2tight', 'c2slow'):
        os.makedirs(full_dir, exist_ok=True)
        shutil.copy(os.path.join(dst, 'golden_full.npz'),
                    os.path.join(full_dir, 'golden_full_%s.npz' % tag))
    print('wrote', out, os.path.getsize(out) // 1024, 'KiB')


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('tags', nargs='*', default=['c0', 'c1', 'c2'])
    ap.add_argument('--ref', default=os.environ.get('VULCAN_REFERENCE'),
                    help='the VULCAN source tree (default: $VULCAN_REFERENCE)')
    ap.add_argument('--full-dir', default=None,
                    help='also keep every recorded attempt here (not committed)')
    ap.add_argument('--setup-only', action='store_true',
                    help='radiative-transfer fixtures: recompute only the host set-up '
                         'comparisons of an existing fixture (no reference run)')
    a = ap.parse_args()
    if not a.ref or not os.path.isfile(os.path.join(a.ref, 'op.py')):
        ap.error('give the VULCAN source tree with --ref or VULCAN_REFERENCE (got %r)' % a.ref)
    if a.setup_only:
        for t in a.tags:
            path = os.path.join(HERE, 'golden_%s.npz' % t)
            d = dict(np.load(path, allow_pickle=False))
            d.update(photo_setup_check(d, a.ref))
            np.savez_compressed(path, **d)
            print('updated', path)
        return
    with tempfile.TemporaryDirectory() as w:
        for t in a.tags:
            make(t, a.ref, w, a.full_dir)


if __name__ == '__main__':
    main()
