"""`.vul` output and `vulcan_ini` restart, the reference's file seam.

The reference saves a run as a pickle (protocol 4) of
``{'variable': var_save, 'atm': vars(atm), 'parameter': vars(para)}``
(op.Output.save_out, op.py:3216-3256), with ``var_save`` holding
``species``, ``nr`` and the fields of store.Variables.var_save (store.py:83):
``k`` (dict reaction index -> [nz]), ``y``, ``ymix``, ``y_ini``, ``t``, ``dt``,
``longdy``, ``longdydt``, ``atom_ini``, ``atom_sum``, ``atom_loss``,
``atom_conden`` (dicts over atom_list), ``aflux_change`` and ``Rf`` (dict
reaction index -> text), with photochemistry also the radiative-transfer
entries (store.py:85-86, ``photo_fields``).  Downstream scripts (the
reference's plot_py/) read ``variable['ymix']``, ``variable['species']``,
``atm['pco']``, ``atm['zco']``, ``atm['zmco']`` and friends.

``ini_mix = 'vulcan_ini'`` (build_atm.py:166-181) starts a run from the ``y``
of such a file, species matched by name; :func:`read_vul_y` does the same.
"""
from __future__ import annotations

import pickle

import numpy as np

ATM_KEYS = ('pco', 'pico', 'Tco', 'Kzz', 'vz', 'M', 'n_0', 'mu', 'g', 'Hp', 'dz', 'zco',
            'dzi', 'Dzz', 'Dzz_cen', 'ms', 'alpha', 'Ti', 'Hpi', 'top_flux', 'bot_flux',
            'bot_vdep', 'pref_indx', 'gs', 'Rp')
# atm entries of the reference's file for options this step does not run
# (condensation, fixed species, molecular-diffusion advection and settling
# velocities): written as the reference writes them when those are off
CONDENSE_DICT_KEYS = ('conden_min_lev', 'fix_sp_indx', 'r_p', 'rho_p', 'sat_mix', 'sat_p')


PHOTO_KEYS = ('nbin', 'bins', 'dbin1', 'dbin2', 'tau', 'sflux', 'aflux', 'cross', 'cross_scat',
              'cross_J', 'J_sp', 'n_branch')


def photo_fields(tables, tau, aflux, J):
    """The photochemistry entries of var_save (store.py:85-86) for one column:
    ``tables`` a photo.PhotoTables, ``tau`` [nz+1, nbins], ``aflux`` [nz,
    nbins] and ``J`` [nz, nch] of that column (Ros2Handle.photo_get rows)."""
    chans = list(zip(tables.ch_sp, tables.ch_br))
    sflux = tables.sflux_top * np.exp(-1. * tau / np.cos(tables.sl_angle))
    J_sp = {(sp, 0): np.zeros(aflux.shape[0]) for sp in tables.absp_sp}
    n_branch = {sp: 0 for sp in tables.absp_sp}
    for c, (sp, br) in enumerate(chans):
        J_sp[(sp, br)] = np.array(J[:, c])
        J_sp[(sp, 0)] = J_sp[(sp, 0)] + J[:, c]
        n_branch[sp] = max(n_branch[sp], br)
    return {'nbin': len(tables.bins), 'bins': np.array(tables.bins),
            'dbin1': float(tables.dbin1), 'dbin2': float(tables.dbin2),
            'tau': np.array(tau), 'sflux': sflux, 'aflux': np.array(aflux),
            'cross': {sp: np.array(tables.cross[i]) for i, sp in enumerate(tables.absp_sp)},
            'cross_scat': {sp: np.array(tables.cross_scat[i]) for i, sp in enumerate(tables.scat_sp)},
            'cross_J': {c: np.array(tables.cross_J[i]) for i, c in enumerate(chans)},
            'J_sp': J_sp, 'n_branch': n_branch}


def vul_dict(net, item, y, ymix, t, dt, count, end_case, atom_list, longdy=0.0, longdydt=0.0,
             delta=0.0, photo=None, counters=None):
    """The save_out dictionary of one column (state arrays [nz, ni]); with
    ``photo`` (photo_fields) also the photochemistry entries; ``counters``
    (the column's row of Ros2Handle.counters()) adds the rejection counts the
    reference keeps in para (delta_count, nega_count, loss_count)."""
    from .column import atom_totals
    col = item['col']
    k = item['k']
    atom_sum = atom_totals(net, y, atom_list)
    atom_ini = np.asarray(item['atom_ini'], dtype=float)
    var = {'species': list(net.species), 'nr': net.nr,
           'k': {i + 1: np.array(k[i]) for i in range(k.shape[0])},
           'y': np.array(y), 'ymix': np.array(ymix),
           'y_ini': np.array(item.get('y_ini', item['y'])),
           't': float(t), 'dt': float(dt), 'longdy': float(longdy), 'longdydt': float(longdydt),
           'atom_ini': {a: float(v) for a, v in zip(atom_list, atom_ini)},
           'atom_sum': {a: float(v) for a, v in zip(atom_list, atom_sum)},
           'atom_loss': {a: float((s - i) / i) for a, s, i in zip(atom_list, atom_sum, atom_ini)},
           'atom_conden': {a: 0.0 for a in atom_list},
           'aflux_change': 0.0,
           'Rf': {r.index: r.text for r in net.reactions}}
    if photo is not None:
        var.update(photo)
    atm = {key: np.array(getattr(col, key)) if hasattr(getattr(col, key, None), '__len__')
           else getattr(col, key) for key in ATM_KEYS if hasattr(col, key)}
    if getattr(col, 'zco', None) is not None:      # layer mid-points (f_mu_dz's zmco)
        z = np.asarray(col.zco)
        atm['zmco'] = 0.5 * (z[:-1] + z[1:])
    nz, ni = np.asarray(y).shape
    atm['vm'] = np.zeros((nz, ni))
    atm['vs'] = np.zeros((nz - 1, ni))
    atm['bot_fix_sp'] = np.zeros(ni)
    atm['gas_indx'] = list(range(ni))
    for key in CONDENSE_DICT_KEYS:
        atm[key] = {}
    para = {'count': int(count), 'end_case': int(end_case), 'delta': float(delta),
            'solver_str': 'Ros2GPU'}
    if counters is not None:       # attempts, delta / negativity / loss rejections, ...
        para.update(delta_count=int(counters[1]), nega_count=int(counters[2]),
                    loss_count=int(counters[3]))
    return {'variable': var, 'atm': atm, 'parameter': para}


def write_vul(path, data):
    with open(path, 'wb') as f:
        pickle.dump(data, f, protocol=4)


def write_batch(paths, net, items, state, atom_list, conv=None, photo=None, counters=None):
    """One .vul per column of a batch state (Ros2Handle.state()); ``paths``
    lists the file names; ``conv`` = (longdy, longdydt) per column; ``photo``
    = (tables, tau, aflux, J) of the batch (Ros2Handle.photo_get) adds the
    photochemistry entries; ``counters`` = Ros2Handle.counters() the
    rejection counts."""
    off = np.concatenate([[0], np.cumsum([it['col'].nz for it in items])])
    for c, (path, it) in enumerate(zip(paths, items)):
        sl = slice(off[c], off[c + 1])
        ld = conv[0][c] if conv is not None else 0.0
        ldt = conv[1][c] if conv is not None else 0.0
        ph = None
        if photo is not None:
            tables, tau, aflux, J = photo
            # staggered rows of column c start at off[c] + c (nz + 1 of them)
            ph = photo_fields(tables, tau[off[c] + c:off[c + 1] + c + 1], aflux[sl], J[sl])
        write_vul(path, vul_dict(net, it, state['y'][sl], state['ymix'][sl], state['t'][c],
                                 state['dt'][c], state['count'][c], state['end_case'][c],
                                 atom_list, ld, ldt, state['delta'][c], photo=ph,
                                 counters=None if counters is None else counters[c]))


def read_vul_y(path, species, nz=None):
    """y [nz, len(species)] from a .vul file, species matched by name (a
    species the file does not hold stays 0 and is listed in the second
    return value), as ini_mix = 'vulcan_ini' does."""
    with open(path, 'rb') as f:
        d = pickle.load(f)
    v = d['variable']
    src = v['species']
    y_src = np.asarray(v['y'])
    if nz is not None and y_src.shape[0] != nz:
        raise ValueError('%s has %d layers, the run %d' % (path, y_src.shape[0], nz))
    y = np.zeros((y_src.shape[0], len(species)))
    missing = []
    for i, sp in enumerate(species):
        if sp in src:
            y[:, i] = y_src[:, src.index(sp)]
        else:
            missing.append(sp)
    return y, missing
