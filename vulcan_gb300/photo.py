"""Photochemistry radiative transfer: host set-up of the tables the device
path (vk_photo_setup / vk_photo_update) runs on.

Restates the reference's make_bins_read_cross (op.py:495-782) and read_sflux
(build_atm.py:617-656) for T-independent cross sections without
photoionisation (the reference's defaults: T_cross_sp = [], use_ion = False);
the per-layer temperature-dependent tables of T_cross_sp come from TCross (the
same function's T branch) or as given, e.g. the reference's own var.cross_T /
var.cross_J_T, and are uploaded by attach_cross_T:

* bins: from the shortest absorption edge (not below the stellar file's
  first wavelength or 2 nm) to min(longest edge, the file's last wavelength
  or 700 nm, the longest photolysis threshold), step dbin1 below dbin_12trans
  and dbin2 above;
* cross sections interpolated linearly onto the bins with zero outside the
  tabulated range; branch cross sections = dissociation cross section x the
  branching ratio (held constant beyond its table);
* top-of-atmosphere flux: the stellar surface flux x (r_star R_sun / (a AU))^2
  interpolated onto the bins.

The J integral's bin weights follow the reference's four-part trapezoid sums
(op.py:2770-2773), including its index semantics when dbin_12trans lies
outside the bins.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

R_SUN = 6.957E10          # cm (phy_const.py)
AU = 1.49597871E13         # cm (phy_const.py)


def _interp(x, xp, fp, left=0.0, right=0.0):
    """Linear interpolation as the reference's scipy interp1d does it: the
    table sorted by its abscissa first (stable; a few of the reference's
    tables are not in order), ``left`` / ``right`` outside it."""
    o = np.argsort(xp, kind='mergesort')
    return np.interp(x, np.asarray(xp)[o], np.asarray(fp)[o], left=left, right=right)


def j_weights(nbins, i12, dbin1, dbin2):
    """Weight of each bin in the reference's J sum (see module docstring)."""
    w = np.zeros(nbins)
    idx = np.arange(nbins)
    w[idx[:i12]] += dbin1
    w[idx[0]] -= 0.5 * dbin1
    w[idx[i12 - 1]] -= 0.5 * dbin1
    w[idx[i12:]] += dbin2
    w[idx[i12]] -= 0.5 * dbin2
    w[idx[-1]] -= 0.5 * dbin2
    return w


@dataclass
class PhotoTables:
    bins: np.ndarray
    dbin1: float
    dbin2: float
    i12: int                  # index of dbin_12trans in bins (-1 if outside)
    sflux_top: np.ndarray
    absp_sp: list             # absorbers (photolysis species)
    cross: np.ndarray         # [nabs, nbins]
    scat_sp: list
    cross_scat: np.ndarray    # [nscat, nbins]
    ch_sp: list               # photolysis channels
    ch_br: list
    cross_J: np.ndarray       # [nch, nbins]
    sl_angle: float
    edd: float
    f_diurnal: float
    flux_atol: float

    def weights(self):
        return j_weights(len(self.bins), self.i12, self.dbin1, self.dbin2)

    @classmethod
    def from_fixture(cls, d):
        """Tables recorded from the reference's own set-up (tests/golden)."""
        absp = [str(s) for s in d['absp_sp']]
        return cls(bins=np.asarray(d['bins'], float), dbin1=float(d['dbin1']),
                   dbin2=float(d['dbin2']), i12=int(d['sflux_din12_indx']),
                   sflux_top=np.asarray(d['sflux_top'], float), absp_sp=absp,
                   cross=np.asarray(d['cross'], float), scat_sp=[str(s) for s in d['scat_sp']],
                   cross_scat=np.asarray(d['cross_scat'], float),
                   ch_sp=[str(s) for s in d['ch_sp']], ch_br=[int(b) for b in d['ch_br']],
                   cross_J=np.asarray(d['cross_J'], float), sl_angle=float(d['sl_angle']),
                   edd=float(d['edd']), f_diurnal=float(d['f_diurnal']),
                   flux_atol=float(d['flux_atol']))

    @classmethod
    def from_reference_files(cls, net, ref_root, sflux_file, r_star, orbit_radius,
                             sl_angle, scat_sp=('H2', 'He'), edd=0.5, dbin1=0.1, dbin2=2.0,
                             dbin_12trans=240.0, f_diurnal=1.0, flux_atol=1.0,
                             cross_folder='thermo/photo_cross/'):
        """Tables from the reference's data layout (cross-section folder,
        thresholds.txt, rayleigh/ and a stellar flux file), for the photolysis
        channels of ``net`` (Network.from_file(..., use_photo=True))."""
        cf = os.path.join(ref_root, cross_folder)
        chans = sorted(net.photo_index())
        photo_sp = sorted({sp for sp, _ in chans})
        lab = np.genfromtxt(os.path.join(cf, 'thresholds.txt'), dtype=str, usecols=0)
        thr = np.genfromtxt(os.path.join(cf, 'thresholds.txt'), skip_header=1)[:, 1]
        threshold = {l: v for l, v in zip(lab, thr) if l in net.species}
        sraw = np.genfromtxt(os.path.join(ref_root, sflux_file), dtype=float, skip_header=1,
                             names=['lambda', 'flux'])
        def_min, def_max = max(sraw['lambda'][0], 2.), min(sraw['lambda'][-1], 700.)
        raw, ratio = {}, {}
        bin_min = bin_max = diss_max = None
        for sp in photo_sp:
            raw[sp] = np.genfromtxt(os.path.join(cf, sp, sp + '_cross.csv'), dtype=float,
                                    delimiter=',', skip_header=1, names=['lambda', 'cross', 'disso'])
            ratio[sp] = np.genfromtxt(os.path.join(cf, sp, sp + '_branch.csv'), dtype=float,
                                      delimiter=',', skip_header=1, names=True)
            lo, hi = raw[sp]['lambda'][0], raw[sp]['lambda'][-1]
            bin_min = lo if bin_min is None else min(bin_min, lo)
            bin_max = hi if bin_max is None else max(bin_max, hi)
            diss_max = threshold[sp] if diss_max is None else max(diss_max, threshold[sp])
        bin_min = max(bin_min, def_min)
        bin_max = min(bin_max, def_max, diss_max)
        if bin_min <= dbin_12trans <= bin_max:
            bins = np.concatenate((np.arange(bin_min, dbin_12trans, dbin1),
                                   np.arange(dbin_12trans, bin_max, dbin2)))
        else:
            bins = np.arange(bin_min, bin_max, dbin1)
        interp0 = lambda x, xp, fp: _interp(x, xp, fp)
        cross = np.array([interp0(bins, raw[sp]['lambda'], raw[sp]['cross']) for sp in photo_sp])
        cross_J = []
        for sp, br in chans:
            key = 'br_ratio_%d' % br
            # held at the table's first and last rows as written (fill_value)
            r = _interp(bins, ratio[sp]['lambda'], ratio[sp][key],
                        ratio[sp][key][0], ratio[sp][key][-1])
            cross_J.append(interp0(bins, raw[sp]['lambda'], raw[sp]['disso']) * r)
        scat = []
        for sp in scat_sp:
            s = np.genfromtxt(os.path.join(cf, 'rayleigh', sp + '_scat.txt'), dtype=float,
                              skip_header=1, names=['lambda', 'cross'])
            scat.append(interp0(bins, s['lambda'], s['cross']))
        top = interp0(bins, sraw['lambda'], sraw['flux'] * (r_star * R_SUN / (AU * orbit_radius)) ** 2)
        hit = np.nonzero(bins == dbin_12trans)[0]
        return cls(bins=bins, dbin1=dbin1, dbin2=dbin2, i12=int(hit[-1]) if hit.size else -1,
                   sflux_top=top, absp_sp=photo_sp, cross=cross, scat_sp=list(scat_sp),
                   cross_scat=np.array(scat), ch_sp=[c[0] for c in chans],
                   ch_br=[c[1] for c in chans], cross_J=np.array(cross_J), sl_angle=sl_angle,
                   edd=edd, f_diurnal=f_diurnal, flux_atol=flux_atol)


class TCross:
    """Temperature-dependent cross sections (vulcan_cfg.T_cross_sp) of one
    column, restating the T branch of make_bins_read_cross (files op.py:542-557,
    per-layer tables op.py:640-747).  A species' tables are its
    ``<sp>_cross_<T>K.csv`` files plus the room-temperature file as 300 K.
    For a layer at T:

    * T between two tabulated temperatures (Tlow <= T < Thigh): inside the
      wavelengths both tables cover, log10 of the cross section linear in T
      (log10 0 taken as -100, a result of -100 giving 0), the branch ratio as
      for the T-independent channels; outside, the T-independent values;
    * T at or below every tabulated temperature: the lowest table (its own
      wavelength range) unless that is the 300 K one, which means the
      T-independent values; likewise above every temperature with the highest.
    """

    def __init__(self, tables, raw, ratio):
        self.tables = tables
        self.raw = raw            # sp -> {T: (lambda, cross, disso)}
        self.ratio = ratio        # (sp, branch) -> branch ratio on the bins

    @classmethod
    def from_reference_files(cls, tables, ref_root, T_cross_sp,
                             cross_folder='thermo/photo_cross/'):
        import re
        read = lambda path: np.genfromtxt(path, dtype=float, delimiter=',', skip_header=1,
                                          usecols=(0, 1, 2)).T
        raw, ratio = {}, {}
        for sp in T_cross_sp:
            if sp not in tables.absp_sp:
                continue
            d = os.path.join(ref_root, cross_folder, sp)
            tabs = {}
            for name in os.listdir(d):
                m = re.fullmatch(re.escape(sp) + r'_cross_(\d+)K\.csv', name)
                if m:
                    tabs[int(m.group(1))] = read(os.path.join(d, name))
            tabs[300] = read(os.path.join(d, sp + '_cross.csv'))
            raw[sp] = tabs
            br = np.genfromtxt(os.path.join(d, sp + '_branch.csv'), dtype=float, delimiter=',',
                               skip_header=1, names=True)
            for s, b in zip(tables.ch_sp, tables.ch_br):
                if s == sp:
                    key = 'br_ratio_%d' % b
                    ratio[(s, b)] = _interp(tables.bins, br['lambda'], br[key],
                                            br[key][0], br[key][-1])
        return cls(tables, raw, ratio)

    def for_column(self, Tco):
        """(cross_T {sp: [nz, nbins]}, cross_J_T {(sp, branch): [nz, nbins]})."""
        t = self.tables
        bins = t.bins
        interp0 = lambda tab, col: _interp(bins, tab[0], tab[col])
        cross_T, cross_J_T = {}, {}
        for sp, tabs in self.raw.items():
            base = t.cross[t.absp_sp.index(sp)]
            chans = [(i, (s, b)) for i, (s, b) in enumerate(zip(t.ch_sp, t.ch_br)) if s == sp]
            Ts = np.array(sorted(tabs), dtype=float)
            ct = np.zeros((len(Tco), len(bins)))
            cj = {c: np.zeros((len(Tco), len(bins))) for _, c in chans}
            for lev, Tz in enumerate(Tco):
                lo, hi = Ts[Ts <= Tz], Ts[Ts > Tz]
                if lo.size and hi.size:
                    A, B = tabs[int(lo.max())], tabs[int(hi.min())]
                    inside = (bins >= max(A[0][0], B[0][0])) & (bins <= min(A[0][-1], B[0][-1]))
                    frac = lambda la, lb: (lb - la) / (hi.min() - lo.max()) * (Tz - lo.max()) + la
                    with np.errstate(divide='ignore'):
                        v = frac(_log10_floor(interp0(A, 1)), _log10_floor(interp0(B, 1)))
                        vj = frac(_log10_floor(interp0(A, 2)), _log10_floor(interp0(B, 2)))
                    row = np.where(v == -100, 0.0, 10 ** v)
                    rowj = np.where(vj == -100, 0.0, 10 ** vj)
                    ct[lev] = np.where(inside, row, base)
                    for i, c in chans:
                        cj[c][lev] = np.where(inside, rowj * self.ratio[c], t.cross_J[i])
                else:
                    edge = Ts.min() if not (Ts < Tz).any() else Ts.max()
                    if edge == 300:
                        ct[lev] = base
                        for i, c in chans:
                            cj[c][lev] = t.cross_J[i]
                        continue
                    E = tabs[int(edge)]
                    inside = (bins >= E[0][0]) & (bins <= E[0][-1])
                    ct[lev] = np.where(inside, interp0(E, 1), base)
                    for i, c in chans:
                        cj[c][lev] = np.where(inside, interp0(E, 2) * self.ratio[c], t.cross_J[i])
            cross_T[sp] = ct
            cross_J_T.update(cj)
        return cross_T, cross_J_T

    def for_columns(self, Tcos):
        """for_column of every column of a batch, layers stacked in batch
        order (the [L, nbins] tables attach_cross_T uploads)."""
        parts = [self.for_column(T) for T in Tcos]
        cross_T = {sp: np.concatenate([p[0][sp] for p in parts]) for sp in parts[0][0]}
        cross_J_T = {c: np.concatenate([p[1][c] for p in parts]) for c in parts[0][1]}
        return cross_T, cross_J_T


def _log10_floor(x):
    """log10 with -inf replaced by -100, as the reference does before
    interpolating in temperature."""
    v = np.log10(x)
    v[np.isinf(v)] = -100.
    return v


def attach(handle, tables, net):
    """vk_photo_setup on a Ros2Handle for the network's species and channels."""
    from .capi import check, lib, ptr
    sp = {s: i for i, s in enumerate(net.species)}
    pidx = net.photo_index()
    abs_sp = np.array([sp[s] for s in tables.absp_sp], dtype=np.int32)
    abs_photo = np.ones(len(abs_sp), dtype=np.int32)
    scat_sp = np.array([sp[s] for s in tables.scat_sp], dtype=np.int32)
    kidx = np.array([pidx[(s, b)] for s, b in zip(tables.ch_sp, tables.ch_br)], dtype=np.int32)
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    check(lib().vk_photo_setup(
        handle.h, len(tables.bins), ptr(c(tables.bins)), ptr(c(tables.weights())),
        len(abs_sp), ptr(abs_sp, C.c_int), ptr(abs_photo, C.c_int), ptr(c(tables.cross)),
        len(scat_sp), ptr(scat_sp, C.c_int), ptr(c(tables.cross_scat)),
        len(kidx), ptr(kidx, C.c_int), ptr(c(tables.cross_J)), ptr(c(tables.sflux_top)),
        tables.sl_angle, tables.edd, tables.f_diurnal, tables.flux_atol), handle.h)
    handle.photo_dims = (len(tables.bins), len(kidx))
    handle.photo_tables = tables


def attach_cross_T(handle, cross_T, cross_J_T):
    """vk_photo_set_cross_T for the handle's current batch: cross_T {absorber:
    [L, nbins]} and cross_J_T {(species, branch): [L, nbins]} -- the
    reference's var.cross_T / var.cross_J_T (op.py:640-745), the layers of the
    batch's columns stacked in batch order.  Empty dicts remove the tables."""
    from .capi import check, lib, ptr
    t = handle.photo_tables
    L, nb = handle.batch.L, len(t.bins)
    chans = list(zip(t.ch_sp, t.ch_br))
    aslot = np.array([t.absp_sp.index(sp) for sp in cross_T], dtype=np.int32)
    cslot = np.array([chans.index(tuple(c)) for c in cross_J_T], dtype=np.int32)

    def stack(tab):
        if not tab:
            return None
        a = np.ascontiguousarray(np.array([tab[key] for key in tab], dtype=np.float64))
        if a.shape[1:] != (L, nb):
            raise ValueError('per-layer cross sections must be [L, nbins] = [%d, %d]' % (L, nb))
        return a

    ct, cj = stack(cross_T), stack(cross_J_T)
    check(lib().vk_photo_set_cross_T(handle.h, len(aslot), ptr(aslot, C.c_int), ptr(ct),
                                     len(cslot), ptr(cslot, C.c_int), ptr(cj)), handle.h)
