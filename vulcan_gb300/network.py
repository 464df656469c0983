"""VULCAN network-file compiler: text network -> reaction tables + FP64 rate constants.

Reads the same text format as the reference (``thermo/*_network.txt``):

    id  [ A + B -> C + D ]  A  B  C  [A_inf B_inf C_inf]  ref ...

with section markers ``# 3-body``, ``# 3-body reactions without high-pressure
rates``, ``# special``, ``# condensation``, ``# radiative``, ``# photo``,
``# ionisation`` and ``# reverse stops``, ``2*X`` stoichiometry and the ``M``
third-body pseudo-species.  Reactions are numbered 1, 3, 5, ... (forward);
k index ``i+1`` is the reverse of ``i``.

Semantics follow the reference's code generator and rate reader:
  * species order = order of first appearance in the chemistry table
    (make_chem_funs.py:155-165, chem_dict);
  * which reactions enter the chemistry (photo/ion lines only with photo on)
    (make_chem_funs.py:36-105);
  * forward rates k = A T^B exp(-C/T), Lindemann fall-off k0/(1+k0 M/kinf),
    the hard-coded ``OH + CH3 + M -> CH3OH + M`` form (op.py:135-212);
  * reverse rates k_{i+1} = k_i / Keq with
    Keq = exp(-(sum nu_p g_p - sum nu_r g_r)) (corr T)^(n_r - n_p)
    (make_chem_funs.py:568-580, op.py:287-309, chem_funs Gibbs/gibbs_sp),
    g/RT from two-range NASA-9 polynomials switched at 1000 K;
  * reverse rates beyond ``# reverse stops`` are zero; ``remove_list`` zeroes
    rates (op.py:312-318); optional low-T caps (op.py:320-342).

Everything here runs once per network / per column on the host in FP64.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

# Physical constants in cgs, same values as the reference's phy_const.py.
KB = 1.38064852E-16
NAVO = 6.02214086E+23
CORR = KB / 1.0e6          # gibbs_text.txt:1  (P0 = 1 bar)

SPECIAL_OH_CH3 = 'OH + CH3 + M -> CH3OH + M'
# use_lowT_limit_rates (op.ReadRate.lim_lowT_rates, op.py:320-342): reaction
# -> (T_max, form, (A, B, C, A_inf, B_inf, C_inf)); at T <= T_max the forward
# rate becomes A T^B exp(-C/T) ('arrhenius') or the fall-off of that k0 and
# k_inf = A_inf T^B_inf exp(-C_inf/T) ('falloff') -- Moses et al. 2005 values
LOWT_CAPS = {
    'H + CH3 + M -> CH4 + M': (277.5, 'falloff', (6e-29, 0., 0., 2.06E-10, -0.4, 0.)),
    'H + C2H4 + M -> C2H5 + M': (300., 'arrhenius', (3.7E-30, 0., 0., 0., 0., 0.)),
    'H + C2H5 + M -> C2H6 + M': (200., 'arrhenius', (2.49E-27, 0., 0., 0., 0., 0.)),
}


@dataclass
class Reaction:
    index: int                      # forward k index (odd)
    text: str                       # 'A + B -> C + D'
    reac: list                      # [(nu, name)] in written order, incl. 'M'
    prod: list
    kind: str                       # arrhenius|falloff|k0|special|conden|photo|ion
    A: float = 0.0
    B: float = 0.0
    C: float = 0.0
    A_inf: float = 0.0
    B_inf: float = 0.0
    C_inf: float = 0.0
    photo_sp: str = ''
    photo_br: int = 0

    def side_factors(self, side):
        """Merged (species, exponent) list and M power for one side."""
        terms = self.reac if side == 'f' else self.prod
        merged, mpow = {}, 0
        for nu, name in terms:
            if name == 'M':
                mpow += nu
            else:
                merged[name] = merged.get(name, 0) + nu
        return list(merged.items()), mpow


def _split_terms(rf):
    """Parse 'A + 2*B + M -> C + D' into ([(nu,name)...], [(nu,name)...]).

    Mirrors make_chem_funs.py:150-176 (term.split('*'), '->' switches side)."""
    reac, prod = [], []
    cur = reac
    for term in rf.split():
        if term == '+':
            continue
        if term == '->':
            cur = prod
            continue
        parts = term.split('*')
        if len(parts) == 1:
            nu, name = 1, parts[0]
        else:
            nu, name = int(parts[0]), parts[1]
        cur.append((nu, name))
    return reac, prod


@dataclass
class Network:
    """A compiled VULCAN network (chemistry reactions only, k index 1..nr)."""
    path: str
    use_photo: bool
    species: list
    reactions: list
    stop_rev_indx: int
    nasa9: np.ndarray = None          # [ni, 20] (low 0:10, high 10:20)
    compo_atoms: list = field(default_factory=list)
    compo: np.ndarray = None          # [ni, natoms] element counts
    mass: np.ndarray = None           # [ni] molar mass

    @property
    def ni(self):
        return len(self.species)

    @property
    def nr(self):
        return 2 * len(self.reactions)

    @property
    def npair(self):
        return len(self.reactions)

    # ------------------------------------------------------------------ parse
    @classmethod
    def from_file(cls, network_path, thermo_dir=None, com_file=None,
                  use_photo=False):
        """Parse a VULCAN network text file.

        ``thermo_dir`` holds ``NASA9/<sp>.txt`` (Gibbs data); ``com_file`` is
        ``all_compose.txt`` (element counts and masses).  Both default to the
        network file's own directory, as in the reference layout."""
        if thermo_dir is None:
            thermo_dir = os.path.dirname(os.path.abspath(network_path))
        if com_file is None:
            com_file = os.path.join(thermo_dir, 'all_compose.txt')
        with open(network_path) as f:
            lines = f.readlines()
        reactions, stop_rev = cls._parse_lines(lines, use_photo)
        species = []
        seen = set()
        for r in reactions:
            for nu, name in r.reac + r.prod:
                if name != 'M' and name not in seen:
                    seen.add(name)
                    species.append(name)
        net = cls(path=os.path.abspath(network_path), use_photo=use_photo,
                  species=species, reactions=reactions,
                  stop_rev_indx=stop_rev)
        net._load_nasa9(os.path.join(thermo_dir, 'NASA9'))
        net._load_compo(com_file)
        return net

    @staticmethod
    def _parse_lines(lines, use_photo):
        """Section-marker state machine of make_chem_funs.read_network
        (make_chem_funs.py:17-110) combined with the coefficient reading of
        op.ReadRate.read_rate (op.py:85-283)."""
        i = 1
        re_tri = re_tri_k0 = False
        special = conden = photo = ion = False
        stop_rev = None
        out = []
        for line in lines:
            if line.startswith('# 3-body'):
                re_tri = True
            if line.startswith('# 3-body reactions without high-pressure rates'):
                re_tri_k0 = True
            elif line.startswith('# special'):
                re_tri = re_tri_k0 = False
                special = True
            elif line.startswith('# condensation'):
                re_tri = re_tri_k0 = False
                special = False
                conden = True
            elif line.startswith('# radiative'):
                re_tri = re_tri_k0 = False
                special = conden = False
            elif line.startswith('# photo'):
                re_tri = re_tri_k0 = False
                special = conden = False
                photo = True
            elif line.startswith('# ionisation'):
                re_tri = re_tri_k0 = False
                special = conden = photo = False
                ion = True
            elif line.startswith('# reverse stops'):
                stop_rev = i
            if line.startswith('#') or not line.strip():
                continue
            rf = line.partition('[')[-1].rpartition(']')[0].strip()
            reac, prod = _split_terms(rf)
            cols = line.partition(']')[-1].split()
            r = Reaction(index=i, text=rf, reac=reac, prod=prod, kind='arrhenius')
            if special:
                r.kind = 'special'
            elif conden:
                r.kind = 'conden'
            elif photo or ion:
                r.kind = 'photo' if photo else 'ion'
                r.photo_sp = cols[0]
                r.photo_br = int(cols[1])
            else:
                r.A, r.B, r.C = float(cols[0]), float(cols[1]), float(cols[2])
                if re_tri and not re_tri_k0:
                    r.A_inf, r.B_inf, r.C_inf = (float(cols[3]), float(cols[4]),
                                                 float(cols[5]))
                    r.kind = 'falloff'
                elif re_tri:
                    if len(cols) >= 6:
                        # op.py:162 would read an undefined k_inf here.
                        raise ValueError('3-body (k0 only) line with >=6 columns: ' + rf)
                    r.kind = 'k0'
            # photo / ion lines enter the chemistry only with photochemistry on
            # (make_chem_funs.py:76-79)
            if (photo or ion) and not use_photo:
                i += 2
                continue
            out.append(r)
            i += 2
        if stop_rev is None:
            raise ValueError("network has no '# reverse stops' marker")
        return out, stop_rev

    def _load_nasa9(self, nasa_dir):
        rows = []
        for sp in self.species:
            a = np.loadtxt(os.path.join(nasa_dir, sp + '.txt')).flatten()
            if a.size < 20:
                raise ValueError('NASA-9 file for %s has %d numbers' % (sp, a.size))
            # only the first two ranges are used (chem_funs nasa9[i,'low'/'high'])
            rows.append(a[:20])
        self.nasa9 = np.array(rows, dtype=np.float64)

    def _load_compo(self, com_file):
        with open(com_file) as f:
            header = f.readline().split()
            table = {}
            for line in f:
                t = line.split()
                if t:
                    table[t[0]] = t[1:]
        atoms = header[1:-1]
        self.compo_atoms = atoms
        comp = np.zeros((self.ni, len(atoms)))
        mass = np.zeros(self.ni)
        missing = [sp for sp in self.species if sp not in table]
        if missing:      # the reference fails here too (compo_row.index, build_atm.py)
            raise ValueError('species not in the composition file %s: %s'
                             % (com_file, ', '.join(missing)))
        for k, sp in enumerate(self.species):
            row = table[sp]
            comp[k] = [int(v) for v in row[:len(atoms)]]
            mass[k] = float(row[len(atoms)])
        self.compo = comp
        self.mass = mass

    # --------------------------------------------------------- serialisation
    def to_npz(self, path):
        """Store the compiled network (no source text) as a small .npz."""
        r = self.reactions
        np.savez_compressed(
            path,
            species=np.array(self.species),
            use_photo=self.use_photo,
            stop_rev_indx=self.stop_rev_indx,
            index=np.array([x.index for x in r]),
            text=np.array([x.text for x in r]),
            kind=np.array([x.kind for x in r]),
            params=np.array([[x.A, x.B, x.C, x.A_inf, x.B_inf, x.C_inf] for x in r]),
            photo_sp=np.array([x.photo_sp for x in r]),
            photo_br=np.array([x.photo_br for x in r]),
            nasa9=self.nasa9, compo=self.compo, mass=self.mass,
            compo_atoms=np.array(self.compo_atoms))

    @classmethod
    def from_npz(cls, path):
        d = np.load(path, allow_pickle=False)
        reactions = []
        for idx, text, kind, p, psp, pbr in zip(d['index'], d['text'], d['kind'],
                                                d['params'], d['photo_sp'],
                                                d['photo_br']):
            reac, prod = _split_terms(str(text))
            reactions.append(Reaction(int(idx), str(text), reac, prod, str(kind),
                                      *[float(v) for v in p], photo_sp=str(psp),
                                      photo_br=int(pbr)))
        return cls(path=str(path), use_photo=bool(d['use_photo']),
                   species=[str(s) for s in d['species']], reactions=reactions,
                   stop_rev_indx=int(d['stop_rev_indx']), nasa9=d['nasa9'],
                   compo_atoms=[str(a) for a in d['compo_atoms']],
                   compo=d['compo'], mass=d['mass'])

    # ------------------------------------------------------------ thermo / k
    def gibbs_RT(self, T):
        """g/RT per species, [ni, nz] (chem_funs h_RT - s_R, low range T<1000)."""
        T = np.asarray(T, dtype=np.float64)
        out = np.empty((self.ni, T.size))
        lnT = np.log(T)
        for s in range(self.ni):
            lo, hi = self.nasa9[s, :10], self.nasa9[s, 10:]
            out[s] = (T < 1000) * _g_rt(T, lnT, lo) + (T >= 1000) * _g_rt(T, lnT, hi)
        return out

    def keq(self, T):
        """Equilibrium constant of every forward reaction, [npair, nz]."""
        T = np.asarray(T, dtype=np.float64)
        g = self.gibbs_RT(T)
        sidx = {s: k for k, s in enumerate(self.species)}
        out = np.empty((self.npair, T.size))
        for p, r in enumerate(self.reactions):
            dg = np.zeros(T.size)
            nr_ = npr = 0
            for nu, name in r.reac:
                if name != 'M':
                    dg = dg - nu * g[sidx[name]]
                    nr_ += nu
            for nu, name in r.prod:
                if name != 'M':
                    dg = dg + nu * g[sidx[name]]
                    npr += nu
            kq = np.exp(-dg)
            if npr - nr_ != 0:
                kq = kq * (CORR * T) ** (nr_ - npr)
            out[p] = kq
        return out

    def rate_constants(self, Tco, M, remove_list=(), use_lowT_limit_rates=False):
        """FP64 rate constants, array [nr, nz]; row i-1 holds k[i].

        Photo/ion forward slots are zero placeholders (filled by J rates);
        reverse slots at or beyond ``# reverse stops`` are zero."""
        Tco = np.asarray(Tco, dtype=np.float64)
        M = np.asarray(M, dtype=np.float64)
        nz = Tco.size
        k = np.zeros((self.nr, nz))
        for p, r in enumerate(self.reactions):
            i = r.index
            if r.kind in ('arrhenius', 'k0'):
                kf = r.A * Tco ** r.B * np.exp(-r.C / Tco)
            elif r.kind == 'falloff':
                k0 = r.A * Tco ** r.B * np.exp(-r.C / Tco)
                kinf = r.A_inf * Tco ** r.B_inf * np.exp(-r.C_inf / Tco)
                kf = k0 / (1 + k0 * M / kinf)
            elif r.kind == 'special':
                if r.text != SPECIAL_OH_CH3:
                    raise ValueError('no rate form for special reaction ' + r.text)
                kf = _special_oh_ch3(Tco, M)
            else:                       # conden, photo, ion
                kf = np.zeros(nz)
            k[2 * p] = kf
        if use_lowT_limit_rates:
            self._lim_lowT(k, Tco, M)
        kq = self.keq(Tco)
        for p, r in enumerate(self.reactions):
            ir = r.index + 1
            if ir < self.stop_rev_indx and r.kind not in ('conden',):
                k[2 * p + 1] = 0.0 if ir in remove_list else k[2 * p] / kq[p]
            else:
                k[2 * p + 1] = 0.0
        for i in remove_list:
            if 1 <= i <= self.nr:
                k[i - 1] = 0.0
        return k

    def _lim_lowT(self, k, Tco, M):
        """Low-temperature caps of op.ReadRate.lim_lowT_rates (op.py:320-342),
        applied to the forward rates before the reverse rates are formed
        (vulcan.py:130-136 order)."""
        for p, r in enumerate(self.reactions):
            cap = LOWT_CAPS.get(r.text)
            if cap is None:
                continue
            t_max, kind, (A, B, C, A2, B2, C2) = cap
            m = Tco <= t_max
            k0 = A * Tco ** B * np.exp(-C / Tco)
            if kind == 'falloff':
                kinf = A2 * Tco ** B2 * np.exp(-C2 / Tco)
                k0 = k0 / (1. + k0 * M / kinf)
            k[2 * p][m] = k0[m]

    def rate_caps(self):
        """Per-pair tables for vk_set_rate_caps: (kind [npair], T_max [npair],
        params [npair, 6]) of the low-temperature caps (LOWT_CAPS)."""
        codes = {'arrhenius': 1, 'falloff': 2}
        kind = np.zeros(self.npair, dtype=np.int32)
        t_max = np.zeros(self.npair)
        params = np.zeros((self.npair, 6))
        for p, r in enumerate(self.reactions):
            cap = LOWT_CAPS.get(r.text)
            if cap is not None:
                t_max[p], kind[p], params[p] = cap[0], codes[cap[1]], cap[2]
        return kind, t_max, params

    def rate_params(self):
        """Per-pair tables for vk_set_rate_params: (kind, rev, params [npair, 6],
        nasa9 [ni, 20]); kind 1 Arrhenius (two-body, k0-only three-body), 2
        fall-off, 3 the OH + CH3 + M form, 0 photolysis / ionisation /
        condensation (forward slot as uploaded); rev = 1 where the reverse rate
        is k_f / Keq (before '# reverse stops', not condensation)."""
        codes = {'arrhenius': 1, 'k0': 1, 'falloff': 2}
        kind = np.zeros(self.npair, dtype=np.int32)
        rev = np.zeros(self.npair, dtype=np.int32)
        params = np.zeros((self.npair, 6))
        for p, r in enumerate(self.reactions):
            if r.kind == 'special':
                if r.text != SPECIAL_OH_CH3:
                    raise ValueError('no rate form for special reaction ' + r.text)
                kind[p] = 3
            else:
                kind[p] = codes.get(r.kind, 0)
            rev[p] = int(r.index + 1 < self.stop_rev_indx and r.kind != 'conden')
            params[p] = (r.A, r.B, r.C, r.A_inf, r.B_inf, r.C_inf)
        return kind, rev, params, np.ascontiguousarray(self.nasa9, dtype=np.float64)

    def photo_index(self):
        """{(species, branch): forward k index} for photolysis reactions."""
        return {(r.photo_sp, r.photo_br): r.index for r in self.reactions
                if r.kind == 'photo'}

    # --------------------------------------------------------- kernel tables
    def pair_tables(self):
        """Flat factor tables per reaction pair for the C-ABI descriptor.

        Returns dict of int32 arrays: fwd_ptr/fwd_sp/fwd_nu (reactants merged
        by species, M excluded), rev_ptr/rev_sp/rev_nu (products), fwd_m/rev_m
        (powers of M)."""
        sidx = {s: k for k, s in enumerate(self.species)}
        out = {k: [] for k in ('fwd_sp', 'fwd_nu', 'rev_sp', 'rev_nu', 'fwd_m', 'rev_m')}
        fptr, rptr = [0], [0]
        for r in self.reactions:
            ff, fm = r.side_factors('f')
            rf, rm = r.side_factors('r')
            for name, nu in ff:
                out['fwd_sp'].append(sidx[name])
                out['fwd_nu'].append(nu)
            for name, nu in rf:
                out['rev_sp'].append(sidx[name])
                out['rev_nu'].append(nu)
            fptr.append(len(out['fwd_sp']))
            rptr.append(len(out['rev_sp']))
            out['fwd_m'].append(fm)
            out['rev_m'].append(rm)
        res = {k: np.asarray(v, dtype=np.int32) for k, v in out.items()}
        res['fwd_ptr'] = np.asarray(fptr, dtype=np.int32)
        res['rev_ptr'] = np.asarray(rptr, dtype=np.int32)
        return res

    def compo_for(self, atom_list):
        """Element-count matrix [ni, len(atom_list)] for the conservation sums."""
        cols = [self.compo_atoms.index(a) for a in atom_list]
        return np.ascontiguousarray(self.compo[:, cols], dtype=np.float64)


def _g_rt(T, lnT, a):
    h = (-a[0] / T ** 2 + a[1] * lnT / T + a[2] + a[3] * T / 2. + a[4] * T ** 2 / 3.
         + a[5] * T ** 3 / 4. + a[6] * T ** 4 / 5. + a[8] / T)
    s = (-a[0] / T ** 2 / 2. - a[1] / T + a[2] * lnT + a[3] * T + a[4] * T ** 2 / 2.
         + a[5] * T ** 3 / 3. + a[6] * T ** 4 / 4. + a[9])
    return h - s


def _special_oh_ch3(T, M):
    """Pressure-dependent OH + CH3 + M -> CH3OH + M (op.py:197-207)."""
    k = 1.932E3 * T ** -9.88 * np.exp(-7544. / T) + 5.109E-11 * T ** -6.25 * np.exp(-1433. / T)
    kinf = 1.031E-10 * T ** -0.018 * np.exp(16.74 / T)
    Fc = 0.1855 * np.exp(-T / 155.8) + 0.8145 * np.exp(-T / 1675.) + np.exp(-4531. / T)
    nn = 0.75 - 1.27 * np.log(Fc)
    ff = np.exp(np.log(Fc) / (1. + (np.log(k * M / kinf) / nn) ** 2))
    return k / (1 + k * M / kinf) * ff
