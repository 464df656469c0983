"""Seeded synthetic stress network: 150 species, 1200 reversible reactions,
60 frozen photolysis channels, written in the reference's own file formats.

The reference ships networks of 41-69 species; this generator makes a larger
one of the same kind so that the block solve runs at ni = 150 (blocks of
150 x 150, the upper end of VK_MAX_NI).  Output, in a directory of the
caller's choosing, is what ``Network.from_file`` (and the reference's
make_chem_funs.py / op.ReadRate) read:

  <name>_network.txt   id [ A + B -> C + D ] A B C   (two-body and
                       unimolecular lines), '# 3-body' fall-off lines with
                       A B C A_inf B_inf C_inf, '# reverse stops', '# photo'
                       lines  id [ A -> B + C ] A branch
  NASA9/<sp>.txt       two ranges of 10 coefficients (a1..a7, 0, b1, b2)
  all_compose.txt      'species H O C He N mass' table

Choices (all seeded):
  * species: H/O/C/N molecules of a composition grid (H 0-8, C 0-3, O 0-3,
    N 0-2), always including the usual background species, plus He (which
    only enters the inert 'He -> He' line, as in the reference networks);
  * reactions conserve every element by construction (products are drawn
    from the species pairs with the reactants' summed composition);
    80 % two-body A + B -> C + D, 15 % three-body A + B + M -> C + M,
    5 % unimolecular A -> B + C;
  * k = A T^B exp(-C/T): two-body A log-U[1e-14, 1e-9] cm^3 s^-1, C U[0, 40000]
    K; three-body k0 = 1e-20 A (cm^6 s^-1) and k_inf = A; unimolecular
    A log-U[1e8, 1e13] s^-1; B = 0.  C is then raised where needed so that
    the reverse rate k/Keq (the reference's rev_rate, op.py:287-309) stays
    below the collision limit (1e-9 cm^3 s^-1 for two-body reverses, 1e13
    s^-1 for first-order ones) over 400-3500 K, as the endothermic direction
    of a real reaction is the slow one; a draw that would need C > 1.5e5 K is
    rejected (its rates would underflow at 400 K);
  * Gibbs data: constant heat capacity cp/R = 2.5 + 0.5 n_atoms, enthalpy of
    formation b1 = sum of per-element terms - 25000 K per bond (n_atoms - 1)
    + U[-6000, 6000] K, entropy offset b2 U[10, 40] + 2 n_atoms, the same in
    both NASA-9 ranges;
  * photolysis: 60 channels A -> B + C of species with >= 2 atoms, J frozen
    per column (configs.photo_J_profile).
"""
from __future__ import annotations

import itertools
import os

import numpy as np

ATOMS = ('H', 'O', 'C', 'He', 'N')
MASS = {'H': 1.00794, 'O': 15.9994, 'C': 12.0107, 'He': 4.002602, 'N': 14.0067}
CORE = {'H2': (2, 0, 0, 0), 'H': (1, 0, 0, 0), 'H2O': (2, 1, 0, 0), 'OH': (1, 1, 0, 0),
        'O': (0, 1, 0, 0), 'O2': (0, 2, 0, 0), 'CH4': (4, 0, 1, 0), 'CH3': (3, 0, 1, 0),
        'CO': (0, 1, 1, 0), 'CO2': (0, 2, 1, 0), 'C': (0, 0, 1, 0), 'N2': (0, 0, 0, 2),
        'NH3': (3, 0, 0, 1), 'NH2': (2, 0, 0, 1), 'N': (0, 0, 0, 1), 'HCN': (1, 0, 1, 1)}


def _formula(h, o, c, n):
    """Hill-order name C..H..N..O.. of a composition (H, O, C, N)."""
    out = ''
    for sym, k in (('C', c), ('H', h), ('N', n), ('O', o)):
        if k:
            out += sym + (str(k) if k > 1 else '')
    return out


def make_species(rng, ni=150):
    """ni species (ni - 1 reactive + He): name -> composition (H, O, C, N)."""
    names = dict(CORE)
    taken = {v for v in CORE.values()}
    grid = [g for g in itertools.product(range(9), range(4), range(4), range(3))
            if sum(g) > 0 and g not in taken]
    pick = rng.permutation(len(grid))[:ni - 1 - len(names)]
    for p in pick:
        h, o, c, n = grid[p]
        names[_formula(h, o, c, n)] = (h, o, c, n)
    return names


CORR = 1.38064852E-16 / 1.0e6          # k_B / P0 (the reference's gibbs_text corr)
T_GRID = np.linspace(400.0, 3500.0, 64)
K2_MAX = 1e-9                             # two-body collision limit (cm^3 s^-1)
K1_MAX = 1e13                             # first-order limit (s^-1)
BOND = 25000.0                            # formation enthalpy per bond (K): associations
                                          # are exothermic, exchanges thermoneutral
EA_MAX = 1.5e5                            # larger barriers: the draw is rejected (k would
                                          # underflow at 400 K and k0/k_inf become 0/0)


def _g_rt(a3, b1, b2, T):
    """g/RT of the constant-cp species model: h/RT - s/R."""
    return a3 * (1.0 - np.log(T)) + b1 / T - b2


def _min_ea(lnA, reac, prod, g, extra_order=0):
    """Smallest activation temperature C (K) keeping the reverse rate below its
    limit over T_GRID; reac/prod are species index lists (M excluded)."""
    dg = sum(g[p] for p in prod) - sum(g[r] for r in reac)          # [T]
    lnK = -dg + (len(reac) - len(prod)) * np.log(CORR * T_GRID)
    order = len(prod) + extra_order                                # reverse order (with M)
    ln_lim = np.log(K2_MAX if order >= 2 else K1_MAX)
    # ln k_r = lnA - C/T - lnK <= ln_lim  <=>  C >= T (lnA - lnK - ln_lim)
    return float(max(0.0, np.max(T_GRID * (lnA - lnK - ln_lim))))


def generate(out_dir, seed=4, ni=150, n_rev=1200, n_photo=60, name='SYN150'):
    """Write the network, NASA-9 and composition files; returns the network
    file path.  Deterministic in (seed, ni, n_rev, n_photo)."""
    rng = np.random.default_rng(seed)
    sp = make_species(rng, ni)
    names = list(sp)
    comp = np.array([sp[s] for s in names])
    # thermo: constant cp, seeded formation enthalpy and entropy offset
    h_el = {'H': -1500.0, 'O': -12000.0, 'C': 8000.0, 'N': 2000.0}
    thermo = []
    for cv in comp:
        nat = max(int(cv.sum()), 1)
        a3 = 2.5 + 0.5 * nat
        b1 = (sum(h_el[e] * k for e, k in zip(('H', 'O', 'C', 'N'), cv)) - BOND * (nat - 1)
              + rng.uniform(-6000, 6000))
        b2 = rng.uniform(10, 40) + 2.0 * nat
        thermo.append((a3, b1, b2))
    g = [_g_rt(a3, b1, b2, T_GRID) for a3, b1, b2 in thermo]
    idx = {tuple(v): k for k, v in enumerate(comp.tolist())}
    # composition sums of unordered pairs (allowing A + A)
    pairs = {}
    for a in range(len(names)):
        for b in range(a, len(names)):
            pairs.setdefault(tuple((comp[a] + comp[b]).tolist()), []).append((a, b))
    seen = set()
    lines = {'bi': [], 'ter': [], 'uni': []}
    n_ter, n_uni = int(round(0.15 * n_rev)), int(round(0.05 * n_rev))
    n_bi = n_rev - n_ter - n_uni

    def key(r, p):
        return (tuple(sorted(r)), tuple(sorted(p)))

    tries = 0
    while len(lines['bi']) < n_bi:
        tries += 1
        if tries > 10 ** 6:
            raise RuntimeError('could not draw enough two-body reactions')
        a, b = sorted(rng.integers(0, len(names), 2))
        cand = [q for q in pairs[tuple((comp[a] + comp[b]).tolist())] if q != (a, b)]
        if not cand:
            continue
        c, d = cand[rng.integers(len(cand))]
        k1, k2 = key((a, b), (c, d)), key((c, d), (a, b))
        if k1 in seen or k2 in seen:
            continue
        seen.add(k1)
        A = 10.0 ** rng.uniform(-14, -9)
        Ea = max(rng.uniform(0, 40000), _min_ea(np.log(A), [a, b], [c, d], g))
        if Ea > EA_MAX:
            seen.discard(k1)
            continue
        lines['bi'].append(('%s + %s -> %s + %s' % (names[a], names[b], names[c], names[d]),
                            '%.4E 0.0 %.1f' % (A, Ea)))
    # species that are the sum of a pair (three-body association, unimolecular split)
    assoc = [(pr, idx[s]) for s, prs in pairs.items() if s in idx for pr in prs]
    tries = 0

    def draw():
        nonlocal tries
        tries += 1
        if tries > 10 ** 6:
            raise RuntimeError('could not draw enough association / split reactions')
        return assoc[rng.integers(len(assoc))]

    while len(lines['ter']) < n_ter:
        (a, b), c = draw()
        k1 = key((a, b, -1), (c, -1))
        if k1 in seen:
            continue
        seen.add(k1)
        A = 10.0 ** rng.uniform(-14, -9)
        # the fall-off rate k0 / (1 + k0 M / k_inf) never exceeds k0 = 1e-20 A exp(-Ea/T)
        # (cm^6 s^-1, the rate law carries M); its reverse C + M -> A + B + M is
        # two-body in (C, M)
        Ea = max(rng.uniform(0, 40000), _min_ea(np.log(1e-20 * A), [a, b], [c], g, extra_order=1))
        if Ea > EA_MAX:
            seen.discard(k1)
            continue
        lines['ter'].append(('%s + %s + M -> %s + M' % (names[a], names[b], names[c]),
                             '%.4E 0.0 %.1f %.4E 0.0 %.1f' % (1e-20 * A, Ea, A, Ea)))
    while len(lines['uni']) < n_uni:
        (b, c), a = draw()
        k1 = key((a,), (b, c))
        if k1 in seen:
            continue
        seen.add(k1)
        A = 10.0 ** rng.uniform(8, 13)
        Ea = max(rng.uniform(0, 40000), _min_ea(np.log(A), [a], [b, c], g))
        if Ea > EA_MAX:
            seen.discard(k1)
            continue
        lines['uni'].append(('%s -> %s + %s' % (names[a], names[b], names[c]),
                             '%.4E 0.0 %.1f' % (A, Ea)))
    photo = []
    used_br = {}
    for k in rng.permutation(len(assoc)):
        if len(photo) >= n_photo:
            break
        (b, c), a = assoc[k]
        if comp[a].sum() < 2:
            continue
        br = used_br.get(a, 0) + 1
        used_br[a] = br
        photo.append(('%s -> %s + %s' % (names[a], names[b], names[c]), '%s %d' % (names[a], br)))
    # --- network text, numbered 1, 3, 5, ...
    out = ['# synthetic stress network: seed %d, %d species' % (seed, ni),
           '# Two-body Reactions']
    i = 1
    for text, coef in lines['bi'] + lines['uni']:
        out.append('%d [ %s ] %s' % (i, text, coef))
        i += 2
    out.append('%d [ He -> He ] 0.0 0.0 0.0' % i)
    i += 2
    out.append('')
    out.append('# 3-body and Disscoiation Reactions')
    for text, coef in lines['ter']:
        out.append('%d [ %s ] %s' % (i, text, coef))
        i += 2
    out.append('')
    out.append('# reverse stops')
    out.append('# photo disscoiation (no reversals)')
    for text, coef in photo:
        out.append('%d [ %s ] %s' % (i, text, coef))
        i += 2
    os.makedirs(os.path.join(out_dir, 'NASA9'), exist_ok=True)
    net_path = os.path.join(out_dir, '%s_network.txt' % name)
    with open(net_path, 'w') as f:
        f.write('\n'.join(out) + '\n')
    # --- thermo files (He: monatomic constants)
    allsp = names + ['He']
    allcomp = np.vstack([comp, [0, 0, 0, 0]])
    for s, (a3, b1, b2) in zip(allsp, thermo + [(2.5, -745.0, 0.9)]):
        row = [0.0, 0.0, a3, 0.0, 0.0, 0.0, 0.0, 0.0, b1, b2]
        with open(os.path.join(out_dir, 'NASA9', s + '.txt'), 'w') as f:
            f.write(' '.join('%.8E' % v for v in row) + '\n')
            f.write(' '.join('%.8E' % v for v in row) + '\n')
    with open(os.path.join(out_dir, 'all_compose.txt'), 'w') as f:
        f.write('species ' + ' '.join(ATOMS) + ' mass\n')
        for s, cv in zip(allsp, allcomp):
            h, o, c, n = (int(v) for v in cv)
            he = 1 if s == 'He' else 0
            m = h * MASS['H'] + o * MASS['O'] + c * MASS['C'] + n * MASS['N'] + he * MASS['He']
            f.write('%s %d %d %d %d %d %.5f\n' % (s, h, o, c, he, n, m))
    return net_path
