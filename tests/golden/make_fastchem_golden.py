"""Equilibrium fixture from the reference's own FastChem (the engine of
ini_mix = 'EQ', build_atm.py:78-164).

Builds FastChem from the reference tree (oracle/fastchem.mk, into
oracle/_ref/), then for a few seeded columns of the 512-column NCHO workload
writes FastChem's inputs the way the reference's ini_fc does -- the column's
element abundances as 12 + log10(n_X / n_H), FastChem's other elements
absent (-20; the network has none of them), the NASA-9 species file
nasa9_logK_SNCHOTi.dat, p in bar and T as '%.3e' / '%.1f' -- runs it, and
stores the mixing ratios of the network's species (tests/golden/golden_eq.npz)
and which of them FastChem lists twice (two data sets under one name, of
which the reference reads the first).

Usage:  python tests/golden/make_fastchem_golden.py [--ref <VULCAN tree>]
        (default: $VULCAN_REFERENCE)
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from vulcan_gb300 import configs, warmstart  # noqa: E402
from vulcan_gb300.network import Network  # noqa: E402

ATOMS = ['H', 'O', 'C', 'He', 'N']
OTHER = ['P', 'S', 'Si', 'Ti', 'V', 'Cl', 'K', 'Na', 'Mg', 'F', 'Ca', 'Fe']
COLUMNS = (0, 60, 100, 300, 511)


def run_fastchem(exe, ref, spec, net, workdir):
    fc = os.path.join(ref, 'fastchem_vulcan')
    ab = warmstart.const_mix_abundances(spec, net, ATOMS)
    rel = {a: ab[i] / ab[0] for i, a in enumerate(ATOMS)}
    os.makedirs(os.path.join(workdir, 'input'))
    os.makedirs(os.path.join(workdir, 'output'))
    with open(os.path.join(workdir, 'input', 'elements.dat'), 'w') as f:
        f.write('#element abundances\n')
        for a in ('C', 'H', 'He', 'N', 'O'):
            f.write('%s\t%.6f\n' % (a, 12 + np.log10(rel[a])))
        for a in OTHER:
            f.write('%s\t-20\n' % a)
        f.write('e-\t0')
    with open(os.path.join(workdir, 'input', 'parameters.dat'), 'w') as f:
        f.write('#element abundance file\ninput/elements.dat\n\n'
                '#elements data file\n%s/fastchem_src/chem_input/chemical_elements.dat\n\n'
                '#species data file\n%s/input/nasa9_logK_SNCHOTi.dat\n\n'
                '#accuracy of chemistry iteration\n1.0e-4\n\n'
                "#max error of Newton's method\n1.0e-4\n\n"
                '#max number of chemistry iterations\n1000\n\n'
                '#max number of Nelder-Mead iterations\n20000\n' % (fc, fc))
    p_bar = ['{:.3e}'.format(p / 1e6) for p in spec.pco]
    t_k = ['{:.1f}'.format(t) for t in spec.Tco]
    with open(os.path.join(workdir, 'input', 'tp.dat'), 'w') as f:
        f.write('#p (bar)    T (K)\n' + '\n'.join(p + '\t' + t for p, t in zip(p_bar, t_k)))
    with open(os.path.join(workdir, 'input', 'config.input'), 'w') as f:
        f.write('#FastChem parameter file\ninput/parameters.dat\n\n'
                '#Atmospheric profile input file\ninput/tp.dat\n\n'
                '#Abundances output file\noutput/eq.dat\n\n'
                '#Monitor output file\noutput/monitor.dat\n\n'
                '#FastChem console verbose level (1 - 4)\n0\n\n'
                '#Output mixing ratios (MR) or particle number densities (ND, default)?\nMR\n')
    subprocess.run([exe, 'input/config.input'], cwd=workdir, check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    lines = [ln for ln in open(os.path.join(workdir, 'output', 'eq.dat')).read().split('\n') if ln.strip()]
    hdr = lines[0].split()
    dat = np.array([[float(v) for v in ln.split()] for ln in lines[1:]])
    x = np.zeros((len(spec.pco), net.ni))
    have = np.zeros(net.ni, dtype=bool)
    dup = np.zeros(net.ni, dtype=bool)      # listed twice by FastChem (two data sets)
    for i, sp in enumerate(net.species):
        if sp in hdr:
            x[:, i] = dat[:, hdr.index(sp)]   # the first, as the reference reads it
            have[i] = True
            dup[i] = hdr.count(sp) > 1
    pco = np.array([float(p) for p in p_bar]) * 1e6
    tco = np.array([float(t) for t in t_k])
    return x, have, dup, pco, tco, ab


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('VULCAN_REFERENCE'),
                    help='the VULCAN source tree (default: $VULCAN_REFERENCE)')
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(os.path.join(a.ref, 'fastchem_vulcan')):
        ap.error('give the VULCAN source tree with --ref or VULCAN_REFERENCE (got %r)' % a.ref)
    subprocess.run(['make', '-s', '-f', os.path.join(REPO, 'oracle', 'fastchem.mk'), 'REF=' + a.ref],
                   check=True)
    exe = os.path.join(REPO, 'oracle', '_ref', 'fastchem')
    net = Network.from_npz(os.path.join(HERE, 'net_NCHO_thermo.npz'))
    specs = configs.config2_columns(ncols=512, seed=2)
    out = {'columns': np.array(COLUMNS), 'atoms': np.array(ATOMS)}
    with tempfile.TemporaryDirectory() as w:
        for c in COLUMNS:
            x, have, dup, pco, tco, ab = run_fastchem(exe, a.ref, specs[c], net,
                                                      os.path.join(w, str(c)))
            out.update({'x_%d' % c: x, 'pco_%d' % c: pco, 'tco_%d' % c: tco, 'abund_%d' % c: ab})
            out['have'], out['dup'] = have, dup
    path = os.path.join(HERE, 'golden_eq.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, os.path.getsize(path) // 1024, 'KiB;', int(out['have'].sum()), 'of',
          net.ni, 'species in FastChem')


if __name__ == '__main__':
    main()
