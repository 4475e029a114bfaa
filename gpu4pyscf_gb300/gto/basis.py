"""Basis-set input handling.

Accepted basis specifications (the forms pyscf.gto.Mole accepts):
* a list of shells in internal format ``[l, [exp, c1, c2, ...], ...]``;
* an NWChem-format string, optionally prefixed with ``unc`` to split every
  primitive into its own shell (the form used by gpu4pyscf's
  scf/tests/test_rhf.py:48-77);
* a dict ``{element or 'default': spec}``;
* a tuple of specs, concatenated (gpu4pyscf scf/tests/test_scf_jk.py:218);
* a name.  Bundled names are ``sto-3g`` and the synthetic same-structure sets
  ``syn-cc-pvdz``, ``syn-6-31g*``, ``syn-def2-svp`` and ``syn-def2-tzvp``.

The ``syn-*`` sets have the shell structure (angular momenta, primitive and
contraction counts per element) of the named basis sets, with exponents drawn
from fixed even-tempered ranges and smooth positive contraction coefficients.
They exercise the same integral classes as the real sets but do not
reproduce their absolute energies; real basis data is not bundled.
"""

import math
import numpy as np

ANGULAR = 'spdfghik'

# STO-3G (Hehre, Stewart, Pople 1969): the universal 1s and 2sp three-Gaussian
# fits scaled by the standard molecular Slater exponents, as tabulated.
_STO3G_1S = [0.15432897, 0.53532814, 0.44463454]
_STO3G_2S = [-0.09996723, 0.39951283, 0.70011547]
_STO3G_2P = [0.15591627, 0.60768372, 0.39195739]
_STO3G_EXPS = {
    'H': ([3.42525091, 0.62391373, 0.16885540], None),
    'C': ([71.6168370, 13.0450960, 3.5305122], [2.9412494, 0.6834831, 0.2222899]),
    'N': ([99.1061690, 18.0523120, 4.8856602], [3.7804559, 0.8784966, 0.2857144]),
    'O': ([130.7093200, 23.8088610, 6.4436083], [5.0331513, 1.1695961, 0.3803890]),
}


def _sto3g(symb):
    if symb not in _STO3G_EXPS:
        raise KeyError(f'sto-3g is bundled for H, C, N, O only, not {symb}')
    e1, e2 = _STO3G_EXPS[symb]
    shells = [[0] + [[e, c] for e, c in zip(e1, _STO3G_1S)]]
    if e2 is not None:
        shells.append([0] + [[e, c] for e, c in zip(e2, _STO3G_2S)])
        shells.append([1] + [[e, c] for e, c in zip(e2, _STO3G_2P)])
    return shells


# -- synthetic same-structure basis sets -----------------------------------
# Each entry: (l, nprim, hi, lo, nctr).  hi/lo are scaled by the element
# factor f = (Z/8)**p with p given per row (core rows scale faster).
_SYN = {
    'syn-cc-pvdz': {
        'H': [(0, 4, 13.0, 0.12, 1, 0.), (0, 1, 0.12, 0.12, 1, 0.), (1, 1, 0.73, 0.73, 1, 0.)],
        'X': [(0, 9, 11700., 0.30, 2, 2.), (0, 1, 0.30, 0.30, 1, .5),
              (1, 3, 17.7, 1.05, 1, 1.), (1, 1, 0.275, 0.275, 1, .5),
              (2, 1, 1.18, 1.18, 1, .5)],
    },
    'syn-6-31g*': {
        'H': [(0, 3, 18.7, 0.64, 1, 0.), (0, 1, 0.16, 0.16, 1, 0.)],
        'X': [(0, 6, 5480., 1.87, 1, 2.), (0, 3, 15.5, 0.30, 1, 1.),
              (1, 3, 15.5, 0.30, 1, 1.), (0, 1, 0.27, 0.27, 1, .5),
              (1, 1, 0.27, 0.27, 1, .5), (2, 1, 0.80, 0.80, 1, .5)],
    },
    'syn-def2-svp': {
        'H': [(0, 3, 13.0, 0.12, 1, 0.), (0, 1, 0.12, 0.12, 1, 0.), (1, 1, 0.80, 0.80, 1, 0.)],
        'X': [(0, 5, 2266., 1.0, 1, 2.), (0, 1, 0.80, 0.80, 1, .5),
              (0, 1, 0.25, 0.25, 1, .5), (1, 3, 17.7, 0.80, 1, 1.),
              (1, 1, 0.22, 0.22, 1, .5), (2, 1, 1.10, 1.10, 1, .5)],
    },
    'syn-def2-tzvp': {
        'H': [(0, 3, 34.0, 0.90, 1, 0.), (0, 1, 0.35, 0.35, 1, 0.),
              (0, 1, 0.12, 0.12, 1, 0.), (1, 1, 0.80, 0.80, 1, 0.)],
        'X': [(0, 6, 27000., 30.0, 1, 2.), (0, 2, 20.0, 6.0, 1, 1.),
              (0, 1, 1.00, 1.00, 1, .6), (0, 1, 0.45, 0.45, 1, .6),
              (0, 1, 0.15, 0.15, 1, .6), (1, 4, 63.0, 1.20, 1, 1.),
              (1, 1, 0.40, 0.40, 1, .6), (1, 1, 0.13, 0.13, 1, .6),
              (2, 1, 2.30, 2.30, 1, .5), (2, 1, 0.65, 0.65, 1, .5),
              (3, 1, 1.40, 1.40, 1, .5)],
    },
}


def _syn_shell(l, nprim, hi, lo, nctr, power, z):
    f = (z / 8.) ** power
    hi *= f
    lo *= f
    if nprim == 1:
        exps = np.array([hi])
    else:
        exps = np.exp(np.linspace(math.log(hi), math.log(lo), nprim))
    # smooth positive contraction profiles, centred at different exponents
    # for each contraction of a general contraction
    x = np.linspace(0., 1., nprim)
    rows = []
    cols = []
    for k in range(nctr):
        mid = 0.65 if k == 0 else 0.95
        c = np.exp(-((x - mid) / 0.35) ** 2)
        if k > 0:
            c = c - 0.3 * np.exp(-((x - 0.3) / 0.3) ** 2)
        cols.append(c)
    cols = np.array(cols).T
    for e, c in zip(exps, cols):
        rows.append([float(e)] + [float(v) for v in c])
    return [l] + rows


def _synthetic(name, symb):
    from .mole import charge_of
    table = _SYN[name]
    z = charge_of(symb)
    rows = table['H'] if z <= 2 else table['X']
    return [_syn_shell(*row, z=z) for row in rows]


def parse_nwchem(text, symb=None):
    """Parse NWChem-format basis text; return {symbol: shells} or the shells
    of ``symb``."""
    from .mole import std_symbol
    out = {}
    cur = None
    for raw in text.splitlines():
        line = raw.split('#')[0].strip()
        if not line or line.upper().startswith('BASIS') or line.upper() == 'END':
            continue
        tok = line.split()
        if tok[0][0].isalpha():
            el = std_symbol(tok[0])
            kinds = tok[1].upper()
            if kinds == 'SP':
                cur = [[0], [1]]
                out.setdefault(el, []).extend(cur)
                cur = ('SP', out[el][-2], out[el][-1])
            else:
                shell = [ANGULAR.index(kinds.lower())]
                out.setdefault(el, []).append(shell)
                cur = ('X', shell)
        else:
            vals = [float(v.replace('D', 'E').replace('d', 'e')) for v in tok]
            if cur[0] == 'SP':
                cur[1].append([vals[0], vals[1]])
                cur[2].append([vals[0], vals[2]])
            else:
                cur[1].append(vals)
    if symb is None:
        return out
    return out.get(std_symbol(symb))


def uncontract(shells):
    """Split every primitive of every shell into its own shell, dropping
    duplicates of the same (l, exponent)."""
    out = []
    seen = set()
    for sh in shells:
        l = sh[0]
        for p in sh[1:]:
            key = (l, p[0])
            if key in seen:
                continue
            seen.add(key)
            out.append([l, [p[0], 1.]])
    return out


def _resolve_one(spec, symb):
    if spec is None:
        return None
    if isinstance(spec, tuple):
        shells = []
        for s in spec:
            r = _resolve_one(s, symb)
            if r:
                shells.extend(r)
        return shells
    if isinstance(spec, list):
        return [list(sh) for sh in spec]
    if isinstance(spec, str):
        s = spec.strip()
        unc = False
        if s.lower().startswith('unc'):
            unc = True
            s = s[3:].lstrip('-_ ')
        if '\n' in s:
            shells = parse_nwchem(s, symb)
        else:
            key = s.lower().replace('_', '-')
            if key in ('sto-3g', 'sto3g'):
                shells = _sto3g(symb)
            elif key in _SYN:
                shells = _synthetic(key, symb)
            else:
                raise KeyError(
                    f"basis data for '{spec}' is not bundled; pass the basis "
                    "explicitly (NWChem text or shell list) or use one of "
                    f"sto-3g, {', '.join(sorted(_SYN))}")
        if shells is None:
            return None
        return uncontract(shells) if unc else shells
    raise TypeError(f'unsupported basis spec {type(spec)}')


def resolve(spec, symb):
    """Shells of element ``symb`` for a basis specification."""
    from .mole import std_symbol
    symb = std_symbol(symb)
    if isinstance(spec, dict):
        sub = None
        for k, v in spec.items():
            if std_symbol(k) == symb if k != 'default' else False:
                sub = v
                break
        if sub is None:
            sub = spec.get('default')
        if sub is None:
            raise KeyError(f'no basis given for {symb}')
        spec = sub
    shells = _resolve_one(spec, symb)
    if shells is None:
        raise KeyError(f'no basis for {symb}')
    # PySCF orders the shells of an atom by angular momentum (stable)
    return sorted(shells, key=lambda sh: sh[0])
