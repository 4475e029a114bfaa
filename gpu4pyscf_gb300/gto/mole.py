"""Molecule and Gaussian basis container with the libcint data layout.

The arrays ``_atm`` (int32 [natm, 6]), ``_bas`` (int32 [nbas, 8]) and ``_env``
(float64) follow the layout that pyscf.gto.Mole hands to libcint, so a real
``pyscf.gto.Mole`` and this class are interchangeable at the J/K boundary
(gpu4pyscf/scf/jk.py:60 takes ``mol`` and reads only these arrays, ``cart``,
``nao`` and ``ao_loc``).

Conventions restated from PySCF (pyscf/gto/mole.py, the module gpu4pyscf builds
on; gpu4pyscf/gto/mole.py:1120-1132 relies on the same ones):
* each contracted radial function is normalised, the primitive coefficients
  stored in ``_env`` already carry the radial factor ``gto_norm(l, alpha)``;
* Cartesian components of a shell are ordered lx descending, then ly
  descending (xx, xy, xz, yy, yz, zz for d);
* spherical components are real solid harmonics ordered m = -l..l, except
  p shells which keep (x, y, z);
* Cartesian s and p functions carry the angular factors 1/sqrt(4 pi) and
  sqrt(3/(4 pi)); Cartesian d and higher functions carry none.
"""

import math
import numpy as np

from . import basis as basis_mod

# Bohr radius in Angstrom used by PySCF for unit conversion (pyscf lib.param.BOHR).
BOHR = 0.52917721092

# libcint slot numbers
CHARGE_OF, PTR_COORD, NUC_MOD_OF, PTR_ZETA, PTR_FRAC_CHARGE = 0, 1, 2, 3, 4
ATM_SLOTS = 6
ATOM_OF, ANG_OF, NPRIM_OF, NCTR_OF, KAPPA_OF, PTR_EXP, PTR_COEFF = 0, 1, 2, 3, 4, 5, 6
BAS_SLOTS = 8
PTR_RANGE_OMEGA = 8
PTR_ENV_START = 20

ELEMENTS = ['X', 'H', 'He', 'Li', 'Be', 'B', 'C', 'N', 'O', 'F', 'Ne',
            'Na', 'Mg', 'Al', 'Si', 'P', 'S', 'Cl', 'Ar', 'K', 'Ca',
            'Sc', 'Ti', 'V', 'Cr', 'Mn', 'Fe', 'Co', 'Ni', 'Cu', 'Zn',
            'Ga', 'Ge', 'As', 'Se', 'Br', 'Kr']
_CHARGE = {s.upper(): z for z, s in enumerate(ELEMENTS)}


def charge_of(symb):
    s = ''.join(c for c in str(symb) if c.isalpha())
    return _CHARGE[s.upper()]


def std_symbol(symb):
    s = ''.join(c for c in str(symb) if c.isalpha())
    return ELEMENTS[_CHARGE[s.upper()]]


def gaussian_int(n, alpha):
    """int_0^inf x^n exp(-alpha x^2) dx."""
    n1 = (n + 1) * .5
    return math.gamma(n1) / (2. * alpha**n1)


def gto_norm(l, expnt):
    """Radial normalisation of r^l exp(-expnt r^2)."""
    return 1. / math.sqrt(gaussian_int(l * 2 + 2, 2 * expnt))


def ncart(l):
    return (l + 1) * (l + 2) // 2


def nsph(l):
    return 2 * l + 1


def cart_components(l):
    """(lx, ly, lz) in libcint order."""
    out = []
    for lx in range(l, -1, -1):
        for ly in range(l - lx, -1, -1):
            out.append((lx, ly, l - lx - ly))
    return out


def common_fac_sp(l):
    if l == 0:
        return 0.282094791773878143
    if l == 1:
        return 0.488602511902919921
    return 1.


def _binom(n, k):
    if k < 0 or k > n:
        return 0
    return math.comb(n, k)


def cart2sph_coeff(l):
    """Matrix c2s [ncart(l), nsph(l)] mapping raw Cartesian components to
    unit-sphere-normalised real solid harmonics.

    The solid harmonics come from the closed-form Cartesian expansion of the
    real regular solid harmonics (Helgaker, Jorgensen, Olsen, "Molecular
    Electronic-Structure Theory", eq. 6.4.47-6.4.50), scaled by
    sqrt((2l+1)/(4 pi)).  p shells keep Cartesian order (x, y, z).
    """
    comps = cart_components(l)
    index = {c: i for i, c in enumerate(comps)}
    c2s = np.zeros((len(comps), 2 * l + 1))
    scale = math.sqrt((2 * l + 1) / (4 * math.pi))
    if l == 1:
        for i in range(3):
            c2s[i, i] = scale
        return c2s
    for col, m in enumerate(range(-l, l + 1)):
        am = abs(m)
        nlm = math.sqrt(2. * math.factorial(l + am) * math.factorial(l - am)
                        / (2. if m == 0 else 1.)) / (2**am * math.factorial(l))
        vm = 0.5 if m < 0 else 0.
        for t in range((l - am) // 2 + 1):
            for u in range(t + 1):
                # v runs over vm, vm+1, ... up to floor(am/2 - vm) + vm
                nv = int(math.floor(am / 2. - vm)) + 1
                for iv in range(nv):
                    v = vm + iv
                    two_v = int(round(2 * v))
                    c = ((-1)**(t + iv) * 0.25**t * _binom(l, t) * _binom(l - t, am + t)
                         * _binom(t, u) * _binom(am, two_v))
                    lx = 2 * t + am - 2 * u - two_v
                    ly = 2 * u + two_v
                    lz = l - 2 * t - am
                    if lx < 0 or c == 0:
                        continue
                    c2s[index[(lx, ly, lz)], col] += nlm * c * scale
    return c2s


def _normalize_contracted(l, exps, coeffs):
    """coeffs [nprim, nctr] -> normalised coefficients including gto_norm."""
    exps = np.asarray(exps, dtype=np.float64)
    cs = np.asarray(coeffs, dtype=np.float64).reshape(len(exps), -1)
    norms = np.array([gto_norm(l, e) for e in exps])
    cs = cs * norms[:, None]
    ee = exps[:, None] + exps[None, :]
    n1 = (2 * l + 3) * .5
    ee = np.vectorize(lambda a: math.gamma(n1) / (2. * a**n1))(ee)
    s1 = 1. / np.sqrt(np.einsum('pi,pq,qi->i', cs, ee, cs))
    return cs * s1[None, :]


def _parse_atoms(atom, unit):
    if isinstance(atom, str):
        items = []
        for line in atom.replace(';', '\n').splitlines():
            line = line.replace(',', ' ').strip()
            if not line or line.startswith('#'):
                continue
            tok = line.split()
            items.append((tok[0], [float(x) for x in tok[1:4]]))
    else:
        items = []
        for a in atom:
            symb, xyz = a[0], a[1]
            if isinstance(symb, (int, np.integer)):
                symb = ELEMENTS[int(symb)]
            items.append((symb, [float(x) for x in xyz]))
    conv = 1. if str(unit).upper().startswith('B') or str(unit).upper() == 'AU' else 1. / BOHR
    return [(s, np.asarray(c) * conv) for s, c in items]


class Mole:
    """Molecule with libcint-layout integral environment.

    Attributes mirror pyscf.gto.Mole: atom, basis, unit, charge, spin, cart,
    omega, natm, nbas, nao, nelectron, _atm, _bas, _env, ao_loc.
    """

    def __init__(self, atom=None, basis='sto-3g', unit='Angstrom', charge=0,
                 spin=0, cart=False, verbose=0):
        self.atom = atom
        self.basis = basis
        self.unit = unit
        self.charge = charge
        self.spin = spin
        self.cart = cart
        self.verbose = verbose
        self._omega = 0.
        self._built = False

    # -- construction -----------------------------------------------------
    def build(self):
        atoms = _parse_atoms(self.atom, self.unit)
        self._atom = [(std_symbol(s), c) for s, c in atoms]
        env = [0.] * PTR_ENV_START
        atm = []
        for symb, coord in self._atom:
            ptr = len(env)
            env.extend(coord.tolist())
            env.append(0.)  # zeta for point nuclei
            atm.append([charge_of(symb), ptr, 1, ptr + 3, 0, 0])
        bas = []
        self._basis = {}
        for ia, (symb, coord) in enumerate(self._atom):
            shells = basis_mod.resolve(self.basis, symb)
            self._basis[symb] = shells
            for shell in shells:
                l = int(shell[0])
                prims = [list(p) for p in shell[1:]]
                exps = [p[0] for p in prims]
                coeffs = np.array([p[1:] for p in prims], dtype=np.float64)
                cs = _normalize_contracted(l, exps, coeffs)
                nprim, nctr = cs.shape
                pexp = len(env)
                env.extend(exps)
                pcoeff = len(env)
                env.extend(cs.T.ravel().tolist())
                bas.append([ia, l, nprim, nctr, 0, pexp, pcoeff, 0])
        self._atm = np.asarray(atm, dtype=np.int32).reshape(-1, ATM_SLOTS)
        self._bas = np.asarray(bas, dtype=np.int32).reshape(-1, BAS_SLOTS)
        self._env = np.asarray(env, dtype=np.float64)
        self._env[PTR_RANGE_OMEGA] = self._omega
        self._built = True
        return self

    # -- properties --------------------------------------------------------
    @property
    def omega(self):
        return self._omega

    @omega.setter
    def omega(self, w):
        self._omega = float(w)
        if self._built:
            self._env[PTR_RANGE_OMEGA] = self._omega

    @property
    def natm(self):
        return len(self._atm)

    @property
    def nbas(self):
        return len(self._bas)

    def atom_charges(self):
        return self._atm[:, CHARGE_OF].copy()

    def atom_coords(self):
        ptr = self._atm[:, PTR_COORD]
        return np.stack([self._env[p:p + 3] for p in ptr])

    def atom_symbol(self, ia):
        return self._atom[ia][0]

    @property
    def nelectron(self):
        return int(self._atm[:, CHARGE_OF].sum()) - self.charge

    @property
    def nelec(self):
        ne = self.nelectron
        nb = (ne - self.spin) // 2
        return ne - nb, nb

    def bas_angular(self, i):
        return int(self._bas[i, ANG_OF])

    def bas_nctr(self, i):
        return int(self._bas[i, NCTR_OF])

    def ao_loc_nr(self, cart=None):
        cart = self.cart if cart is None else cart
        l = self._bas[:, ANG_OF]
        nf = (l + 1) * (l + 2) // 2 if cart else 2 * l + 1
        dims = nf * self._bas[:, NCTR_OF]
        return np.append(0, np.cumsum(dims)).astype(np.int32)

    @property
    def ao_loc(self):
        return self.ao_loc_nr()

    @property
    def nao(self):
        return int(self.ao_loc_nr()[-1])

    def nao_nr(self, cart=None):
        return int(self.ao_loc_nr(cart)[-1])

    def energy_nuc(self):
        z = self.atom_charges().astype(np.float64)
        r = self.atom_coords()
        e = 0.
        for i in range(len(z)):
            for j in range(i):
                e += z[i] * z[j] / np.linalg.norm(r[i] - r[j])
        return e

    def copy(self):
        import copy
        return copy.deepcopy(self)

    def set_geom_(self, atom, unit=None):
        self.atom = atom
        if unit is not None:
            self.unit = unit
        return self.build()

    def cart2sph_coeff(self):
        """Block-diagonal [nao_cart, nao_sph] transformation of the user basis."""
        lc = self.ao_loc_nr(cart=True)
        ls = self.ao_loc_nr(cart=False)
        c = np.zeros((lc[-1], ls[-1]))
        for ib in range(self.nbas):
            l = self.bas_angular(ib)
            blk = cart2sph_coeff(l)
            nc, ns = blk.shape
            for k in range(self.bas_nctr(ib)):
                c[lc[ib] + k * nc: lc[ib] + (k + 1) * nc,
                  ls[ib] + k * ns: ls[ib] + (k + 1) * ns] = blk
        return c


def M(**kwargs):
    """Create and build a Mole (mirrors pyscf.M)."""
    omega = kwargs.pop('omega', None)
    mol = Mole(**kwargs)
    mol.build()
    if omega is not None:
        mol.omega = omega
    return mol
