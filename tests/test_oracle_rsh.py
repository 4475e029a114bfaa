"""Range-separated operators in the CPU oracle (omega in env[8], libcint's
convention: omega > 0 erf(omega r)/r, omega < 0 erfc(|omega| r)/r).

The oracle's attenuated Hermite integrals are pinned against closed forms
that do not go through the Boys function: two normalised s Gaussians of
exponent a on centres R apart give charge clouds of exponent 2a, whose
Coulomb energy is erf(sqrt(mu) R)/R with 1/mu = 1/(2a) + 1/(2b); the
operator erf(omega r)/r is the potential of a Gaussian charge of exponent
omega^2, which adds 1/omega^2 to 1/mu.  On top: full = long + short range
for every integral class up to d, the long range tends to the full operator
as omega grows, and the reference's own check vj(w) + vj(-w) = vj(0)
(gpu4pyscf/scf/tests/test_scf_jk.py:79-80).
"""
import math

import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc


def _coulomb_s(a, b, R, omega=None):
    inv_mu = 1. / (2 * a) + 1. / (2 * b)
    if omega is not None:
        inv_mu += 1. / omega ** 2
    mu = 1. / inv_mu
    if R == 0:
        return 2. * math.sqrt(mu / math.pi)
    return math.erf(math.sqrt(mu) * R) / R


def _h2(R, a, omega=0.):
    mol = gto.M(atom='H 0 0 0; H 0 0 %r' % R, basis={'H': [[0, [a, 1.]]]}, unit='B')
    mol.omega = omega
    return mol


@pytest.mark.parametrize('a', [0.8, 3.1])
@pytest.mark.parametrize('R', [0., 0.7, 2.5])
@pytest.mark.parametrize('omega', [0.0, 0.3, 1.7, -0.3, -1.7])
def test_ss_closed_form(a, R, omega):
    b = a
    eri = orc.eri(_h2(R, a, omega))
    full = _coulomb_s(a, b, R)
    lr = _coulomb_s(a, b, R, abs(omega)) if omega else full
    want = full if omega == 0 else (lr if omega > 0 else full - lr)
    assert abs(eri[0, 0, 1, 1] - want) < 1e-12


def test_full_equals_long_plus_short():
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-cc-pvdz')
    full = orc.eri(mol)
    mol.omega = 0.4
    lr = orc.eri(mol)
    mol.omega = -0.4
    sr = orc.eri(mol)
    assert abs(lr + sr - full).max() < 1e-12
    assert abs(lr).max() > 1e-2 and abs(sr).max() > 1e-2
    # permutational symmetry survives the attenuation
    assert abs(lr - lr.transpose(2, 3, 0, 1)).max() < 1e-13
    assert abs(lr - lr.transpose(1, 0, 2, 3)).max() < 1e-13


def test_long_range_limits():
    mol = gto.M(atom='N 0 0 0; H 0 0.9 0.3', basis='syn-6-31g*')
    full = orc.eri(mol)
    # the short-range remainder erfc(omega r)/r integrates to ~ pi/omega^2
    # times the charge densities (tight core primitives make it visible)
    mol.omega = 1e3
    d3 = abs(orc.eri(mol) - full).max()
    mol.omega = 1e4
    d4 = abs(orc.eri(mol) - full).max()
    assert d4 < 1e-5 and 90 < d3 / d4 < 110
    mol.omega = 1e-4
    assert abs(orc.eri(mol)).max() < 1e-3


def test_jk_identity():
    mol = gto.M(atom='O 0 0 0; H 0 0.8 0.5; H 0 -0.8 0.5', basis='syn-cc-pvdz')
    rng = np.random.default_rng(5)
    dm = rng.random((mol.nao, mol.nao))
    dm = dm + dm.T
    j0, k0 = orc.get_jk(mol, dm, hermi=1)
    mol.omega = 0.2
    j1, k1 = orc.get_jk(mol, dm, hermi=1)
    mol.omega = -0.2
    j2, k2 = orc.get_jk(mol, dm, hermi=1)
    assert abs(j1 + j2 - j0).max() < 1e-11
    assert abs(k1 + k2 - k0).max() < 1e-11
    assert abs(j1 - j0).max() > 1e-2
