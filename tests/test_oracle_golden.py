"""Pin the CPU oracle against the reference's golden fingerprints.

The molecules, basis sets, seeds and fingerprints come from the reference's
own tests (gpu4pyscf/scf/tests/test_rhf.py:168-194 and
gpu4pyscf/scf/tests/test_scf_jk.py:371-386), extracted verbatim into
tests/golden/reference_fingerprints.json by tests/golden/make_golden.py.
"""
import json
import os

import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), 'golden', 'reference_fingerprints.json')))


def _mol1():
    g = GOLD['mol1']
    return gto.M(atom=g['atom'], basis=g['basis'], unit=g['unit'])


def test_mol1_shape():
    mol = _mol1()
    assert mol.nao == 124
    assert sorted(set(mol._bas[:, 1].tolist())) == [0, 1, 2, 3, 4, 5]


@pytest.mark.parametrize('hermi', [1, 0])
def test_mol1_fingerprints(hermi):
    g = GOLD['mol1']
    mol = _mol1()
    np.random.seed(g['seed'])
    nao = mol.nao
    dm = np.random.random((2, nao, nao))
    if hermi == 1:
        dm = dm + dm.transpose(0, 2, 1)
    vj, vk = orc.get_jk(mol, dm, hermi=hermi, tol=1e-13)
    ref = g['hermi%d' % hermi]
    assert abs(orc.fp(vj) - ref['fp_vj']) < 10**-ref['places']
    assert abs(orc.fp(vk) - ref['fp_vk']) < 10**-ref['places']


def test_o2_sto3g_hermi2():
    g = GOLD['o2_sto3g_hermi2']
    mol = gto.M(atom=g['atom'], basis=g['basis'])
    np.random.seed(g['seed'])
    nao = mol.nao
    dm = np.random.rand(2, nao, nao)
    dm = dm - dm.transpose(0, 2, 1)
    vj, vk = orc.get_jk(mol, dm, hermi=0)
    assert abs(orc.fp(vk) - g['fp_vk']) < g['tol']
    assert abs(vj.sum()) < 1e-12


def test_boys_identities():
    import mpmath
    for t in (0., 1e-9, 0.3, 2.5, 17., 34.9, 35.1, 60., 200.):
        f = orc.boys(12, t)
        for m in (0, 3, 12):
            ref = float(mpmath.hyp1f1(m + 0.5, m + 1.5, -t) / (2 * m + 1))
            assert abs(f[m] - ref) <= 2e-15 * ref + 1e-300


def test_eri_symmetry_and_ssss():
    mol = gto.M(atom='H 0 0 0; H 0 0 1.1', basis='sto-3g', unit='B')
    eri = orc.eri(mol)
    assert np.allclose(eri, eri.transpose(1, 0, 2, 3), atol=1e-14)
    assert np.allclose(eri, eri.transpose(2, 3, 0, 1), atol=1e-14)
    # (ss|ss) on one centre from the closed form
    a = np.array(mol._env[mol._bas[0, 5]:mol._bas[0, 5] + 3])
    c = np.array(mol._env[mol._bas[0, 6]:mol._bas[0, 6] + 3]) / np.sqrt(4 * np.pi)
    ref = 0.
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    p, q = a[i] + a[j], a[k] + a[l]
                    ref += c[i] * c[j] * c[k] * c[l] * 2 * np.pi**2.5 / (p * q * np.sqrt(p + q))
    assert abs(eri[0, 0, 0, 0] - ref) < 1e-13


def test_jk_from_full_eri():
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-6-31g*')
    rng = np.random.default_rng(3)
    n = mol.nao
    dm = rng.random((n, n))
    eri = orc.eri(mol)
    vj, vk = orc.get_jk(mol, dm, hermi=0)
    assert np.allclose(vj, np.einsum('ijkl,ji->kl', eri, dm), atol=1e-11)
    assert np.allclose(vk, np.einsum('ijkl,jk->il', eri, dm), atol=1e-11)


def test_oracle_int1e_closed_forms():
    """Normalised spherical AOs have unit overlap; a single normalised s
    Gaussian exp(-a r^2) on a nucleus has T = 3a/2 and V = -2 Z sqrt(2a/pi)."""
    a = 0.83
    mol = gto.M(atom='He 0 0 0', basis={'He': [[0, [a, 1.]]]}, unit='B')
    assert abs(orc.int1e(mol, 'ovlp')[0, 0] - 1) < 1e-14
    assert abs(orc.int1e(mol, 'kin')[0, 0] - 1.5 * a) < 1e-13
    assert abs(orc.int1e(mol, 'nuc')[0, 0] + 2 * 2 * np.sqrt(2 * a / np.pi)) < 1e-13
    mol = gto.M(atom='O 0 0 0; H 0 0.8 0.6', basis='syn-def2-tzvp')
    s = orc.int1e(mol, 'ovlp')
    assert abs(np.diag(s) - 1).max() < 1e-12
