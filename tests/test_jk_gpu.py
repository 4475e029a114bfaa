"""GPU parity of the J/K engine against the CPU oracle (through the C ABI).

Tolerances: FP64 mode max|dJ|, max|dK| <= 1e-10 (the bound the reference's
tests use against PySCF, gpu4pyscf/scf/tests/test_scf_jk.py:105-106);
mixed mode <= 1e-7 elementwise.
"""
import json
import os

import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

H2O = 'O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696'
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), 'golden', 'reference_fingerprints.json')))


def _jk():
    from gpu4pyscf_gb300.scf import jk
    return jk


def _rand_dm(n, seed, sym=True, ndm=None):
    rng = np.random.default_rng(seed)
    shape = (n, n) if ndm is None else (ndm, n, n)
    dm = rng.random(shape) - .3
    if sym:
        dm = dm + np.swapaxes(dm, -1, -2)
    return dm


@pytest.mark.parametrize('basis', ['sto-3g', 'syn-cc-pvdz', 'syn-6-31g*'])
@pytest.mark.parametrize('hermi', [1, 0])
def test_h2o_fp64(basis, hermi):
    jk = _jk()
    mol = gto.M(atom=H2O, basis=basis)
    dm = _rand_dm(mol.nao, 1, sym=(hermi == 1))
    vj, vk = jk.get_jk(mol, dm, hermi=hermi)
    rj, rk = orc.get_jk(mol, dm, hermi=hermi, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_f_shells_fp64_multi_dm():
    """Every class up to (ff|ff) on a three-atom molecule, two densities."""
    jk = _jk()
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3', basis='syn-def2-tzvp')
    dm = _rand_dm(mol.nao, 2, ndm=2)
    vj, vk = jk.get_jk(mol, dm, hermi=1)
    rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_cartesian_and_hermi0_f():
    jk = _jk()
    mol = gto.M(atom='N 0 0 0; O 0 0 2.1', basis='syn-def2-tzvp', cart=True)
    dm = _rand_dm(mol.nao, 3, sym=False)
    vj, vk = jk.get_jk(mol, dm, hermi=0)
    rj, rk = orc.get_jk(mol, dm, hermi=0, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_golden_o2_sto3g_hermi2():
    """The reference's hermi=2 fingerprint (test_scf_jk.py:371-386) on the GPU."""
    jk = _jk()
    g = GOLD['o2_sto3g_hermi2']
    mol = gto.M(atom=g['atom'], basis=g['basis'])
    np.random.seed(g['seed'])
    nao = mol.nao
    dm = np.random.rand(2, nao, nao)
    dm = dm - dm.transpose(0, 2, 1)
    vj, vk = jk.get_jk(mol, dm, hermi=2)
    assert abs(orc.fp(vk.cpu().numpy()) - g['fp_vk']) < g['tol']
    assert abs(vj.cpu().numpy()).sum() < 1e-12


def test_get_j_get_k_consistent():
    jk = _jk()
    mol = gto.M(atom=H2O, basis='syn-def2-svp')
    opt = jk._VHFOpt(mol).build()
    dm = _rand_dm(mol.nao, 4)
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(jk.get_j(mol, dm, hermi=1, vhfopt=opt) - vj).max().item() < 1e-12
    assert abs(jk.get_k(mol, dm, hermi=1, vhfopt=opt) - vk).max().item() < 1e-12


def test_schwarz_factors_match_oracle():
    jk = _jk()
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3', basis='syn-def2-tzvp')
    opt = jk._VHFOpt(mol).build()
    q = opt.q_cond()
    sb = opt.sorted_mol

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    qref = orc.qcond(Raw)
    mask = q > 0
    assert mask.sum() > 0.9 * mask.size
    assert np.allclose(q[mask], qref[mask], rtol=1e-6, atol=0)


def test_screening_tolerance():
    """With the default direct_scf_tol=1e-13 the result stays within 1e-10."""
    jk = _jk()
    mol = gto.M(atom='O 0 0 0; H 0 0.9 0.3; C 0 -1.2 0.8; H 4 0 0; H 0 5 1', basis='syn-cc-pvdz')
    dm = _rand_dm(mol.nao, 5)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_mixed_precision_close_to_fp64():
    jk = _jk()
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3; N 2.5 1 0', basis='syn-def2-tzvp')
    dm = _rand_dm(mol.nao, 6) * .1
    opt = jk._VHFOpt(mol).build()
    vj64, vk64 = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    opt.precision = 'mixed'
    opt.split_thresh = 1e-6
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vj - vj64).max().item() < 1e-7
    assert abs(vk - vk64).max().item() < 1e-7
