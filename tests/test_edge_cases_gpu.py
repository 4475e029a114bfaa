"""Edge cases of the drop-in get_jk on the GPU: a zero density, a single
s function, three densities with hermi=0, skipped J or K, a density far
larger than any the screening was planned for, and an atom pair beyond the
overlap cut.  Bars as the parity tests (1e-10 against the oracle)."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_zero_density_gives_zero():
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; H 0 0 1.8; H 1.7 0 -0.5', basis='syn-def2-svp', unit='B')
    vj, vk = jk.get_jk(mol, np.zeros((mol.nao, mol.nao)), hermi=1)
    assert float(abs(vj).max()) == 0. and float(abs(vk).max()) == 0.


def test_single_s_function():
    """One shell, one function: the (ss|ss) class only."""
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='H 0 0 0', basis='sto-3g', spin=1)
    dm = np.array([[0.7]])
    vj, vk = jk.get_jk(mol, dm, hermi=1)
    rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-12
    assert abs(vk.cpu().numpy() - rk).max() < 1e-12


def test_three_densities_hermi0_and_skips():
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='N 0 0 0; C 0 1.4 0.3; H -0.9 -0.5 0.2', basis='syn-def2-tzvp')
    rng = np.random.default_rng(31)
    dm = rng.random((3, mol.nao, mol.nao)) - .5
    rj, rk = orc.get_jk(mol, dm, hermi=0, tol=0.)
    vj, vk = jk.get_jk(mol, dm, hermi=0)
    assert vj.shape == dm.shape and vk.shape == dm.shape
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10
    vj2, vk2 = jk.get_jk(mol, dm, hermi=0, with_k=False)
    assert vk2 is None and abs(vj2.cpu().numpy() - rj).max() < 1e-10
    vj3, vk3 = jk.get_jk(mol, dm, hermi=0, with_j=False)
    assert vj3 is None and abs(vk3.cpu().numpy() - rk).max() < 1e-10


def test_large_density_keeps_every_pair():
    """Pairs are kept whatever the later densities (no density bound at
    optimizer build): a density scaled by 1e6 gives J and K scaled by 1e6."""
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; H 0 0 1.8; H 9 0 0; C 0 9 1', basis='syn-def2-svp', unit='B')
    rng = np.random.default_rng(32)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    opt = jk._VHFOpt(mol).build()
    vj1, vk1 = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    vj2, vk2 = jk.get_jk(mol, dm * 1e6, hermi=1, vhfopt=opt)
    rj, rk = orc.get_jk(mol, dm * 1e6, hermi=1, tol=0.)
    scale = max(1., float(abs(rk).max()))
    assert abs(vj2.cpu().numpy() - rj).max() < 1e-10 * max(1., float(abs(rj).max()))
    assert abs(vk2.cpu().numpy() - rk).max() < 1e-10 * scale
    assert abs(vj2 - 1e6 * vj1).max().item() < 1e-9 * float(abs(vj2).max())


def test_distant_fragments():
    """Two fragments 40 Bohr apart: their cross pairs fall under the overlap
    cut, the Coulomb coupling through J stays (D blocks of both fragments)."""
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; H 0 0 1.8; O 40 0 0; H 40 0 1.8', basis='syn-6-31g*', unit='B')
    rng = np.random.default_rng(33)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    vj, vk = jk.get_jk(mol, dm, hermi=1)
    rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10
