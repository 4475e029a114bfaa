"""g shells (l = 4) on the GPU: the classes with a g shell run the generic
kernel, everything else the templated ones.  The reference handles l <= 4
on the GPU (gpu4pyscf/scf/jk.py:50) and tests g inputs
(gpu4pyscf/scf/tests/test_scf_jk.py:204-236, the geometry used here, in
Bohr, with one extra g shell of exponent 1 on every atom); with PySCF's
def2-TZVP absent, the synthetic same-structure set stands in and the oracle
is the bar: max |dJ|, |dK| <= 1e-10."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

ATOM = '''O   0.000   -0.    0.1174
H  -0.757    4.   -0.4696
H   0.757    4.   -0.4696
C   1.      1.    0.
H   4.      0.    3.
H   0.      1.    .6'''


def _mol():
    return gto.M(atom=ATOM, basis=('syn-def2-svp', [[4, [1., 1.]]]), unit='B')


@pytest.mark.parametrize('hermi', [1, 0])
def test_g_shell_jk_vs_oracle(hermi):
    from gpu4pyscf_gb300.scf import jk
    mol = _mol()
    rng = np.random.default_rng(9)
    dm = rng.random((mol.nao, mol.nao))
    if hermi == 1:
        dm = dm @ dm.T
    vj, vk = jk.get_jk(mol, dm, hermi=hermi)
    rj, rk = orc.get_jk(mol, dm, hermi=hermi, tol=0.)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_g_shell_cartesian_mixed_and_k_only():
    """Cartesian g functions; mixed precision (the g classes stay FP64);
    get_k alone."""
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom=ATOM, basis=('syn-def2-svp', [[4, [0.8, 1.]]]), unit='B', cart=True)
    rng = np.random.default_rng(10)
    dm = rng.random((2, mol.nao, mol.nao)) - .5
    dm = dm + dm.transpose(0, 2, 1)
    rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
    opt = jk._VHFOpt(mol).build()
    opt.precision, opt.split_thresh = 'mixed', 1e-6
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-7
    assert abs(vk.cpu().numpy() - rk).max() < 1e-7
    opt.precision = 'fp64'
    vk2 = jk.get_k(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vk2.cpu().numpy() - rk).max() < 1e-10
