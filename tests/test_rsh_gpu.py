"""Range-separated J/K on the GPU against the oracle (jk_build_rsh).

Follows the reference's checks in gpu4pyscf/scf/tests/test_scf_jk.py:59-80
(mol.omega = +-0.2 for J and K, vj(w) + vj(-w) = vj(0)) and the factor
convention of gpu4pyscf/scf/jk.py:1122-1168.  FP64 tolerance 1e-10 as for
the full-range operator; mixed precision 1e-7.
"""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TZ = 'O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3'


def _rand_dm(n, seed, sym=True):
    rng = np.random.default_rng(seed)
    dm = rng.random((n, n)) - .3
    return dm + dm.T if sym else dm


def _oracle(mol, dm, omega, hermi=1):
    old = mol.omega
    mol.omega = omega
    try:
        return orc.get_jk(mol, dm, hermi=hermi, tol=0.)
    finally:
        mol.omega = old


@pytest.mark.parametrize('omega', [0.2, -0.2, 0.9])
@pytest.mark.parametrize('hermi', [1, 0])
def test_mol_omega(omega, hermi):
    """mol.omega attenuates J and K (classes up to (ff|ff))."""
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom=TZ, basis='syn-def2-tzvp')
    dm = _rand_dm(mol.nao, 4, sym=hermi == 1)
    rj, rk = _oracle(mol, dm, omega, hermi)
    mol.omega = omega
    vj, vk = jk.get_jk(mol, dm, hermi=hermi)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-10
    assert abs(vk.cpu().numpy() - rk).max() < 1e-10


def test_identity_and_factors():
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-cc-pvdz')
    dm = _rand_dm(mol.nao, 7)
    opt = jk._VHFOpt(mol).build()
    j0, k0 = (x.cpu().numpy() for x in jk.get_jk(mol, dm, hermi=1, vhfopt=opt))
    mol.omega = 0.3
    j1, k1 = (x.cpu().numpy() for x in jk.get_jk(mol, dm, hermi=1, vhfopt=opt))
    mol.omega = -0.3
    j2, k2 = (x.cpu().numpy() for x in jk.get_jk(mol, dm, hermi=1, vhfopt=opt))
    mol.omega = 0.
    assert abs(j1 + j2 - j0).max() < 1e-10
    assert abs(k1 + k2 - k0).max() < 1e-10
    # explicit factors: J stays full range (mol.omega = 0), K mixes the parts
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt, omega=0.3, lr_factor=0.65, sr_factor=0.19)
    assert abs(vj.cpu().numpy() - j0).max() < 1e-10
    assert abs(vk.cpu().numpy() - (0.65 * k1 + 0.19 * k2)).max() < 1e-10
    # long range only through get_k
    vk = jk.get_k(mol, dm, hermi=1, vhfopt=opt, omega=0.3)
    assert abs(vk.cpu().numpy() - k1).max() < 1e-10
    vk = jk.get_k(mol, dm, hermi=1, vhfopt=opt, omega=-0.3)
    assert abs(vk.cpu().numpy() - k2).max() < 1e-10
    # lr == sr is the full-range operator
    vk = jk.get_k(mol, dm, hermi=1, vhfopt=opt, omega=0.3, lr_factor=1., sr_factor=1.)
    assert abs(vk.cpu().numpy() - k0).max() < 1e-10


def test_rsh_mixed_precision():
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom=TZ, basis='syn-def2-tzvp')
    dm = _rand_dm(mol.nao, 9)
    rj, rk = _oracle(mol, dm, -0.25)
    mol.omega = -0.25
    opt = jk._VHFOpt(mol).build()
    opt.precision = 'mixed'
    opt.split_thresh = 1e-6
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vj.cpu().numpy() - rj).max() < 1e-7
    assert abs(vk.cpu().numpy() - rk).max() < 1e-7


def test_rsh_c_abi_errors():
    import torch
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='H 0 0 0; H 0 0 0.74', basis='sto-3g')
    opt = jk._VHFOpt(mol).build()
    n = opt.nao_sorted
    d = torch.zeros((1, n, n), dtype=torch.float64, device='cuda')
    out = torch.empty_like(d)
    lib = libjk.load()
    # omega = 0 with different factors, and no operator at all, are rejected
    for args in ((0., 1., 0.5), (0.3, 0., 0.)):
        err = lib.jk_build_rsh(opt._handle, d.data_ptr(), 1, n, 1, 1, 1, args[0], args[1], args[2], 0, 1e-6,
                               out.data_ptr(), out.data_ptr(), None, None)
        assert err == -1
        assert b'jk_build' in lib.jk_last_error()
