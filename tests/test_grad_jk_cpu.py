"""Host logic of the J/K energy gradient (scf/grad_jk.py) on the CPU: the
extended basis (shells raised with 2 alpha coefficients and lowered) and the
contraction, with the oracle's J/K of the extended basis standing in for the
engine's, against the oracle's analytic gradient."""
import types

import numpy as np
import pytest
import torch

from gpu4pyscf_gb300 import gto
from gpu4pyscf_gb300.gto.sorted_basis import SortedBasis
from gpu4pyscf_gb300.scf import grad_jk
from oracle import oracle as orc

H2O = 'O 0 0.1 0.2; H -1.4 0.1 -0.8; H 1.5 -0.2 -0.7'


@pytest.mark.parametrize('basis, cart, jf, kf', [
    ('sto-3g', False, 1., 1.),
    ('syn-6-31g*', False, 1., .5),
    ('syn-cc-pvdz', True, 0., 1.),
])
def test_extended_basis_route(basis, cart, jf, kf):
    mol = gto.M(atom=H2O, basis=basis, unit='B', cart=cart)
    rng = np.random.default_rng(4)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    sb = SortedBasis(mol)
    ext = grad_jk.extended_basis(sb)
    ds = sb.coeff @ dm @ sb.coeff.T
    dext = np.zeros((ext['nao'], ext['nao']))
    dext[np.ix_(ext['orig'], ext['orig'])] = ds
    emol = types.SimpleNamespace(_atm=ext['atm'], _bas=ext['bas'], _env=ext['env'])
    vj, vk, _ = orc.get_jk_cart(emol, dext, hermi=1)
    g = grad_jk.contract(ext, vj, vk, ds, mol.natm, jf, kf)
    ref = orc.jk_energy_grad(mol, dm, jf, kf)
    assert abs(g - ref).max() < 1e-10 * max(1., abs(ref).max())
    # the torch branch (the one the GPU path takes), here on CPU tensors
    gt = grad_jk.contract(ext, torch.as_tensor(vj), torch.as_tensor(vk), torch.as_tensor(ds),
                          mol.natm, jf, kf)
    assert abs(gt.numpy() - g).max() < 1e-12 * max(1., abs(g).max())


def test_extended_basis_layout():
    mol = gto.M(atom=H2O, basis='syn-6-31g*', unit='B')
    sb = SortedBasis(mol)
    ext = grad_jk.extended_basis(sb)
    ls = ext['bas'][:, 1]
    assert (np.diff(ls) >= 0).all()                    # sorted by l
    assert ext['nao'] == int(((ls + 1) * (ls + 2) // 2).sum())
    # every original shell has one raised copy and, for l > 0, a lowered one
    nl = np.bincount(np.asarray(sb._bas)[:, 1], minlength=4)
    ne = np.bincount(ls, minlength=4)
    assert ne[3] == nl[2] and ne[0] == nl[0] + nl[1]
    assert (ext['down'][ext['ax'] == 0] == -1).all()


def test_g_shells_rejected():
    # raised copies of g shells would need l = 5, beyond the kernels
    mol = gto.M(atom='O 0 0 0; H 0 0 1.8', basis=('syn-def2-svp', [[4, [1., 1.]]]), unit='B')
    with pytest.raises(NotImplementedError):
        grad_jk.extended_basis(SortedBasis(mol))
