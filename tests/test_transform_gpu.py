"""The sparse C transforms of _VHFOpt (jk_sparse_mm) against dense products
with the same C, for spherical and Cartesian bases, with and without the
diffuse-primitive split, stacked and single matrices."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('cart, cutoff', [(False, None), (True, None), (False, 0.3)])
def test_sparse_transforms_match_dense(cart, cutoff):
    import torch
    from gpu4pyscf_gb300.scf import jk
    extra = [[0, [10., .3], [1., .5], [.2, .4], [.05, .2]], [4, [1.1, 1.]]]
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; N 0.757 0 -0.4696',
                basis=('syn-def2-tzvp', extra), cart=cart, spin=1)
    opt = jk._VHFOpt(mol, diffuse_cutoff=cutoff).build()
    C = opt.coeff
    ns, nu = C.shape
    rng = np.random.default_rng(5)
    D = torch.as_tensor(rng.random((2, nu, nu)), device='cuda')
    V = torch.as_tensor(rng.random((2, ns, ns)), device='cuda')
    B = torch.as_tensor(rng.random((nu, 7)), device='cuda')
    ref = C @ D @ C.T
    assert abs(opt.apply_coeff_C_mat_CT(D) - ref).max().item() < 1e-12
    assert abs(opt.apply_coeff_C_mat_CT(D[1]) - ref[1]).max().item() < 1e-12
    assert abs(opt.apply_coeff_CT_mat_C(V) - C.T @ V @ C).max().item() < 1e-12
    assert abs(opt.apply_coeff_C_mat(B) - C @ B).max().item() < 1e-12
    # numpy input
    out = opt.apply_coeff_C_mat_CT(D[0].cpu().numpy())
    assert abs(out - ref[0]).max().item() < 1e-12
