"""Deterministic accumulation (jk_opt_set_deterministic): J and K built
twice are bitwise identical, in FP64 and in mixed precision, with every
kernel family in play (register-resident, block-cooperative, and the
generic kernel of the g classes), and they agree with the default FP64
accumulation and the oracle."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_bitwise_reproducible(precision):
    import torch
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3; N 2.4 0.8 -0.3; H -0.8 1.9 0.1',
                basis=('syn-def2-tzvp', [[4, [1.1, 1.]]]))
    rng = np.random.default_rng(21)
    dm = rng.random((2, mol.nao, mol.nao)) - .4
    dm = dm + dm.transpose(0, 2, 1)
    opt = jk._VHFOpt(mol).build()
    opt.precision, opt.split_thresh = precision, 1e-4
    ref_j, ref_k = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    opt.deterministic = True
    runs = [jk.get_jk(mol, dm, hermi=1, vhfopt=opt) for _ in range(3)]
    torch.cuda.synchronize()
    for vj, vk in runs[1:]:
        assert torch.equal(vj, runs[0][0])
        assert torch.equal(vk, runs[0][1])
    # against the default accumulation: FP64 rounding of the atomics' order;
    # in mixed mode also the FP32 sums over the lanes of a warp, which the
    # default FP32 digestion forms and the deterministic one does not
    tol = 1e-11 if precision == 'fp64' else 1e-9
    assert abs(runs[0][0] - ref_j).max().item() < tol
    assert abs(runs[0][1] - ref_k).max().item() < tol
    if precision == 'fp64':
        rj, rk = orc.get_jk(mol, dm, hermi=1, tol=0.)
        assert abs(runs[0][0].cpu().numpy() - rj).max() < 1e-10
        assert abs(runs[0][1].cpu().numpy() - rk).max() < 1e-10
    opt.deterministic = False
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vj - ref_j).max().item() < tol
