"""Batched J/K for several molecules in shared class launches, and its CUDA
graph replay, against per-molecule builds and the oracle."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from gpu4pyscf_gb300.gto import molgen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _mols():
    rng = np.random.default_rng(5)
    out = [gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-6-31g*')]
    for seed, n in ((1, 5), (2, 9), (3, 14)):
        out.append(molgen.make_mol(molgen.formula_for(n, rng), seed, 'syn-6-31g*'))
    out.append(gto.M(atom='N 0 0 0; C 0 0 1.3; O 1.2 0 1.9', basis='syn-def2-tzvp'))
    return out


def _dms(mols, seed=0):
    rng = np.random.default_rng(seed)
    res = []
    for i, m in enumerate(mols):
        k = 1 + i % 3
        x = rng.normal(size=(k, m.nao, m.nao)) / m.nao
        res.append(x @ x.transpose(0, 2, 1))
    return res


def test_batch_matches_single_builds():
    from gpu4pyscf_gb300.scf import jk, jk_batch
    mols = _mols()
    dms = _dms(mols)
    b = jk_batch.BatchJK(mols)
    js, ks = b.get_jk(dms, hermi=1)
    for m, d, vj, vk in zip(mols, dms, js, ks):
        rj, rk = jk.get_jk(m, d, hermi=1)
        assert abs(vj - rj).max().item() < 1e-11
        assert abs(vk - rk).max().item() < 1e-11
    rj, rk = orc.get_jk(mols[0], dms[0], hermi=1)
    assert abs(js[0].cpu().numpy() - rj).max() < 1e-10
    assert abs(ks[0].cpu().numpy() - rk).max() < 1e-10


def test_batch_hermi0():
    from gpu4pyscf_gb300.scf import jk, jk_batch
    mols = _mols()[:3]
    rng = np.random.default_rng(2)
    dms = [rng.random((2, m.nao, m.nao)) - .5 for m in mols]
    b = jk_batch.BatchJK(mols)
    js, ks = b.get_jk(dms, hermi=0)
    for m, d, vj, vk in zip(mols, dms, js, ks):
        rj, rk = jk.get_jk(m, d, hermi=0)
        assert abs(vj - rj).max().item() < 1e-11
        assert abs(vk - rk).max().item() < 1e-11


def test_batch_graph_replay():
    import torch
    from gpu4pyscf_gb300.scf import jk_batch
    mols = _mols()
    b = jk_batch.BatchJK(mols)
    dms0 = _dms(mols, 0)
    dms1 = _dms(mols, 1)
    b.capture(dms0)
    for dms in (dms1, dms0, dms1):
        out = b.replay(dms)
        torch.cuda.synchronize()
        ref = b.get_jk(dms)
        for a, r in zip(out[0] + out[1], ref[0] + ref[1]):
            assert abs(a - r).max().item() < 1e-11


def test_variants_and_autotune_keep_results():
    """Every launch variant the autotuner can pick gives the same J/K (the
    pattern of the reference's scheme monkeypatch test,
    gpu4pyscf/scf/tests/test_scf_j_engine.py:75-93)."""
    import torch
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3; N 2.4 0.8 -0.3', basis='syn-def2-tzvp')
    rng = np.random.default_rng(4)
    dm = rng.random((mol.nao, mol.nao)) - .4
    dm = dm + dm.T
    opt = jk._VHFOpt(mol).build()
    ref_j, ref_k = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    nq = libjk.load().jk_n_quartet_classes()
    for alt, grid in ((1, 0), (0, 1), (1, 3), (0, 8)):
        for q in range(nq):
            opt.set_variant(q, 0, alt, grid)
        vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
        assert abs(vj - ref_j).max().item() < 1e-11, (alt, grid)
        assert abs(vk - ref_k).max().item() < 1e-11, (alt, grid)
    for q in range(nq):
        opt.set_variant(q, 0, 0, 0)
    opt.tune(dm)
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    assert abs(vj - ref_j).max().item() < 1e-11
    assert abs(vk - ref_k).max().item() < 1e-11
    torch.cuda.synchronize()
