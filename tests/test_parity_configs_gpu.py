"""GPU parity of the benchmarked workloads against the CPU oracle.

The bench line times J/K builds of the 30-atom C10N3O5H12 molecule
(syn-def2-tzvp, 720 sorted Cartesian functions) for its SAD density and for
a dense SCF density, and of a 64-molecule syn-6-31g* batch.  These tests
check exactly those builds, through the C ABI, against the oracle's J/K of
the same sorted density:

* FP64: max |dJ|, |dK| <= 1e-10 (the bound of the reference's tests
  against PySCF, gpu4pyscf/scf/tests/test_scf_jk.py:45-57, 105-106);
* mixed FP32/FP64 at splits 1e-6 and 1e-8: <= 1e-7 elementwise and
  |dE_2e| < 1 uHa;
* the mixed split is per quartet: the FP64 and FP32 launches of a mixed
  build compute every screened quartet exactly once.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-7
MIXED_DE = 1e-6


def _c30():
    import bench
    return bench.make_mol('c30')


def _oracle_sorted(opt, dms_sorted):
    """Oracle J/K of densities given in the optimizer's sorted basis."""
    from oracle import oracle as orc
    sb = opt.sorted_mol

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    vj, vk, _ = orc.get_jk_cart(Raw, dms_sorted, hermi=1, tol=1e-13)
    return vj, vk


def _check(opt, dm_user, tag):
    import torch
    from gpu4pyscf_gb300.scf import jk  # noqa: F401
    dms = opt.apply_coeff_C_mat_CT(torch.as_tensor(dm_user, device='cuda')[None]).contiguous()
    ref_j, ref_k = _oracle_sorted(opt, dms[0].cpu().numpy())
    d = dms[0].cpu().numpy()
    opt.precision = 'fp64'
    vj, vk = opt._build(dms, 1, True, True, stats=True)
    n64 = opt.last_stats['quartets_fp64']
    ej = abs(vj[0].cpu().numpy() - ref_j).max()
    ek = abs(vk[0].cpu().numpy() - ref_k).max()
    assert ej <= FP64_TOL and ek <= FP64_TOL, (tag, 'fp64', ej, ek)
    for split in (1e-6, 1e-8):
        opt.precision, opt.split_thresh = 'mixed', split
        vj, vk = opt._build(dms, 1, True, True, stats=True)
        st = opt.last_stats
        assert st['quartets_fp64'] + st['quartets_fp32'] == n64, (tag, split, st, n64)
        dj = vj[0].cpu().numpy() - ref_j
        dk = vk[0].cpu().numpy() - ref_k
        de = 0.5 * np.sum(d * dj) - 0.25 * np.sum(d * dk)
        assert abs(dj).max() <= MIXED_TOL and abs(dk).max() <= MIXED_TOL, (tag, split)
        assert abs(de) < MIXED_DE, (tag, split, de)
    opt.precision = 'fp64'


def test_c30_sad_density_vs_oracle():
    import bench
    from gpu4pyscf_gb300.scf import jk
    mol = _c30()
    dm = bench.make_density(mol)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    _check(opt, dm, 'c30 SAD')


def test_c30_dense_density_vs_oracle():
    import bench
    mol = _c30()
    dm, mf = bench.dense_density(mol)
    _check(mf.opt, dm.cpu().numpy() if hasattr(dm, 'cpu') else dm, 'c30 dense')


def test_batch_molecules_vs_oracle():
    """Four molecules of the 64-molecule batch workload (the generator and
    seeds of the bench), all their densities, built together in one batch
    optimizer, against the oracle per molecule."""
    import bench
    import torch
    from gpu4pyscf_gb300.scf import jk_batch
    from oracle import oracle as orc
    mols, dms = bench.make_batch(nmol=64)
    pick = [0, 17, 38, 63]
    sel = [mols[i][0] for i in pick]
    b = jk_batch.BatchJK(sel)
    dsel = [torch.as_tensor(dms[i], device='cuda') for i in pick]
    js, ks = b.get_jk(dsel, hermi=1)
    for m, d, vj, vk in zip(sel, [dms[i] for i in pick], js, ks):
        rj, rk = orc.get_jk(m, d, hermi=1)
        assert abs(vj.cpu().numpy() - rj).max() <= FP64_TOL
        assert abs(vk.cpu().numpy() - rk).max() <= FP64_TOL


def test_batch_mixed_quartet_identity():
    """The whole 64-molecule batch: every mixed build computes each screened
    quartet exactly once (FP64 + FP32 counts equal the FP64 build's), so
    its error against FP64 stays below the split's FP32 error and the
    looser split never beats the tighter one by orders of magnitude."""
    import bench
    import torch
    from gpu4pyscf_gb300.scf import jk_batch
    mols, dms = bench.make_batch(nmol=64)
    dd = [torch.as_tensor(d, device='cuda') for d in dms]
    b = jk_batch.BatchJK([m for m, _ in mols])
    j0, k0 = b.get_jk(dd, stats=True)
    n64 = b.last_stats['quartets_fp64']
    errs = {}
    for split in (1e-8, 1e-6, 1e-4, 1e-6):
        b.precision, b.split_thresh = 'mixed', split
        jm, km = b.get_jk(dd, stats=True)
        st = b.last_stats
        assert st['quartets_fp64'] + st['quartets_fp32'] == n64, (split, st, n64)
        err = max(max(float(abs(a - r).max()), float(abs(c - s).max()))
                  for a, r, c, s in zip(jm, j0, km, k0))
        assert err <= MIXED_TOL, (split, err)
        errs[split] = err
    assert errs[1e-6] < 10 * errs[1e-4] + 1e-12, errs
    b.precision = 'fp64'


def test_fp32_alternative_kernels_vs_fp64():
    """Every FP32 launch variant (the register-resident and the
    block-cooperative family, several grids) of a mixed build at a split
    that sends most quartets to FP32 stays within 1e-7 of the FP64 build."""
    import torch
    from gpu4pyscf_gb300 import gto
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='O 0 0 0; C 0 1.2 0.2; H 0.9 -0.4 0.3; N 2.4 0.8 -0.3', basis='syn-def2-tzvp')
    rng = np.random.default_rng(9)
    dm = rng.random((mol.nao, mol.nao)) - .4
    dm = dm + dm.T
    opt = jk._VHFOpt(mol).build()
    ref_j, ref_k = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    nq = libjk.load().jk_n_quartet_classes()
    opt.precision, opt.split_thresh = 'mixed', 1e-2
    for alt, grid in ((0, 0), (1, 0), (1, 2), (0, 4)):
        for q in range(nq):
            opt.set_variant(q, 1, alt, grid)
        vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
        torch.cuda.synchronize()
        assert abs(vj - ref_j).max().item() <= MIXED_TOL, (alt, grid)
        assert abs(vk - ref_k).max().item() <= MIXED_TOL, (alt, grid)
    for q in range(nq):
        opt.set_variant(q, 1, 0, 0)
    opt.precision = 'fp64'


def test_c30_j_only_vs_oracle():
    """J-only builds screen with the Coulomb blocks D_ij, D_kl alone (the
    J engine's screening): fewer quartets than a J/K build, the same J."""
    import bench
    import torch
    from gpu4pyscf_gb300.scf import jk
    mol = _c30()
    dm = bench.make_density(mol)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    dms = opt.apply_coeff_C_mat_CT(torch.as_tensor(dm, device='cuda')[None]).contiguous()
    ref_j, _ = _oracle_sorted(opt, dms[0].cpu().numpy())
    _, _ = opt._build(dms, 1, True, True, stats=True)
    n_jk = opt.last_stats['quartets_fp64']
    vj, _ = opt._build(dms, 1, True, False, stats=True)
    n_j = opt.last_stats['quartets_fp64']
    assert n_j < n_jk
    assert abs(vj[0].cpu().numpy() - ref_j).max() <= FP64_TOL
