"""Nuclear gradient of the J/K energy on the GPU (scf/grad_jk.py: the
dedicated derivative kernels, and the route through the J/K kernels of the
extended basis) against the oracle's analytic gradient (pinned by finite
differences in tests/test_oracle_grad.py) and against each other.  Follows the
reference's check of _jk_energy_per_atom against int2e_ip1 contractions
(gpu4pyscf/scf/tests/test_scf_jk.py:388-413).  Collected after the J/K
parity tests it builds on (and before the allocation-free test, which must
come last)."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

H2O = 'O 0 0.1 0.2; H -1.4 0.1 -0.8; H 1.5 -0.2 -0.7'


@pytest.mark.parametrize('method', ['ip1', 'extended'])
@pytest.mark.parametrize('basis, cart, jf, kf, omega', [
    ('syn-6-31g*', False, 1., .5, 0.),
    ('syn-cc-pvdz', True, 1., 1., 0.),
    ('syn-def2-svp', False, 0., 1., 0.),
    ('syn-6-31g*', False, 0., 1., -0.3),
    ('syn-6-31g*', False, 1., 1., 0.4),
    ('syn-def2-tzvp', False, 1., .5, 0.),
])
def test_grad_vs_oracle(basis, cart, jf, kf, omega, method):
    from gpu4pyscf_gb300.scf import grad_jk
    mol = gto.M(atom=H2O, basis=basis, unit='B', cart=cart)
    mol.omega = omega
    rng = np.random.default_rng(6)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    g = grad_jk.jk_energy_grad(mol, dm, jf, kf, direct_scf_tol=1e-15, method=method).cpu().numpy()
    ref = orc.jk_energy_grad(mol, dm, jf, kf)
    # observed: 1e-13 .. 1e-11 absolute, below 3e-14 relative to the
    # largest component, for every case here (the looser bound an earlier
    # version needed came from a density-dependent pair cut that dropped
    # pairs of the raised shells, whose coefficients 2 alpha c are large)
    scale = max(1., abs(ref).max())
    assert abs(g - ref).max() < 1e-10 * scale
    assert abs(g.sum(axis=0)).max() < 1e-10 * scale


def test_reference_entry():
    from gpu4pyscf_gb300.scf import grad_jk, jk
    mol = gto.M(atom='O 0 0.7375 -0.0528; O 0 -0.7375 -0.1528', basis='syn-def2-svp')
    rng = np.random.default_rng(12)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    opt = jk._VHFOpt(mol).build()
    e = grad_jk._jk_energy_per_atom(opt, dm, j_factor=1., k_factor=.5)
    ref = orc.jk_energy_grad(mol, dm, 1., .5)
    assert abs(e - ref).max() < 1e-10 * max(1., abs(ref).max())


def test_antisymmetric_density_k():
    """The reference's own case (gpu4pyscf/scf/tests/test_scf_jk.py:388-403):
    K-only gradient of an antisymmetric density."""
    from gpu4pyscf_gb300.scf import grad_jk, jk
    mol = gto.M(atom='O 0 0.7375 -0.0528; O 0 -0.7375 -0.1528', basis='syn-def2-svp')
    rng = np.random.default_rng(12)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm1 = a - a.T
    opt = jk._VHFOpt(mol).build()
    e = grad_jk._jk_energy_per_atom(opt, dm1, j_factor=0, k_factor=1.)
    ref = orc.jk_energy_grad(mol, dm1, 0., 1.)
    assert abs(e - ref).max() < 1e-10 * max(1., abs(ref).max())


def test_spin_densities():
    """Two spin densities: J of their sum and K of each with k_factor not
    halved, which is the one-density gradient of the sum (J only) plus the
    one-density K gradients with twice the factor."""
    from gpu4pyscf_gb300.scf import grad_jk, jk
    mol = gto.M(atom=H2O, basis='syn-def2-svp', unit='B')
    rng = np.random.default_rng(14)
    a = rng.random((mol.nao, mol.nao)) - .5
    b = rng.random((mol.nao, mol.nao)) - .5
    da, db = a @ a.T, .5 * b @ b.T
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-15).build()
    g2 = grad_jk._jk_energy_per_atom(opt, np.stack([da, db]), j_factor=1., k_factor=.7)
    ref = (grad_jk._jk_energy_per_atom(opt, da + db, j_factor=1., k_factor=0.)
           + grad_jk._jk_energy_per_atom(opt, da, j_factor=0., k_factor=1.4)
           + grad_jk._jk_energy_per_atom(opt, db, j_factor=0., k_factor=1.4))
    assert abs(g2 - ref).max() < 1e-11 * max(1., abs(ref).max())
    ro = orc.jk_energy_grad(mol, da + db, 1., 0.) + orc.jk_energy_grad(mol, da, 0., 1.4) \
        + orc.jk_energy_grad(mol, db, 0., 1.4)
    assert abs(g2 - ro).max() < 1e-10 * max(1., abs(ro).max())


def test_ip1_vs_extended_larger():
    """A 12-atom molecule with f shells: the dedicated kernels against the
    extended-basis route (two independent GPU paths), with the optimizer
    reused and the default screening."""
    import bench
    from gpu4pyscf_gb300.scf import grad_jk, jk
    mol = bench.make_mol('c30')
    mol = gto.M(atom=[mol._atom[i] for i in range(12)], basis='syn-def2-tzvp', unit='B')
    rng = np.random.default_rng(15)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T / mol.nao
    opt = jk._VHFOpt(mol).build()
    g1 = grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt).cpu().numpy()
    g2 = grad_jk.jk_energy_grad(mol, dm, 1., .5, method='extended').cpu().numpy()
    scale = max(1., abs(g2).max())
    assert abs(g1 - g2).max() < 1e-9 * scale
    assert abs(g1.sum(axis=0)).max() < 1e-9 * scale
    # the optimizer still builds J/K after a gradient build
    vj, vk = jk.get_jk(mol, dm, hermi=1, vhfopt=opt)
    rj, rk = jk.get_jk(mol, dm, hermi=1)
    assert abs(vj - rj).max().item() < 1e-10 and abs(vk - rk).max().item() < 1e-10


def test_g_shells_rejected_by_ip1():
    from gpu4pyscf_gb300.scf import grad_jk
    mol = gto.M(atom='O 0 0 0; H 0 0 1.8', basis=('syn-6-31g*', [[4, [1.1, 1.]]]), unit='B')
    with pytest.raises((NotImplementedError, RuntimeError)):
        grad_jk.jk_energy_grad(mol, np.eye(mol.nao))
