"""The oracle's nuclear gradient of the J/K energy (oracle_jk_grad: the
quantity gpu4pyscf's _jk_energy_per_atom returns for an RHF density,
gpu4pyscf/grad/rhf.py:60-171) pinned by finite differences of the oracle's
own J/K energy at displaced geometries with the density held fixed in the AO
basis (five-point stencil), and by translational invariance.  Test
infrastructure for the GPU gradient kernels."""
import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from oracle import oracle as orc

GEOM = [('O', (0., 0., 0.2)), ('H', (-1.4, 0.1, -0.8)), ('H', (1.5, -0.2, -0.7))]


def _mol(coords, basis, cart, omega=0.):
    atom = '; '.join('%s %.12f %.12f %.12f' % (s, *c) for (s, _), c in zip(GEOM, coords))
    mol = gto.M(atom=atom, basis=basis, unit='B', cart=cart)
    mol.omega = omega
    return mol


def _energy(coords, dm, basis, cart, jf, kf, omega):
    mol = _mol(coords, basis, cart, omega)
    vj, vk = orc.get_jk(mol, dm, hermi=1)
    return .5 * jf * np.sum(dm * vj) - .25 * kf * np.sum(dm * vk)


@pytest.mark.parametrize('basis, cart, jf, kf, omega', [
    ('sto-3g', False, 1., 1., 0.),
    ('syn-6-31g*', True, 1., 0., 0.),
    ('syn-6-31g*', False, 0., 1., 0.),
    ('syn-6-31g*', False, 1., .5, -0.3),
])
def test_finite_differences(basis, cart, jf, kf, omega):
    coords = np.array([c for _, c in GEOM])
    mol = _mol(coords, basis, cart, omega)
    rng = np.random.default_rng(3)
    a = rng.random((mol.nao, mol.nao)) - .5
    dm = a @ a.T
    g = orc.jk_energy_grad(mol, dm, jf, kf)
    assert abs(g.sum(axis=0)).max() < 1e-10       # translational invariance
    h = 1e-3
    fd = np.zeros_like(g)
    for A in range(len(GEOM)):
        for x in range(3):
            e = []
            for step in (-2, -1, 1, 2):
                c = coords.copy()
                c[A, x] += step * h
                e.append(_energy(c, dm, basis, cart, jf, kf, omega))
            fd[A, x] = (e[0] - 8 * e[1] + 8 * e[2] - e[3]) / (12 * h)
    # agreement seen: 2e-12 .. 9e-11 (stencil truncation and rounding)
    assert abs(g - fd).max() < 1e-9 * max(1., abs(g).max())
