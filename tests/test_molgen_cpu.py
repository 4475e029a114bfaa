"""Seeded synthetic molecules (gto/molgen.py): the random walk's bond and
clearance laws, and H-saturated molecules (closed shell, every valence
filled), on the CPU."""
import numpy as np
import pytest

from gpu4pyscf_gb300.gto import molgen

VAL = molgen.VALENCE


def _bonds(atoms, cut=1.55):
    X = np.array([c for _, c in atoms])
    D = np.linalg.norm(X[:, None] - X[None], axis=-1)
    np.fill_diagonal(D, np.inf)
    return D, D < cut


@pytest.mark.parametrize('seed', [0, 1, 2])
def test_walk_laws(seed):
    atoms = molgen.random_molecule({'C': 10, 'N': 3, 'O': 5, 'H': 12}, seed)
    assert len(atoms) == 30
    heavy = [k for k, (s, _) in enumerate(atoms) if s != 'H']
    D, _ = _bonds(atoms)
    # every heavy atom but the first bonds to an earlier one at 1.0-1.5 A
    for k in heavy[1:]:
        assert 1.0 - 1e-9 <= D[k, :k].min() <= 1.5 + 1e-9


@pytest.mark.parametrize('seed', [11, 12, 13, 14])
def test_saturated(seed):
    f = {'C': 9, 'N': 3, 'O': 4}
    for s in range(seed, seed + 50 * 1000003, 1000003):
        try:
            atoms = molgen.random_molecule(f, s, saturate=True)
            break
        except RuntimeError:
            continue
    syms = [a for a, _ in atoms]
    z = {'C': 6, 'N': 7, 'O': 8, 'H': 1}
    assert sum(z[a] for a in syms) % 2 == 0
    D, _ = _bonds(atoms)
    nheavy = sum(1 for a in syms if a != 'H')
    # hydrogens: 1.0-1.1 A from their heavy atom; 1.6 A from other
    # hydrogens and 1.8 A from other heavy atoms, except 1.45 A where one
    # of the two lies within 1.6 A of the other's heavy atom
    par = {k: int(np.argmin(D[k, :nheavy])) for k, a in enumerate(syms) if a == 'H'}
    for k, p in par.items():
        assert 1.0 - 1e-9 <= D[k, p] <= 1.1 + 1e-9
        for j, b in enumerate(syms):
            if j == k or j == p:
                continue
            near = D[p, j] < 1.6 or (b == 'H' and D[par[j], k] < 1.6)
            lim = 1.45 if near else (1.6 if b == 'H' else 1.8)
            assert D[k, j] >= lim - 1e-9
    # H count = free valences of the heavy-atom tree: sum(val) - 2 (n - 1)
    nh = syms.count('H')
    assert nh == sum(VAL[a] for a in syms if a != 'H') - 2 * (nheavy - 1)
