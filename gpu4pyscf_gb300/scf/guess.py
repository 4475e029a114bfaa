"""Initial densities.

block_density: per-atom block-diagonal positive semidefinite density (X X^T
of seeded Gaussian X on each atom's AOs) scaled so that each block's trace
equals the atom's electron count.  It has the atom-block sparsity of a
superposition-of-atomic-densities guess and serves as a GPU-free density of
realistic screening behaviour.
"""
import numpy as np


def atom_ao_slices(mol):
    bas = np.asarray(mol._bas)
    ls = bas[:, 1]
    nf = (ls + 1) * (ls + 2) // 2 if mol.cart else 2 * ls + 1
    loc = np.append(0, np.cumsum(nf * bas[:, 3]))
    out = {}
    for ib in range(len(bas)):
        ia = int(bas[ib, 0])
        lo, hi = out.get(ia, (loc[ib], loc[ib + 1]))
        out[ia] = (min(lo, loc[ib]), max(hi, loc[ib + 1]))
    return [out[ia] for ia in sorted(out)]


def block_density(mol, seed=0):
    rng = np.random.default_rng(seed)
    n = mol.nao
    dm = np.zeros((n, n))
    z = np.asarray(mol._atm[:, 0])
    for ia, (lo, hi) in enumerate(atom_ao_slices(mol)):
        m = hi - lo
        x = rng.normal(size=(m, m)) / np.sqrt(m)
        d = x @ x.T
        d *= z[ia] / np.trace(d)
        dm[lo:hi, lo:hi] = d
    return dm
