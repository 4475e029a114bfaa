"""Initial densities.

sad_density: superposition of atomic densities.  Each distinct element is
computed once in the molecule's own basis by a spin-restricted,
spherically averaged atomic Hartree-Fock with fractional occupations of the
ground-state configuration (e.g. O: 1s^2 2s^2 2p^4, each 2p orbital holding
4/3 electrons), on the same GPU J/K engine; the molecular guess is the
block-diagonal assembly of the atomic densities (the role of
init_guess_by_minao / init_guess_by_atom in gpu4pyscf/scf/hf.py:414-561).

block_density: per-atom block-diagonal positive semidefinite density (X X^T
of seeded Gaussian X on each atom's AOs) scaled so each block's trace is the
atom's electron count; a GPU-free density with the block sparsity of a
superposition-of-atoms guess.
"""
import numpy as np

# electrons per (l channel) subshell, in filling order, neutral atoms H..Ar
_SUBSHELLS = [(0, 2), (0, 2), (1, 6), (0, 2), (1, 6)]  # 1s 2s 2p 3s 3p


def atomic_config(z):
    """{l: [electrons in each subshell of that l, lowest first]}."""
    left = int(z)
    if left > 18:
        raise NotImplementedError('SAD configurations are tabulated for H..Ar')
    out = {0: [], 1: []}
    for l, cap in _SUBSHELLS:
        if left <= 0:
            break
        n = min(cap, left)
        out[l].append(n)
        left -= n
    return out


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


def _ao_l(mol):
    bas = np.asarray(mol._bas)
    out = []
    for ib in range(len(bas)):
        l = int(bas[ib, 1])
        nf = (l + 1) * (l + 2) // 2 if mol.cart else 2 * l + 1
        out += [l] * (nf * int(bas[ib, 3]))
    return np.array(out)


def atom_density(symb, shells, cart=False, max_cycle=60, tol=1e-9):
    """Spherically averaged fractional-occupation atomic density (numpy).

    J/K and one-electron integrals come from the GPU engine; the tiny
    eigenproblems are solved on the host."""
    import scipy.linalg
    from ..gto.mole import M, charge_of
    from . import hf, jk
    amol = M(atom=[(symb, (0., 0., 0.))], basis={symb: shells}, unit='Bohr', cart=cart)
    cfg = atomic_config(charge_of(symb))
    opt = jk._VHFOpt(amol).build()
    S, T, V = hf.int1e_sorted(opt)
    C = opt.coeff
    S = (C.T @ S @ C).cpu().numpy()
    H = (C.T @ (T + V) @ C).cpu().numpy()
    aol = _ao_l(amol)

    def occupy(e, c):
        # l character of each MO by Mulliken weights
        w = c * (S @ c)
        lw = np.stack([w[aol == l].sum(0) for l in range(int(aol.max()) + 1)])
        lch = np.argmax(lw, axis=0)
        occ = np.zeros_like(e)
        for l, subs in cfg.items():
            idx = np.nonzero(lch == l)[0]
            idx = idx[np.argsort(e[idx])]
            k, deg = 0, 2 * l + 1
            for n in subs:
                occ[idx[k:k + deg]] = n / deg
                k += deg
        return occ

    e, c = scipy.linalg.eigh(H, S)
    dm = (c * occupy(e, c)) @ c.T
    e_last = 0.
    for it in range(max_cycle):
        vj, vk = jk.get_jk(amol, dm, hermi=1, vhfopt=opt)
        f = H + vj.cpu().numpy() - 0.5 * vk.cpu().numpy()
        etot = 0.5 * float(np.sum(dm * (H + f)))
        e, c = scipy.linalg.eigh(f, S)
        new = (c * occupy(e, c)) @ c.T
        delta = abs(new - dm).max()
        dm = 0.5 * (dm + new) if delta > 1e-3 else new
        if abs(etot - e_last) < tol and delta < 1e-7:
            break
        e_last = etot
    return dm


_ATOM_CACHE = {}


def sad_density(mol):
    """Block-diagonal superposition of atomic densities in mol's AO basis.
    Atomic densities are cached per (element, basis shells, cart)."""
    from ..gto.mole import std_symbol
    n = mol.nao
    dm = np.zeros((n, n))
    cache = _ATOM_CACHE
    slices = atom_ao_slices(mol)
    for ia in range(mol.natm):
        symb = std_symbol(mol.atom_symbol(ia))
        key = (symb, repr(mol._basis[symb]), bool(mol.cart))
        if key not in cache:
            cache[key] = atom_density(symb, mol._basis[symb], cart=bool(mol.cart))
        lo, hi = slices[ia]
        dm[lo:hi, lo:hi] = cache[key]
    return dm
