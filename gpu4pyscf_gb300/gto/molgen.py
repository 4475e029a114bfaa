"""Seeded synthetic C/N/O/H molecules.

Heavy atoms are placed by a self-avoiding random walk: each new heavy atom
bonds to the previous one (or, when the walk is stuck, to another heavy atom
with free valence) at a distance drawn from U(1.0, 1.5) Angstrom in a random
direction, and is accepted only if it stays at least 2.0 Angstrom from every
atom it is not bonded to.  Hydrogens then cap free valences (C 4, N 3, O 2)
with the same bond-length law and the same clearance: as many as the
formula asks for, or (saturate=True, ``_saturate``) one per free valence at
X-H distances, which gives a closed-shell molecule (C, N and O all have
Z + valence even, so the electron count of a saturated tree is even).
"""

import numpy as np

VALENCE = {'C': 4, 'N': 3, 'O': 2, 'H': 1}


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def _ok(pos, coords, skip, dmin):
    for k, c in enumerate(coords):
        if k == skip:
            continue
        if np.linalg.norm(pos - c) < dmin:
            return False
    return True


def _saturate(symbols, coords, free, rng, ndir=4096, bond=(1.0, 1.1), d_heavy=1.8, d_h=1.6, d_13=1.45):
    """One hydrogen per free valence, heavy atoms with the most free
    valences first.  The hydrogens of one heavy atom are placed together:
    among ndir random sets of directions (X-H bond lengths from U(1.0, 1.1)
    A) the set farthest from every other atom and from each other is kept;
    it needs 1.8 A to other heavy atoms and 1.6 A to other hydrogens
    (geminal H-H in CH4 is 1.78 A), except 1.45 A to any atom within 1.6 A
    of its own heavy atom (the heavy atoms bonded to it and their
    hydrogens)."""
    symbols, coords = list(symbols), [np.asarray(c) for c in coords]
    nheavy = len(symbols)
    for parent in sorted(range(nheavy), key=lambda k: -free[k]):
        m = max(free[parent], 0)
        if m == 0:
            continue
        dirs = rng.normal(size=(ndir, m, 3))
        dirs /= np.linalg.norm(dirs, axis=-1)[..., None]
        pos = coords[parent] + dirs * rng.uniform(*bond, size=(ndir, m, 1))
        idx = [k for k in range(len(coords)) if k != parent]
        others = np.array([coords[k] for k in idx])
        # atoms within 1.6 A of the parent (its bonded heavy atoms and their
        # hydrogens) are 1-3 neighbours of its hydrogens: with heavy-atom
        # bonds as short as 1.0 A they need a smaller clearance
        near = np.linalg.norm(others - coords[parent], axis=-1) < 1.6
        lim = np.where(near, d_13, np.array([d_h if symbols[k] == 'H' else d_heavy for k in idx]))
        margin = (np.linalg.norm(pos[:, :, None, :] - others[None, None], axis=-1) - lim).min(axis=(1, 2))
        for i in range(m):
            for j in range(i):
                margin = np.minimum(margin, np.linalg.norm(pos[:, i] - pos[:, j], axis=-1) - d_h)
        best = int(np.argmax(margin))
        if margin[best] < 0:
            raise RuntimeError('could not place hydrogen; try another seed')
        for i in range(m):
            symbols.append('H')
            coords.append(pos[best, i])
    return [(s, c) for s, c in zip(symbols, coords)]


def random_molecule(formula, seed, bond=(1.0, 1.5), dmin=2.0, max_tries=400, saturate=False):
    """Return a list of (symbol, xyz in Angstrom) for formula {'C': 10, ...}
    (with saturate=True the formula's H count is ignored)."""
    rng = np.random.default_rng(seed)
    heavy = []
    for el in ('C', 'N', 'O'):
        heavy += [el] * int(formula.get(el, 0))
    rng.shuffle(heavy)
    n_h = int(formula.get('H', 0))
    symbols, coords, free = [], [], []
    for k, el in enumerate(heavy):
        if k == 0:
            symbols.append(el)
            coords.append(np.zeros(3))
            free.append(VALENCE[el])
            continue
        placed = False
        parents = [k - 1] + [p for p in rng.permutation(k) if p != k - 1]
        for parent in parents:
            if free[parent] <= 0:
                continue
            for _ in range(max_tries):
                pos = coords[parent] + _unit(rng) * rng.uniform(*bond)
                if _ok(pos, coords, parent, dmin):
                    symbols.append(el)
                    coords.append(pos)
                    free.append(VALENCE[el] - 1)
                    free[parent] -= 1
                    placed = True
                    break
            if placed:
                break
        if not placed:
            raise RuntimeError('random walk got stuck; try another seed')
    if saturate:
        return _saturate(symbols, coords, free, rng)
    for _ in range(n_h):
        cands = [k for k in range(len(heavy)) if free[k] > 0]
        if not cands:
            cands = list(range(len(heavy)))
        placed = False
        for parent in rng.permutation(cands):
            for _t in range(max_tries):
                pos = coords[parent] + _unit(rng) * rng.uniform(*bond)
                if _ok(pos, coords, parent, dmin):
                    symbols.append('H')
                    coords.append(pos)
                    free.append(0)
                    free[parent] -= 1
                    placed = True
                    break
            if placed:
                break
        if not placed:
            raise RuntimeError('could not place hydrogen; try another seed')
    return [(s, c) for s, c in zip(symbols, coords)]


def formula_for(natm, rng):
    """C/N/O/H composition with the proportions of C10 N3 O5 H12."""
    nheavy = max(1, int(round(natm * 0.6)))
    nh = natm - nheavy
    frac = np.array([10, 3, 5], dtype=float) / 18.
    counts = np.floor(frac * nheavy).astype(int)
    while counts.sum() < nheavy:
        counts[rng.choice(3, p=frac)] += 1
    return {'C': int(counts[0]), 'N': int(counts[1]), 'O': int(counts[2]), 'H': int(nh)}


def atom_string(atoms):
    return '; '.join('%s %.10f %.10f %.10f' % (s, *c) for s, c in atoms)


def make_mol(formula, seed, basis, **kw):
    from .mole import M
    seed_try = seed
    for attempt in range(50):
        try:
            atoms = random_molecule(formula, seed_try)
            break
        except RuntimeError:
            seed_try = seed_try + 1000003
    else:
        raise RuntimeError('no geometry found')
    return M(atom=atom_string(atoms), basis=basis, **kw)
