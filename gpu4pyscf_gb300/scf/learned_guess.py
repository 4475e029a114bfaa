"""Learned initial density from geometry (atom-pair network).

For every atom pair (A <= B) a dense network (3 hidden layers of width 256,
SiLU, FP32; ``scf/mlp.py`` on the kernels of include/gb300mlp.h) maps
pair features to the correction of the density block D[A, B] over the
superposition-of-atoms (SAD) density, in the user AO basis, padded to the
largest atomic block of the basis; the guess is SAD plus the predicted
correction, so an untrained network falls back to SAD.  Features, all in the molecular
frame: element one-hots of A and B, distance and its decays, the
displacement and its direction, an element-resolved radial environment of
each atom (Gaussians at 6 radii per element) and a same-atom flag.  The
predicted blocks are assembled (D[B, A] = D[A, B]^T, diagonal blocks
symmetrised) and projected onto the nearest idempotent density with the
right electron count (``RHF.project_density``: its nocc strongest natural
orbitals, doubly occupied), which starts the SCF.  Without the projection
the DIIS error vector of the first Fock matrix, a commutator with a
non-idempotent density, under-reports how far that Fock matrix is from
self-consistency, and DIIS leans on it.

Training data are converged FP64 densities produced by this engine's own
RHF on seeded conformers (random displacements of seeded base molecules).
``superposition-of-atoms`` (SAD) stays the default guess; ``RHF.init_guess =
'learned'`` with ``RHF.guess_model`` set uses the network.
"""

import json
import time

import numpy as np
import torch

from ..gto import M
from ..gto.mole import std_symbol
from . import guess, hf, mlp

ELEMS = ['H', 'C', 'N', 'O']
ENV_MU = np.array([1.0, 1.8, 2.6, 3.6, 4.8, 6.5])
ENV_W = 0.6
NFEAT = 8 + 3 + 3 + 3 + 2 * 4 * len(ENV_MU) + 1


def _atoms(mol):
    coords = mol.atom_coords()
    symbs = [std_symbol(mol.atom_symbol(i)) for i in range(mol.natm)]
    return symbs, coords


def pair_features(mol):
    """(features [npair, NFEAT] float64, pairs [(A, B)])."""
    symbs, R = _atoms(mol)
    n = len(symbs)
    onehot = np.zeros((n, 4))
    for i, s in enumerate(symbs):
        onehot[i, ELEMS.index(s)] = 1.
    dist = np.linalg.norm(R[:, None] - R[None], axis=-1)
    env = np.zeros((n, 4, len(ENV_MU)))
    for a in range(n):
        for c in range(n):
            if a == c:
                continue
            env[a, ELEMS.index(symbs[c])] += np.exp(-(dist[a, c] - ENV_MU) ** 2 / (2 * ENV_W ** 2))
    env = env.reshape(n, -1)
    pairs, feats = [], []
    for a in range(n):
        for b in range(a, n):
            d = R[b] - R[a]
            r = dist[a, b]
            u = d / r if r > 0 else np.zeros(3)
            f = np.concatenate([onehot[a], onehot[b], [r, 1. / (1. + r), np.exp(-0.5 * r)], d, u,
                                env[a], env[b], [1. if a == b else 0.]])
            pairs.append((a, b))
            feats.append(f)
    return np.array(feats), pairs


def block_slices(mol):
    return guess.atom_ao_slices(mol)


class GuessModel:
    """Feature scaling + network + block layout."""

    def __init__(self, nblock, hidden=256, seed=0):
        self.nblock = nblock
        self.net = mlp.DenseMLP([NFEAT, hidden, hidden, hidden, nblock * nblock], seed=seed)
        # zero output layer: the untrained model predicts no correction (SAD)
        self.net.W[-1].zero_()
        self.net.b[-1].zero_()
        self.mu = np.zeros(NFEAT)
        self.sd = np.ones(NFEAT)

    def save(self, path):
        st = self.net.state()
        np.savez(path, nblock=self.nblock, sizes=np.asarray(st['sizes']), mu=self.mu, sd=self.sd,
                 **{'W%d' % i: w for i, w in enumerate(st['W'])}, **{'b%d' % i: b for i, b in enumerate(st['b'])})

    @classmethod
    def load(cls, path):
        z = np.load(path)
        sizes = [int(x) for x in z['sizes']]
        m = cls(int(z['nblock']), hidden=sizes[1])
        m.net.load({'W': [z['W%d' % i] for i in range(len(sizes) - 1)],
                    'b': [z['b%d' % i] for i in range(len(sizes) - 1)]})
        m.mu, m.sd = z['mu'], z['sd']
        return m

    def _x(self, feats):
        return torch.as_tensor(((feats - self.mu) / self.sd).astype(np.float32), device='cuda')

    def predict_blocks(self, feats):
        return self.net.forward(self._x(feats), keep=False).cpu().numpy().astype(np.float64)

    def predict_density(self, mol):
        feats, pairs = pair_features(mol)
        blocks = self.predict_blocks(feats).reshape(-1, self.nblock, self.nblock)
        sl = block_slices(mol)
        dm = np.zeros((mol.nao, mol.nao))
        base = guess.sad_density(mol)
        for (a, b), blk in zip(pairs, blocks):
            (a0, a1), (b0, b1) = sl[a], sl[b]
            x = blk[:a1 - a0, :b1 - b0]
            if a == b:
                x = 0.5 * (x + x.T)
                dm[a0:a1, a0:a1] = x
            else:
                dm[a0:a1, b0:b1] = x
                dm[b0:b1, a0:a1] = x.T
        return base + dm


def targets(mol, dm, nblock):
    """Padded density blocks [npair, nblock^2] and their masks."""
    _, pairs = pair_features(mol)
    sl = block_slices(mol)
    T = np.zeros((len(pairs), nblock, nblock))
    Mk = np.zeros_like(T)
    for k, (a, b) in enumerate(pairs):
        (a0, a1), (b0, b1) = sl[a], sl[b]
        T[k, :a1 - a0, :b1 - b0] = dm[a0:a1, b0:b1]
        Mk[k, :a1 - a0, :b1 - b0] = 1.
    return T.reshape(len(pairs), -1), Mk.reshape(len(pairs), -1)


# -- data -------------------------------------------------------------------
def base_formula(rng):
    nh = int(rng.integers(8, 21))
    frac = np.array([10, 3, 5], dtype=float) / 18.
    counts = np.floor(frac * nh).astype(int)
    while counts.sum() < nh:
        counts[rng.choice(3, p=frac)] += 1
    n_h = int(round(0.7 * nh))
    f = {'C': int(counts[0]), 'N': int(counts[1]), 'O': int(counts[2]), 'H': n_h}
    if (6 * f['C'] + 7 * f['N'] + 8 * f['O'] + f['H']) % 2:
        f['H'] += 1
    return f


def make_conformers(nbase, nconf, basis, seed=0, sigma=0.05, saturate=True):
    """Seeded base molecules (8-20 heavy atoms; hydrogens on every free
    valence unless saturate=False, which keeps the formula's H count and
    gives open-valence, small-gap molecules with several SCF solutions) and
    nconf conformers each (Gaussian displacements of sigma Angstrom);
    returns [[mol, ...], ...]."""
    from ..gto import molgen
    rng = np.random.default_rng(seed)
    out = []
    for b in range(nbase):
        f = base_formula(rng)
        atoms = None
        s = 7919 * (b + 1) + seed
        for _ in range(50):
            try:
                atoms = molgen.random_molecule(f, s, saturate=saturate)
                break
            except RuntimeError:
                s += 1000003
        confs = []
        for c in range(nconf):
            disp = rng.normal(scale=sigma, size=(len(atoms), 3))
            at = [(sym, xyz + d) for (sym, xyz), d in zip(atoms, disp)]
            confs.append(M(atom=molgen.atom_string(at), basis=basis))
        out.append(confs)
    return out


def converged_density(mol, dm0=None, conv_tol=1e-9, precision='fp64'):
    mf = hf.RHF(mol)
    mf.conv_tol = conv_tol
    mf.precision = precision
    mf.kernel(dm0=dm0)
    return mf


def generate(confsets, holdout, conv_tol=1e-8, log=None):
    """Converged densities of every conformer except the last ``holdout`` of
    each base molecule (those are kept for evaluation).  Each conformer
    starts from the converged density of the one before it."""
    data = []
    cycles = []
    t0 = time.perf_counter()
    for b, confs in enumerate(confsets):
        prev = None
        for c, mol in enumerate(confs[:len(confs) - holdout]):
            mf = converged_density(mol, dm0=prev, conv_tol=conv_tol)
            prev = mf.dm.cpu().numpy()
            data.append((mol, prev))
            if c:
                cycles.append(mf.cycles)
        if log:
            log('base %d: %d conformers, %.1f s' % (b, len(confs) - holdout, time.perf_counter() - t0))
    generate.chained_cycles = float(np.mean(cycles)) if cycles else None
    return data


def generate_batched(confsets, holdout, conv_tol=1e-8, chunk=64, log=None):
    """As ``generate``, with the SCFs of up to ``chunk`` conformers of one
    base molecule run together by ``BatchRHF`` (one batched J/K build per
    cycle), each from the SAD guess."""
    from .hf_batch import BatchRHF
    data = []
    cycles = []
    t0 = time.perf_counter()
    for b, confs in enumerate(confsets):
        train = confs[:len(confs) - holdout]
        for i in range(0, len(train), chunk):
            part = train[i:i + chunk]
            mf = BatchRHF(part, conv_tol=conv_tol)
            mf.kernel()
            if not all(mf.converged):
                raise RuntimeError('an SCF of the training set did not converge')
            for mol, dm in zip(part, mf.dms):
                data.append((mol, dm.cpu().numpy()))
            cycles.extend(mf.cycles)
        if log:
            log('base %d: %d conformers, %.1f s' % (b, len(train), time.perf_counter() - t0))
    generate_batched.mean_cycles = float(np.mean(cycles)) if cycles else None
    return data


def build_arrays(data, nblock):
    Xs, Ts, Ms = [], [], []
    for mol, dm in data:
        f, _ = pair_features(mol)
        t, m = targets(mol, dm - guess.sad_density(mol), nblock)
        Xs.append(f)
        Ts.append(t)
        Ms.append(m)
    return np.concatenate(Xs), np.concatenate(Ts), np.concatenate(Ms)


def train(data, nblock, epochs=40, batch=4096, lr=1e-3, seed=0, log=None):
    X, T, Mk = build_arrays(data, nblock)
    model = GuessModel(nblock, seed=seed)
    model.mu = X.mean(0)
    model.sd = X.std(0) + 1e-6
    Xd = model._x(X)
    Td = torch.as_tensor(T.astype(np.float32), device='cuda')
    Md = torch.as_tensor(Mk.astype(np.float32), device='cuda')
    n = len(X)
    g = torch.Generator(device='cpu').manual_seed(seed)
    hist = []
    steps = epochs * ((n + batch - 1) // batch)
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).cuda()
        tot = 0.
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            rate = lr * 0.5 * (1 + np.cos(np.pi * step / steps))
            y = model.net.forward(Xd[idx])
            loss, grad = mlp.mse(y, Td[idx], Md[idx])
            model.net.backward(grad)
            model.net.adam_step(lr=float(rate))
            tot += loss.item() * len(idx)
            step += 1
        hist.append(tot / n)
        if log and (ep % 10 == 0 or ep == epochs - 1):
            log('epoch %d loss %.3e' % (ep, tot / n))
    model.loss_history = hist
    return model


def evaluate(model, mols, conv_tol=1e-8, n_raw=None):
    """SCF cycles to conv_tol and converged energy from the SAD guess and
    from the learned guess (projected to the nearest idempotent density),
    per held-out molecule; on the first ``n_raw`` molecules also from the
    unprojected learned density.  rms_* are the RMS element errors of the
    guesses against the density converged from SAD."""
    rows = []
    for k, mol in enumerate(mols):
        a = hf.RHF(mol)
        a.conv_tol = conv_tol
        e_sad = a.kernel()
        d_conv = a.dm
        raw = model.predict_density(mol)
        b = hf.RHF(mol)
        b.conv_tol = conv_tol
        proj = b.project_density(raw)
        e_ml = b.kernel(dm0=proj)
        sad = torch.as_tensor(guess.sad_density(mol), device='cuda')
        rms = lambda d: float(torch.sqrt(torch.mean((torch.as_tensor(d, device='cuda') - d_conv) ** 2)).item())
        row = {'natm': mol.natm, 'nao': mol.nao, 'cycles_sad': a.cycles, 'cycles_learned': b.cycles,
               'e_sad': e_sad, 'e_learned': e_ml, 'converged': bool(a.converged and b.converged),
               'rms_sad': rms(sad), 'rms_learned_raw': rms(raw), 'rms_learned': rms(proj)}
        if n_raw is None or k < n_raw:
            c = hf.RHF(mol)
            c.conv_tol = conv_tol
            row['e_learned_raw'] = c.kernel(dm0=raw)
            row['cycles_learned_raw'] = c.cycles
        rows.append(row)
    cs = np.array([r['cycles_sad'] for r in rows])
    cl = np.array([r['cycles_learned'] for r in rows])
    de = np.array([r['e_learned'] - r['e_sad'] for r in rows])
    res = {'n': len(rows), 'mean_cycles_sad': float(cs.mean()), 'mean_cycles_learned': float(cl.mean()),
           'cycle_reduction': float(1 - cl.mean() / cs.mean()), 'max_abs_dE': float(np.abs(de).max()),
           'n_dE_above_1e-7': int((np.abs(de) > 1e-7).sum()), 'min_dE': float(de.min()),
           'all_converged': all(r['converged'] for r in rows),
           'mean_rms_sad': float(np.mean([r['rms_sad'] for r in rows])),
           'mean_rms_learned_raw': float(np.mean([r['rms_learned_raw'] for r in rows])),
           'mean_rms_learned': float(np.mean([r['rms_learned'] for r in rows])), 'rows': rows}
    raw_rows = [r for r in rows if 'cycles_learned_raw' in r]
    if raw_rows:
        res['raw'] = {'n': len(raw_rows),
                      'mean_cycles_sad': float(np.mean([r['cycles_sad'] for r in raw_rows])),
                      'mean_cycles_learned_raw': float(np.mean([r['cycles_learned_raw'] for r in raw_rows])),
                      'max_abs_dE': float(max(abs(r['e_learned_raw'] - r['e_sad']) for r in raw_rows))}
    return res


def evaluate_batched(model, mols, conv_tol=1e-8, chunk=64):
    """``evaluate`` with the SCFs batched (``BatchRHF``): per held-out
    molecule the cycles to conv_tol and the converged energy from SAD and
    from the learned guess (projected to the nearest idempotent density),
    and the RMS element errors of both guesses against the density converged
    from SAD."""
    from .hf_batch import BatchRHF
    rows = []
    for i in range(0, len(mols), chunk):
        part = mols[i:i + chunk]
        a = BatchRHF(part, conv_tol=conv_tol)
        e_sad = a.kernel()
        raws = [model.predict_density(m) for m in part]
        guesses = [a.single[k].project_density(r) for k, r in enumerate(raws)]
        b = BatchRHF(part, conv_tol=conv_tol)
        e_ml = b.kernel(dm0s=guesses)
        c = BatchRHF(part, conv_tol=conv_tol)
        e_raw = c.kernel(dm0s=raws)
        for k, mol in enumerate(part):
            d_conv = a.dms[k]
            sad = torch.as_tensor(guess.sad_density(mol), device='cuda')
            rms = lambda d: float(torch.sqrt(torch.mean((torch.as_tensor(d, device='cuda') - d_conv) ** 2)).item())
            rows.append({'natm': mol.natm, 'nao': mol.nao, 'cycles_sad': a.cycles[k],
                         'cycles_learned': b.cycles[k], 'cycles_learned_raw': c.cycles[k],
                         'e_sad': e_sad[k], 'e_learned': e_ml[k], 'e_learned_raw': e_raw[k],
                         'converged': bool(a.converged[k] and b.converged[k] and c.converged[k]),
                         'conv_sad': bool(a.converged[k]), 'conv_learned': bool(b.converged[k]),
                         'conv_raw': bool(c.converged[k]),
                         'rms_sad': rms(sad), 'rms_learned': rms(guesses[k]), 'rms_learned_raw': rms(raws[k])})
    cs = np.array([r['cycles_sad'] for r in rows])
    cl = np.array([r['cycles_learned'] for r in rows])
    cr = np.array([r['cycles_learned_raw'] for r in rows])
    de = np.array([r['e_learned'] - r['e_sad'] for r in rows])
    der = np.array([r['e_learned_raw'] - r['e_sad'] for r in rows])
    return {'n': len(rows), 'mean_cycles_sad': float(cs.mean()), 'mean_cycles_learned': float(cl.mean()),
            'mean_cycles_learned_raw': float(cr.mean()),
            'cycle_reduction': float(1 - cl.mean() / cs.mean()),
            'cycle_reduction_raw': float(1 - cr.mean() / cs.mean()),
            'max_abs_dE': float(np.abs(de).max()), 'max_abs_dE_raw': float(np.abs(der).max()),
            'n_dE_above_1e-7': int((np.abs(de) > 1e-7).sum()),
            'all_converged': all(r['converged'] for r in rows),
            'converged_sad': int(sum(r['conv_sad'] for r in rows)),
            'converged_learned': int(sum(r['conv_learned'] for r in rows)),
            'converged_learned_raw': int(sum(r['conv_raw'] for r in rows)),
            'mean_rms_sad': float(np.mean([r['rms_sad'] for r in rows])),
            'mean_rms_learned': float(np.mean([r['rms_learned'] for r in rows])),
            'mean_rms_learned_raw': float(np.mean([r['rms_learned_raw'] for r in rows])), 'rows': rows}


def run(nbase=10, nconf=60, holdout=10, basis='syn-def2-svp', epochs=300, seed=0, out=None, lr=2e-3, n_raw=20,
        batched=False):
    log = lambda m: print(m, flush=True)
    t0 = time.perf_counter()
    confsets = make_conformers(nbase, nconf, basis, seed)
    nblock = max(b - a for cs in confsets for (a, b) in block_slices(cs[0]))
    data = generate_batched(confsets, holdout, log=log) if batched else generate(confsets, holdout, log=log)
    t_gen = time.perf_counter() - t0
    t1 = time.perf_counter()
    model = train(data, nblock, epochs=epochs, lr=lr, seed=seed, log=log)
    t_train = time.perf_counter() - t1
    held = [m for cs in confsets for m in cs[len(cs) - holdout:]]
    t2 = time.perf_counter()
    # interleave the bases so that a prefix (n_raw) covers all of them
    held = [held[(i % nbase) * holdout + i // nbase] for i in range(len(held))]
    res = evaluate_batched(model, held) if batched else evaluate(model, held, n_raw=n_raw)
    res.update({'workload': '%d base molecules (8-20 heavy atoms, C/N/O/H, H-saturated) x %d conformers '
                            '(sigma 0.05 A), %s; %d held out' % (nbase, nconf, basis, len(held)),
                'train_conformers': len(data), 'train_pairs': int(sum(m.natm * (m.natm + 1) // 2 for m, _ in data)),
                'final_train_loss': model.loss_history[-1], 'first_train_loss': model.loss_history[0],
                'training_scf_cycles': (generate_batched.mean_cycles if batched else generate.chained_cycles),
                'epochs': epochs, 'lr': lr, 'batched_scf': batched,
                'generate_s': t_gen, 'train_s': t_train, 'evaluate_s': time.perf_counter() - t2})
    if out:
        slim = dict(res)
        slim['rows'] = res['rows'][:20]
        with open(out, 'w') as f:
            json.dump(slim, f, indent=1)
    return res, model


if __name__ == '__main__':
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument('--bases', type=int, default=10)
    ap.add_argument('--conformers', type=int, default=60)
    ap.add_argument('--holdout', type=int, default=10)
    ap.add_argument('--epochs', type=int, default=300)
    ap.add_argument('--lr', type=float, default=2e-3)
    ap.add_argument('--n-raw', type=int, default=20)
    ap.add_argument('--basis', default='syn-def2-svp')
    ap.add_argument('--out', default=None)
    ap.add_argument('--batched', action='store_true', help='run the SCFs batched (BatchRHF)')
    a = ap.parse_args()
    res, _ = run(a.bases, a.conformers, a.holdout, a.basis, a.epochs, out=a.out, lr=a.lr, n_raw=a.n_raw,
                 batched=a.batched)
    print(json.dumps({k: v for k, v in res.items() if k != 'rows'}))
