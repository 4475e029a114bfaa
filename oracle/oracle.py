"""CPU oracle for J/K builds, one-electron integrals and RHF.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline leg; the product package never
imports it.

What it restates (all in the user's AO basis, PySCF conventions):
* get_jk(mol, dm, hermi, tol): vj = einsum('ijkl,ji->kl'), vk =
  einsum('ijkl,jk->il') over the full ERI tensor, as pyscf.scf.hf.get_jk,
  the oracle of gpu4pyscf/scf/tests/test_scf_jk.py:22,45 and
  gpu4pyscf/scf/tests/test_rhf.py:96-98.  hermi handling follows
  gpu4pyscf/scf/jk.py:594-605 (hermi=2 gives vj = 0).
* Cartesian -> spherical transformation: real solid harmonics normalised on
  the unit sphere, p in (x, y, z) order, m = -l..l otherwise, s/p Cartesian
  factors 1/sqrt(4pi), sqrt(3/(4pi)).  The coefficients here are obtained by
  a least-squares fit of scipy's spherical harmonics, independently of the
  closed-form table in the product.
* rhf(mol): a plain Roothaan-Hall SCF with DIIS in numpy, the restatement of
  gpu4pyscf/scf/hf.py:206-341 used to check the product's RHF energies.

Parity pin: tests/test_oracle_golden.py reproduces the golden fingerprints
of gpu4pyscf/scf/tests/test_rhf.py:168-194 (inline uncontracted basis up to h
shells, hermi=1 and hermi=0, two densities) with this oracle.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, 'liboracle_jk.so')
_lib = None
_lock = threading.Lock()


def build(force=False):
    """Compile the C++ oracle with g++ and OpenMP."""
    src = os.path.join(_HERE, 'jk_oracle.cpp')
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    cmd = ['g++', '-O3', '-std=c++17', '-fopenmp', '-shared', '-fPIC',
           src, '-o', _LIB_PATH]
    subprocess.check_call(cmd)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = ctypes.CDLL(_LIB_PATH)
            for name in ('oracle_eri_full', 'oracle_qcond', 'oracle_jk', 'oracle_int1e', 'oracle_jk_grad'):
                getattr(_lib, name).restype = ctypes.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _env_args(mol):
    atm = np.ascontiguousarray(mol._atm, dtype=np.int32)
    bas = np.ascontiguousarray(mol._bas, dtype=np.int32)
    env = np.ascontiguousarray(mol._env, dtype=np.float64)
    return atm, bas, env


def boys(m, t):
    out = np.zeros(m + 1)
    lib().oracle_boys(ctypes.c_int(m), ctypes.c_double(t), _p(out))
    return out


# -- Cartesian -> spherical by least squares ------------------------------
_C2S_CACHE = {}


def _cart_comps(l):
    return [(lx, ly, l - lx - ly) for lx in range(l, -1, -1) for ly in range(l - lx, -1, -1)]


def c2s_fit(l):
    """[ncart, nsph] coefficients fitted from scipy's spherical harmonics."""
    if l in _C2S_CACHE:
        return _C2S_CACHE[l]
    from scipy.special import sph_harm_y
    rng = np.random.default_rng(1234 + l)
    npts = 40 * (l + 1) ** 2
    v = rng.normal(size=(npts, 3))
    r = np.linalg.norm(v, axis=1)
    x, y, z = v.T
    theta = np.arccos(z / r)
    phi = np.arctan2(y, x)
    comps = _cart_comps(l)
    A = np.stack([x**a * y**b * z**c for a, b, c in comps], axis=1)
    if l == 1:
        ms = [1, -1, 0]  # PySCF keeps p in x, y, z order
    else:
        ms = list(range(-l, l + 1))
    cols = []
    for m in ms:
        ylm = sph_harm_y(l, abs(m), theta, phi)
        if m > 0:
            yr = np.sqrt(2) * (-1) ** m * ylm.real
        elif m < 0:
            yr = np.sqrt(2) * (-1) ** m * ylm.imag
        else:
            yr = ylm.real
        target = r**l * yr
        coef, *_ = np.linalg.lstsq(A, target, rcond=None)
        coef[abs(coef) < 1e-12] = 0.
        cols.append(coef)
    c = np.array(cols).T
    _C2S_CACHE[l] = c
    return c


def ao_c_matrix(mol):
    """[nao_cart, nao_user] map from raw Cartesian functions to user AOs."""
    bas = np.asarray(mol._bas)
    ls = bas[:, 1]
    nctr = bas[:, 3]
    ncart = (ls + 1) * (ls + 2) // 2
    nuser = ncart if mol.cart else 2 * ls + 1
    lc = np.append(0, np.cumsum(ncart * nctr))
    lu = np.append(0, np.cumsum(nuser * nctr))
    C = np.zeros((lc[-1], lu[-1]))
    for ib in range(len(bas)):
        l = int(ls[ib])
        if mol.cart:
            fac = {0: 1 / np.sqrt(4 * np.pi), 1: np.sqrt(3 / (4 * np.pi))}.get(l, 1.)
            blk = np.eye(ncart[ib]) * fac
        else:
            blk = c2s_fit(l)
        nc, nu = blk.shape
        for k in range(nctr[ib]):
            C[lc[ib] + k * nc: lc[ib] + (k + 1) * nc, lu[ib] + k * nu: lu[ib] + (k + 1) * nu] = blk
    return C


# -- integrals --------------------------------------------------------------
def eri_cart(mol):
    atm, bas, env = _env_args(mol)
    C = ao_c_matrix(mol)
    n = C.shape[0]
    eri = np.zeros((n, n, n, n))
    lib().oracle_eri_full(_p(atm), len(atm), _p(bas), len(bas), _p(env), _p(eri))
    return eri


def eri(mol):
    C = ao_c_matrix(mol)
    e = eri_cart(mol)
    return np.einsum('ijkl,ip,jq,kr,ls->pqrs', e, C, C, C, C, optimize=True)


def qcond(mol):
    atm, bas, env = _env_args(mol)
    q = np.zeros((len(bas), len(bas)))
    lib().oracle_qcond(_p(atm), len(atm), _p(bas), len(bas), _p(env), _p(q), 0)
    return q


def get_jk_cart(mol, dm_cart, hermi=1, tol=0., with_j=True, with_k=True,
                nthreads=0, bra_stride=1):
    """J/K in the raw Cartesian basis; returns (vj, vk, stats)."""
    atm, bas, env = _env_args(mol)
    dms = np.ascontiguousarray(np.asarray(dm_cart, dtype=np.float64))
    shape = dms.shape
    n = shape[-1]
    dms = dms.reshape(-1, n, n)
    vj = np.zeros_like(dms)
    vk = np.zeros_like(dms)
    stats = np.zeros(4, dtype=np.int64)
    err = lib().oracle_jk(_p(atm), len(atm), _p(bas), len(bas), _p(env), _p(dms),
                          len(dms), int(hermi), ctypes.c_double(tol), int(with_j),
                          int(with_k), _p(vj), _p(vk), int(nthreads),
                          ctypes.c_longlong(bra_stride), _p(stats))
    if err:
        raise RuntimeError('oracle_jk failed')
    return vj.reshape(shape), vk.reshape(shape), stats


def jk_energy_grad(mol, dm, j_factor=1., k_factor=1., nthreads=0):
    """[natm, 3] nuclear gradient of E = j/2 sum (ij|kl) D_ji D_lk
    - k/4 sum (ij|kl) D_jk D_li at fixed symmetric user-basis density D: what
    gpu4pyscf's _jk_energy_per_atom returns for an RHF density
    (gpu4pyscf/grad/rhf.py:60-171)."""
    atm, bas, env = _env_args(mol)
    C = ao_c_matrix(mol)
    dmc = np.ascontiguousarray(C @ np.asarray(dm, dtype=np.float64) @ C.T)
    g = np.zeros((mol.natm, 3))
    err = lib().oracle_jk_grad(_p(atm), len(atm), _p(bas), len(bas), _p(env), _p(dmc),
                               ctypes.c_double(j_factor), ctypes.c_double(k_factor), _p(g), int(nthreads))
    if err:
        raise RuntimeError('oracle_jk_grad failed')
    return g


def get_jk(mol, dm, hermi=1, tol=0., with_j=True, with_k=True, nthreads=0):
    """J/K in the user AO basis (spherical unless mol.cart)."""
    C = ao_c_matrix(mol)
    dm = np.asarray(dm, dtype=np.float64)
    shape = dm.shape
    dms = dm.reshape(-1, shape[-1], shape[-1])
    dmc = np.einsum('pi,nij,qj->npq', C, dms, C)
    vj, vk, _ = get_jk_cart(mol, dmc, hermi, tol, with_j, with_k, nthreads)
    vj = np.einsum('pi,npq,qj->nij', C, vj, C).reshape(shape)
    vk = np.einsum('pi,npq,qj->nij', C, vk, C).reshape(shape)
    return (vj if with_j else None), (vk if with_k else None)


def int1e(mol, kind):
    atm, bas, env = _env_args(mol)
    C = ao_c_matrix(mol)
    n = C.shape[0]
    out = np.zeros((n, n))
    k = {'ovlp': 0, 'kin': 1, 'nuc': 2}[kind]
    lib().oracle_int1e(_p(atm), len(atm), _p(bas), len(bas), _p(env), k, _p(out))
    return C.T @ out @ C


def fp(a):
    """PySCF's lib.fp fingerprint: dot(cos(arange(size)), ravel(a))."""
    a = np.asarray(a)
    return float(np.dot(np.cos(np.arange(a.size)), a.ravel()))


def energy_nuc(mol):
    z = np.asarray(mol._atm[:, 0], dtype=np.float64)
    r = np.stack([mol._env[p:p + 3] for p in mol._atm[:, 1]])
    e = 0.
    for i in range(len(z)):
        for j in range(i):
            e += z[i] * z[j] / np.linalg.norm(r[i] - r[j])
    return e


def rhf(mol, conv_tol=1e-10, max_cycle=100, dm0=None, tol=0.):
    """Reference closed-shell SCF with DIIS; returns (e_tot, dm, ncycle)."""
    import scipy.linalg
    S = int1e(mol, 'ovlp')
    H = int1e(mol, 'kin') + int1e(mol, 'nuc')
    nocc = mol.nelectron // 2
    enuc = energy_nuc(mol)

    def make_dm(F):
        e, c = scipy.linalg.eigh(F, S)
        return 2 * c[:, :nocc] @ c[:, :nocc].T

    dm = make_dm(H) if dm0 is None else dm0
    e_old = 0.
    fs, errs = [], []
    for cyc in range(max_cycle):
        vj, vk = get_jk(mol, dm, hermi=1, tol=tol)
        F = H + vj - 0.5 * vk
        e = 0.5 * np.einsum('ij,ji', dm, H + F) + enuc
        err = F @ dm @ S - S @ dm @ F
        fs.append(F)
        errs.append(err)
        fs, errs = fs[-8:], errs[-8:]
        nd = len(fs)
        B = -np.ones((nd + 1, nd + 1))
        B[nd, nd] = 0
        for i in range(nd):
            for j in range(nd):
                B[i, j] = np.vdot(errs[i], errs[j])
        rhs = np.zeros(nd + 1)
        rhs[nd] = -1
        c = np.linalg.solve(B, rhs)[:nd]
        Fd = sum(ci * fi for ci, fi in zip(c, fs))
        if abs(e - e_old) < conv_tol and np.linalg.norm(err) < np.sqrt(conv_tol):
            return e, dm, cyc + 1
        e_old = e
        dm = make_dm(Fd)
    return e, dm, max_cycle


def _ao_l(mol):
    bas = np.asarray(mol._bas)
    out = []
    for ib in range(len(bas)):
        l = int(bas[ib, 1])
        nf = (l + 1) * (l + 2) // 2 if mol.cart else 2 * l + 1
        out += [l] * (nf * int(bas[ib, 3]))
    return np.array(out)


_CFG = [(0, 2), (0, 2), (1, 6), (0, 2), (1, 6)]


def _config(z):
    left, out = int(z), {0: [], 1: []}
    for l, cap in _CFG:
        if left <= 0:
            break
        out[l].append(min(cap, left))
        left -= min(cap, left)
    return out


def atom_density(symb, shells, cart=False, max_cycle=80, tol=1e-10):
    """Spherically averaged fractional-occupation atomic RHF density (the
    superposition-of-atomic-densities guess of gpu4pyscf/scf/hf.py:414-561,
    restated in numpy on the oracle's integrals)."""
    import scipy.linalg
    from gpu4pyscf_gb300.gto.mole import M, charge_of
    amol = M(atom=[(symb, (0., 0., 0.))], basis={symb: shells}, unit='Bohr', cart=cart)
    cfg = _config(charge_of(symb))
    S = int1e(amol, 'ovlp')
    H = int1e(amol, 'kin') + int1e(amol, 'nuc')
    eri_ = eri(amol)
    aol = _ao_l(amol)

    def occupy(e, c):
        w = c * (S @ c)
        lw = np.stack([w[aol == l].sum(0) for l in range(aol.max() + 1)])
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
    for _ in range(max_cycle):
        f = H + np.einsum('ijkl,ji->kl', eri_, dm) - 0.5 * np.einsum('ijkl,jk->il', eri_, dm)
        etot = np.sum(dm * (H + f)) * .5
        e, c = scipy.linalg.eigh(f, S)
        new = (c * occupy(e, c)) @ c.T
        delta = abs(new - dm).max()
        dm = 0.5 * (dm + new) if delta > 1e-3 else new
        if abs(etot - e_last) < tol and delta < 1e-7:
            break
        e_last = etot
    return dm


def sad_density(mol):
    from gpu4pyscf_gb300.gto.mole import std_symbol
    bas = np.asarray(mol._bas)
    ls = bas[:, 1]
    nf = (ls + 1) * (ls + 2) // 2 if mol.cart else 2 * ls + 1
    loc = np.append(0, np.cumsum(nf * bas[:, 3]))
    n = loc[-1]
    dm = np.zeros((n, n))
    cache = {}
    for ia in range(mol.natm):
        sh = np.nonzero(bas[:, 0] == ia)[0]
        lo, hi = loc[sh.min()], loc[sh.max() + 1]
        symb = std_symbol(mol.atom_symbol(ia))
        if symb not in cache:
            cache[symb] = atom_density(symb, mol._basis[symb], cart=bool(mol.cart))
        dm[lo:hi, lo:hi] = cache[symb]
    return dm
