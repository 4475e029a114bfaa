"""Host-side logic without a GPU: basis sorting and transforms, the C ABI
library exports, input validation."""
import ctypes
import os
import re

import numpy as np
import pytest

from gpu4pyscf_gb300 import gto
from gpu4pyscf_gb300.gto.sorted_basis import SortedBasis
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize('l', range(6))
def test_cart2sph_matches_oracle_fit(l):
    assert np.allclose(gto.cart2sph_coeff(l), orc.c2s_fit(l), atol=1e-11)


@pytest.mark.parametrize('cart', [False, True])
def test_sorted_basis_transform(cart):
    """J/K through the sorted Cartesian basis equal the direct user-basis J/K."""
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696',
                basis='syn-cc-pvdz', cart=cart)
    sb = SortedBasis(mol)
    assert sb.nao_user == mol.nao
    ls = sb._bas[:, 1]
    assert np.all(np.diff(ls) >= 0)
    assert np.all(sb._bas[:, 3] == 1)
    rng = np.random.default_rng(0)
    dm = rng.random((mol.nao, mol.nao))
    dm = dm + dm.T
    C = sb.coeff
    dms = C @ dm @ C.T

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    vj_s, vk_s, _ = orc.get_jk_cart(Raw, dms, hermi=1)
    vj = C.T @ vj_s @ C
    vk = C.T @ vk_s @ C
    vj0, vk0 = orc.get_jk(mol, dm, hermi=1)
    assert abs(vj - vj0).max() < 1e-10
    assert abs(vk - vk0).max() < 1e-10


@pytest.mark.parametrize('cart', [False, True])
def test_diffuse_primitives_peeled(cart):
    """Primitives at or below the cutoff leave their contraction as shells of
    their own (gpu4pyscf/gto/mole.py:1157-1251): a 4-primitive s and a
    general p contraction with diffuse members split into compact and
    single-primitive shells, and J/K through the split basis equal the
    user-basis J/K."""
    extra = [[0, [10., .3], [1., .5], [.2, .4], [.05, .2]],
             [1, [3., .4, .1], [.8, .5, .3], [.25, .3, .8]]]
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696',
                basis=('syn-6-31g*', extra), cart=cart)
    sb0 = SortedBasis(mol, 0.)
    sb = SortedBasis(mol, 0.3)
    # one shell per contraction's compact part plus one per diffuse primitive
    expect = 0
    for bb in np.asarray(mol._bas):
        e = mol._env[bb[5]:bb[5] + bb[2]]
        for k in range(bb[3]):
            c = mol._env[bb[6] + k * bb[2]:bb[6] + (k + 1) * bb[2]]
            expect += int(np.any((e > .3) & (c != 0))) + int(np.sum((e <= .3) & (c != 0)))
    assert sb.nbas == expect > sb0.nbas + mol.natm * (2 + 2) - 1
    assert np.all(sb._bas[:, 3] == 1)
    exps = [sb._env[b[5]:b[5] + b[2]] for b in sb._bas]
    assert all(len(e) == 1 or np.all(e > 0.3) for e in exps)
    rng = np.random.default_rng(3)
    dm = rng.random((mol.nao, mol.nao)) - .5
    dm = dm + dm.T
    vj0, vk0 = orc.get_jk(mol, dm, hermi=1)
    C = sb.coeff

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    vj_s, vk_s, _ = orc.get_jk_cart(Raw, C @ dm @ C.T, hermi=1)
    assert abs(C.T @ vj_s @ C - vj0).max() < 1e-10
    assert abs(C.T @ vk_s @ C - vk0).max() < 1e-10


def _sparse_emul(side, rows, a, R, K, M):
    """The formulas of jk_sparse_mm in numpy (a: [n, ., .])."""
    ptr, idx, val = rows
    out = np.zeros((a.shape[0], R, M))
    for r in range(R):
        for m in range(M):
            if side == 0:
                p = slice(ptr[m], ptr[m + 1])
                out[:, r, m] = a[:, r, idx[p]] @ val[p]
            else:
                p = slice(ptr[r], ptr[r + 1])
                out[:, r, m] = np.einsum('p,np->n', val[p], a[:, idx[p], m])
    return out


@pytest.mark.parametrize('cart, cutoff', [(False, 0.), (True, 0.), (False, 0.3)])
def test_sparse_transform_rows(cart, cutoff):
    """The compressed rows of C and C^T with the sparse-product formulas of
    jk_sparse_mm give C D C^T and C^T V C."""
    extra = [[0, [10., .3], [1., .5], [.2, .4], [.05, .2]]]
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696',
                basis=('syn-def2-tzvp', extra), cart=cart)
    sb = SortedBasis(mol, cutoff)
    C = sb.coeff
    ns, nu = C.shape
    rng = np.random.default_rng(4)
    D = rng.random((2, nu, nu))
    V = rng.random((2, ns, ns))
    rc, rt = sb.coeff_rows(), sb.coeff_rows(transpose=True)
    assert rc[0][-1] == len(rc[2]) == np.count_nonzero(C) and rt[0][-1] == len(rt[2])
    t = _sparse_emul(0, rc, D, nu, nu, ns)
    ds = _sparse_emul(1, rc, t, ns, nu, ns)
    assert abs(ds - C @ D @ C.T).max() < 1e-12
    t = _sparse_emul(0, rt, V, ns, ns, nu)
    vu = _sparse_emul(1, rt, t, nu, ns, nu)
    assert abs(vu - C.T @ V @ C).max() < 1e-12


def test_basis_parsing_forms():
    m1 = gto.M(atom='C 0 0 0', basis=('sto-3g', [[3, [1.4, 1.]]]))
    assert list(m1._bas[:, 1]) == [0, 0, 1, 3]
    m2 = gto.M(atom='C 0 0 0; H 0 0 1', basis={'C': 'syn-def2-svp', 'default': 'sto-3g'})
    assert m2.nbas == 6 + 1
    with pytest.raises(KeyError):
        gto.M(atom='C 0 0 0', basis='def2-tzvp')


def test_library_exports_header_symbols():
    from gpu4pyscf_gb300.lib import libjk
    lib = libjk.load()
    hdr = open(os.path.join(ROOT, 'include', 'gb300jk.h')).read()
    names = re.findall(r'^[A-Za-z_][\w \*]*?\b(jk_\w+)\s*\(', hdr, re.M)
    assert set(libjk.EXPORTS) <= set(names)
    for n in names:
        assert hasattr(lib, n), n


def test_lmax_above_g_rejected():
    # l = 5 (h): the reference sends it to PySCF's CPU code; this engine has
    # no CPU path and refuses it
    from gpu4pyscf_gb300.scf import jk
    mol = gto.M(atom='C 0 0 0; H 0 0 1', basis=('sto-3g', [[5, [1., 1.]]]))
    with pytest.raises(NotImplementedError):
        jk._VHFOpt(mol).build()


def test_bad_arguments_rejected_without_gpu():
    from gpu4pyscf_gb300.lib import libjk
    lib = libjk.load()
    h = ctypes.c_void_p()
    assert lib.jk_opt_create(None, 0, None, 0, None, 0, 1e-13, 0, ctypes.byref(h)) == -1
    assert b'invalid' in lib.jk_last_error()
    assert lib.jk_build(None, None, 1, 1, 1, 1, 1, 0, 0., None, None, None, None) == -1
    assert lib.jk_energy_grad(None, None, 1, 1, 1., 1., 0., 1., 1., None, None, None) == -1
    assert lib.jk_opt_natm(None) == -1


def _header_arity(path):
    """{function name: number of parameters} of the prototypes in a header."""
    text = open(path).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    out = {}
    for m in re.finditer(r'^[A-Za-z_][\w \*]*?\b((?:jk|mlp)_\w+)\s*\(([^)]*)\)\s*;', text, re.M):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ('', 'void') else len(args.split(','))
    return out


def test_ctypes_signatures_match_headers():
    """The ctypes bindings (the reference-side stub a maintainer would add)
    declare exactly the parameters of the C prototypes."""
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import mlp
    lib = libjk.load()
    arity = _header_arity(os.path.join(ROOT, 'include', 'gb300jk.h'))
    arity.update(_header_arity(os.path.join(ROOT, 'include', 'gb300mlp.h')))
    mlp._lib()
    checked = 0
    for name, n in arity.items():
        f = getattr(lib, name)
        if f.argtypes is None:
            continue
        assert len(f.argtypes) == n, (name, len(f.argtypes), n)
        checked += 1
    assert checked >= 20
