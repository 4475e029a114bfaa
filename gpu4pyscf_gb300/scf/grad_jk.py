"""Nuclear gradient of the J/K energy.

Counterpart of gpu4pyscf's ``_jk_energy_per_atom`` (gpu4pyscf/grad/rhf.py:
60-171, kernel ``RYS_per_atom_jk_ip1`` in gpu4pyscf/lib/gvhf-rys/
rys_contract_jk_ip1.cu:1747-1797): the [natm, 3] gradient of

    E = j_factor/2 sum (ij|kl) D_ji D_lk - k_factor/4 sum (ij|kl) D_jk D_li

with respect to the nuclear positions, at fixed densities.

Two routes.  The product path (``method='ip1'``) is the engine's dedicated
derivative kernels (``jk_energy_grad`` of the C ABI, csrc/jk_grad.cu): per
screened shell quartet the derivative integrals on three centres,
contracted with the quartet's density weights into per-atom sums, with the
optimizer's pair lists and work units; shells up to f.  It takes one
(symmetric or antisymmetric) density, or two spin densities, as the
reference does.

The second route (``method='extended'``), kept as an independent check on
the GPU, uses the J/K kernels unchanged.  The derivative of a raw Cartesian
primitive c x^a exp(-alpha r^2) along x is a_x times the function lowered
by one in x minus the function raised by one with coefficient 2 alpha c.
So the derivative integrals are ordinary integrals over an extended basis
holding, for every shell of the sorted basis, the shell itself, a copy
with l + 1 and coefficients 2 alpha c, and (l > 0) a copy with l - 1.  One
J/K build of the extended basis, with the density on the original shells
only, gives for every derived function i'

    vj[i', j] = sum_kl (i'j|kl) D_lk,     vk[i', l] = sum_jk (i'j|kl) D_jk,

and with D symmetric the four centres of a quartet contribute alike:

    dE/dR_A = -4 sum_{i on A} [ j/2 sum_j (d_x i)vj[., j] D_ji
                                - k/4 sum_l (d_x i)vk[., l] D_li ].

Raised copies of f shells are g shells, the highest the J/K kernels take,
so both routes stop at f.
"""

import ctypes

import numpy as np
import torch

from ..gto.sorted_basis import SortedBasis
from ..lib import libjk

LMAX_GRAD = 3  # raised copies must stay within the kernels' g


def _comps(l):
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


def extended_basis(sb):
    """Extended sorted basis of SortedBasis ``sb`` (see the module notes).

    Returns a dict: ``atm``, ``bas``, ``env`` (libcint layout, shells sorted
    by l), ``nao`` (extended AOs), and per sorted AO: ``orig`` (its index in
    the extended basis), ``up`` [nao, 3] (the raised component along x, y,
    z), ``down`` [nao, 3] (the lowered one, -1 if none), ``ax`` [nao, 3]
    (the exponent a_x of that direction) and ``atom``."""
    bas = np.asarray(sb._bas)
    env = list(np.asarray(sb._env, dtype=np.float64))
    if len(bas) and int(bas[:, 1].max()) > LMAX_GRAD:
        raise NotImplementedError('J/K gradients need shells up to d (raised copies are one l higher)')
    # (l, kind, parent): kind 0 original, 1 raised, 2 lowered
    entries = []
    for s, row in enumerate(bas):
        l, nprim = int(row[1]), int(row[2])
        exps = np.asarray(env[row[5]:row[5] + nprim])
        coef = np.asarray(env[row[6]:row[6] + nprim])
        entries.append((l, 0, s, row[5], row[6]))
        pc = len(env)
        env.extend((coef * 2. * exps).tolist())
        entries.append((l + 1, 1, s, row[5], pc))
        if l > 0:
            entries.append((l - 1, 2, s, row[5], row[6]))
    order = sorted(range(len(entries)), key=lambda t: (entries[t][0], t))
    ext_bas = []
    first = {}          # (kind, parent) -> first extended AO
    off = 0
    for t in order:
        l, kind, s, pe, pc = entries[t]
        row = bas[s]
        ext_bas.append([row[0], l, row[2], 1, 0, pe, pc, 0])
        first[(kind, s)] = off
        off += (l + 1) * (l + 2) // 2
    nao_s = int(sb.nao)
    orig = np.zeros(nao_s, dtype=np.int64)
    up = np.zeros((nao_s, 3), dtype=np.int64)
    down = np.full((nao_s, 3), -1, dtype=np.int64)
    ax = np.zeros((nao_s, 3))
    atom = np.zeros(nao_s, dtype=np.int64)
    for s, row in enumerate(bas):
        l = int(row[1])
        cl, cu = _comps(l), _comps(l + 1)
        cd = _comps(l - 1) if l > 0 else []
        for a, (x, y, z) in enumerate(cl):
            i = int(sb.ao_loc[s]) + a
            orig[i] = first[(0, s)] + a
            atom[i] = int(row[0])
            for d, step in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
                up[i, d] = first[(1, s)] + cu.index((x + step[0], y + step[1], z + step[2]))
                n = (x, y, z)[d]
                ax[i, d] = n
                if n > 0:
                    down[i, d] = first[(2, s)] + cd.index((x - step[0], y - step[1], z - step[2]))
    return {'atm': np.ascontiguousarray(sb._atm, dtype=np.int32),
            'bas': np.ascontiguousarray(ext_bas, dtype=np.int32).reshape(-1, 8),
            'env': np.ascontiguousarray(env, dtype=np.float64), 'nao': off,
            'orig': orig, 'up': up, 'down': down, 'ax': ax, 'atom': atom}


def contract(ext, vj, vk, dm, natm, j_factor=1., k_factor=1.):
    """[natm, 3] gradient from the extended-basis J/K (numpy arrays or torch
    tensors, [nao_ext, nao_ext]) and the sorted-basis density dm."""
    is_t = isinstance(vj, torch.Tensor)
    idx = (lambda a: torch.as_tensor(a, device=vj.device)) if is_t else (lambda a: a)
    orig, up, down = idx(ext['orig']), idx(ext['up']), idx(ext['down'])
    ax = torch.as_tensor(ext['ax'], device=vj.device, dtype=vj.dtype) if is_t else ext['ax']
    down0 = down.clone() if is_t else down.copy()
    down0[down0 < 0] = 0              # rows of a_x = 0 contribute nothing

    def dterm(v):
        vo = v[:, orig]               # columns: original functions
        # (d_x i) v[., j] = a_x v[i - 1x, j] - v[i + 1x, j], for x = 0, 1, 2
        r = -vo[up] + ax[..., None] * vo[down0]      # [nao, 3, nao]
        # sum_j r[i, x, j] dm[j, i]
        return (r * dm.T[:, None, :]).sum(-1)          # [nao, 3]

    per_ao = -4. * (.5 * j_factor * dterm(vj) - .25 * k_factor * dterm(vk))
    if is_t:
        g = torch.zeros((natm, 3), dtype=vj.dtype, device=vj.device)
        g.index_add_(0, idx(ext['atom']), per_ao)
        return g
    g = np.zeros((natm, 3))
    np.add.at(g, ext['atom'], per_ao)
    return g


def jk_energy_grad(mol, dm, j_factor=1., k_factor=1., direct_scf_tol=1e-13, method='ip1', vhfopt=None,
                   stats=None):
    """[natm, 3] nuclear gradient (torch, cuda) of the J/K energy of the
    user-basis density dm (gpu4pyscf/grad/rhf.py:60-171), with the operator
    of mol.omega (libcint's sign convention).  dm: [nao, nao] (symmetric or
    antisymmetric) or [2, nao, nao] spin densities (ip1 only).  vhfopt: a
    built _VHFOpt of mol to reuse (ip1).  stats: a dict that receives the
    quartet counts of the build (ip1; synchronises)."""
    from .jk import _env_operator
    omega, lr, sr = _env_operator(getattr(mol, 'omega', 0.) or 0.)
    if method == 'ip1':
        return _grad_ip1(mol, dm, j_factor, k_factor, direct_scf_tol, (omega, lr, sr), vhfopt, stats)
    if method != 'extended':
        raise ValueError('method must be ip1 or extended')
    return _grad_extended(mol, dm, j_factor, k_factor, direct_scf_tol, (omega, lr, sr))


def _grad_ip1(mol, dm, j_factor, k_factor, direct_scf_tol, op, vhfopt=None, stats=None):
    from .jk import _VHFOpt
    opt = vhfopt if vhfopt is not None else _VHFOpt(mol, direct_scf_tol=direct_scf_tol).build()
    if opt._handle is None:
        opt.build()
    if opt.sorted_mol.lmax > LMAX_GRAD:
        raise NotImplementedError('J/K gradients are supported for shells up to f')
    d = torch.as_tensor(np.asarray(dm) if not isinstance(dm, torch.Tensor) else dm,
                        dtype=torch.float64, device='cuda')
    if d.ndim == 2:
        d = d[None]
    if d.ndim != 3 or d.shape[0] > 2:
        raise ValueError('dm must be [nao, nao] or [2, nao, nao]')
    ds = opt.apply_coeff_C_mat_CT(d).contiguous()
    lib = libjk.load()
    natm = lib.jk_opt_natm(opt._handle)
    ejk = torch.empty((natm, 3), dtype=torch.float64, device='cuda')
    omega, lr, sr = op
    st = libjk.JKStats() if stats is not None else None
    libjk.check(lib.jk_energy_grad(opt._handle, ds.data_ptr(), int(ds.shape[0]), int(ds.shape[-1]),
                                   float(j_factor), float(k_factor), float(omega), float(lr), float(sr),
                                   ejk.data_ptr(), torch.cuda.current_stream().cuda_stream,
                                   ctypes.byref(st) if st is not None else None), 'jk_energy_grad')
    if st is not None:
        d = st.as_dict()
        stats.update(quartets=d['quartets_fp64'], prim_quartets=d['prim_quartets_fp64'],
                     kernel_launches=d['kernel_launches'])
    return ejk


def _grad_extended(mol, dm, j_factor, k_factor, direct_scf_tol, op):
    omega, lr, sr = op
    sb = SortedBasis(mol)
    ext = extended_basis(sb)
    lib = libjk.load()
    h = ctypes.c_void_p()
    torch.cuda.current_device()
    libjk.check(lib.jk_opt_create(ext['atm'].ctypes.data, len(ext['atm']), ext['bas'].ctypes.data,
                                  len(ext['bas']), ext['env'].ctypes.data, len(ext['env']),
                                  float(direct_scf_tol), 0, ctypes.byref(h)), 'jk_opt_create')
    try:
        C = torch.as_tensor(sb.coeff, device='cuda')
        d = torch.as_tensor(np.asarray(dm) if not isinstance(dm, torch.Tensor) else dm,
                            dtype=torch.float64, device='cuda')
        ds = C @ d @ C.T
        n = ext['nao']
        orig = torch.as_tensor(ext['orig'], device='cuda')
        dext = torch.zeros((1, n, n), dtype=torch.float64, device='cuda')
        dext[0, orig[:, None], orig[None, :]] = ds
        vj = torch.empty_like(dext)
        vk = torch.empty_like(dext)
        stream = torch.cuda.current_stream().cuda_stream
        if omega == 0.:
            err = lib.jk_build(h, dext.data_ptr(), 1, n, 1, 1, 1, 0, 1e-6, vj.data_ptr(), vk.data_ptr(),
                               stream, None)
        else:
            err = lib.jk_build_rsh(h, dext.data_ptr(), 1, n, 1, 1, 1, omega, lr, sr, 0, 1e-6,
                                   vj.data_ptr(), vk.data_ptr(), stream, None)
        libjk.check(err, 'jk_build')
        return contract(ext, vj[0], vk[0], ds, mol.natm, j_factor, k_factor)
    finally:
        lib.jk_opt_destroy(h)


def _jk_energy_per_atom(vhfopt, dm, j_factor=1., k_factor=1., omega=None, lr_factor=None,
                        sr_factor=None, verbose=None):
    """The reference's entry (gpu4pyscf/grad/rhf.py:60): [natm, 3] numpy
    gradient of j_factor * E_J - k_factor * E_K for dm ([nao, nao] or two
    spin densities), with the optimizer's molecule, screening threshold and
    pair lists.  As in the reference, explicit range-separation factors are
    not accepted; mol.omega applies."""
    assert lr_factor is None and sr_factor is None
    mol = vhfopt.mol
    if omega is not None and omega != (getattr(mol, 'omega', 0.) or 0.):
        raise NotImplementedError('omega other than mol.omega')
    return jk_energy_grad(mol, dm, j_factor, k_factor, vhfopt.direct_scf_tol, vhfopt=vhfopt).cpu().numpy()
