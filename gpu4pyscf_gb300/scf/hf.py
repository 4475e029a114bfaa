"""Restricted closed-shell Hartree-Fock on the GB300 J/K engine.

Counterpart of gpu4pyscf/scf/hf.py for the path the J/K engine serves:
``RHF.kernel`` follows ``SCF._kernel`` (hf.py:206-341) -- initial guess,
then per cycle an incremental Fock build from the density change
(``get_veff``, hf.py:91-109), CDIIS extrapolation on the orthogonalised
commutator error (scf/diis.py:41-90), diagonalisation in the canonically
orthogonalised basis (``eig``, hf.py:763-787) and the convergence test on the
energy change and orbital gradient (hf.py:213-215, 309-312).  Everything
stays on the GPU in FP64 torch tensors; one- and two-electron integrals come
from libgb300jk.so.

Module-level ``get_jk`` mirrors gpu4pyscf.scf.hf.get_jk (hf.py:49-57): numpy
in, numpy out.
"""

import ctypes
import math
import sys
import time

import numpy as np
import torch

from . import jk as jk_mod
from ..lib import libjk


def get_jk(mol, dm, hermi=1, vhfopt=None, with_j=True, with_k=True, omega=None, lr_factor=None,
           sr_factor=None, verbose=None):
    """J/K with the reference's module-level conventions: numpy input gives
    numpy output (gpu4pyscf/scf/hf.py:49-57)."""
    is_np = not isinstance(dm, torch.Tensor)
    vj, vk = jk_mod.get_jk(mol, dm, hermi, vhfopt, with_j, with_k, omega, lr_factor, sr_factor)
    if is_np:
        vj = vj.cpu().numpy() if vj is not None else None
        vk = vk.cpu().numpy() if vk is not None else None
    return vj, vk


def int1e_sorted(opt):
    """Overlap, kinetic and nuclear-attraction matrices in the sorted
    Cartesian basis of ``opt`` (torch, cuda)."""
    smol = opt.sorted_mol
    n = smol.nao
    S = torch.empty((n, n), dtype=torch.float64, device='cuda')
    T = torch.empty_like(S)
    V = torch.empty_like(S)
    atm = np.ascontiguousarray(smol._atm, dtype=np.int32)
    bas = np.ascontiguousarray(smol._bas, dtype=np.int32)
    env = np.ascontiguousarray(smol._env, dtype=np.float64)
    lib = libjk.load()
    err = lib.jk_int1e(atm.ctypes.data, len(atm), bas.ctypes.data, len(bas), env.ctypes.data, len(env),
                       S.data_ptr(), T.data_ptr(), V.data_ptr(), torch.cuda.current_stream().cuda_stream)
    if err:
        raise RuntimeError('jk_int1e failed (%d): %s' % (err, lib.jk_int1e_last_error().decode()))
    return S, T, V


def energy_nuc(mol):
    z = np.asarray(mol._atm[:, 0], dtype=np.float64)
    r = np.stack([np.asarray(mol._env[p:p + 3]) for p in mol._atm[:, 1]])
    e = 0.
    for i in range(len(z)):
        for j in range(i):
            e += z[i] * z[j] / np.linalg.norm(r[i] - r[j])
    return e


class CDIIS:
    """Commutator DIIS on the orthogonalised error F D S - S D F."""

    def __init__(self, space=8):
        self.space = space
        self.fs, self.es = [], []

    def update(self, f, err):
        self.fs.append(f)
        self.es.append(err)
        if len(self.fs) > self.space:
            self.fs.pop(0)
            self.es.pop(0)
        n = len(self.fs)
        B = np.zeros((n + 1, n + 1))
        E = torch.stack([e.reshape(-1) for e in self.es])
        B[:n, :n] = (E @ E.T).cpu().numpy()
        B[n, :n] = B[:n, n] = -1
        rhs = np.zeros(n + 1)
        rhs[n] = -1
        try:
            c = np.linalg.solve(B, rhs)[:n]
        except np.linalg.LinAlgError:
            c = np.linalg.lstsq(B, rhs, rcond=None)[0][:n]
        out = torch.zeros_like(f)
        for ci, fi in zip(c, self.fs):
            out += float(ci) * fi
        return out


class RHF:
    """Closed-shell Hartree-Fock (the RHF of gpu4pyscf/scf/hf.py)."""

    def __init__(self, mol):
        self.mol = mol
        self.conv_tol = 1e-9
        self.conv_tol_grad = None
        self.max_cycle = 50
        self.diis_space = 8
        self.diis_start_cycle = 1
        self.direct_scf = True
        self.direct_scf_tol = 1e-13
        self.init_guess = 'minao'
        self.precision = 'fp64'
        self.split_thresh = 1e-6
        self.level_shift = 0.        # Ha added to virtual orbital energies
        self.level_shift_cycles = None  # cycles the shift applies to (None: all)
        self.damp = 0.                # Fock mixing with the previous cycle's Fock
        self.damp_cycles = 0
        self.lindep = 1e-8
        self.verbose = 0
        self.converged = False
        self.e_tot = 0.
        self.cycles = 0
        self.mo_energy = self.mo_coeff = self.mo_occ = None
        self.scf_summary = {}
        self.guess_model = None   # learned_guess.GuessModel for init_guess='learned'
        self._opt = None
        self._int1e = None

    # -- integrals ---------------------------------------------------------
    @property
    def opt(self):
        if self._opt is None:
            self._opt = jk_mod._VHFOpt(self.mol, self.direct_scf_tol).build()
        self._opt.precision = self.precision
        self._opt.split_thresh = self.split_thresh
        return self._opt

    def _ints(self):
        if self._int1e is None:
            opt = self.opt
            S, T, V = int1e_sorted(opt)
            C = opt.coeff
            tr = lambda M: C.T @ M @ C
            self._int1e = (tr(S), tr(T) + tr(V))
        return self._int1e

    def get_ovlp(self, mol=None):
        return self._ints()[0]

    def get_hcore(self, mol=None):
        return self._ints()[1]

    def energy_nuc(self):
        return energy_nuc(self.mol)

    def get_jk(self, mol=None, dm=None, hermi=1, with_j=True, with_k=True, omega=None):
        return jk_mod.get_jk(self.mol, dm, hermi, self.opt, with_j, with_k, omega)

    def get_j(self, mol=None, dm=None, hermi=1, omega=None):
        return self.get_jk(mol, dm, hermi, True, False, omega)[0]

    def get_k(self, mol=None, dm=None, hermi=1, omega=None):
        return self.get_jk(mol, dm, hermi, False, True, omega)[1]

    def get_veff(self, mol=None, dm=None, dm_last=None, vhf_last=None, hermi=1):
        """J - K/2, built from the density change when direct_scf
        (gpu4pyscf/scf/hf.py:91-109)."""
        if self.direct_scf and dm_last is not None and vhf_last is not None:
            ddm = dm - dm_last
            vj, vk = self.get_jk(mol, ddm, hermi)
            return vhf_last + vj - 0.5 * vk
        vj, vk = self.get_jk(mol, dm, hermi)
        return vj - 0.5 * vk

    # -- linear algebra ----------------------------------------------------
    def _orth(self):
        S = self.get_ovlp()
        s, U = torch.linalg.eigh(S)
        keep = s > self.lindep
        return U[:, keep] / torch.sqrt(s[keep])

    @property
    def _X(self):
        if getattr(self, '_X_cache', None) is None:
            self._X_cache = self._orth()
        return self._X_cache

    def eig(self, fock, s=None):
        X = self._X
        e, c = torch.linalg.eigh(X.T @ fock @ X)
        return e, X @ c

    def get_occ(self, mo_energy=None, mo_coeff=None):
        nocc = self.mol.nelectron // 2
        occ = torch.zeros_like(mo_energy)
        idx = torch.argsort(mo_energy)
        occ[idx[:nocc]] = 2.
        return occ

    def make_rdm1(self, mo_coeff=None, mo_occ=None):
        mo_coeff = self.mo_coeff if mo_coeff is None else mo_coeff
        mo_occ = self.mo_occ if mo_occ is None else mo_occ
        c = mo_coeff[:, mo_occ > 0]
        return (c * mo_occ[mo_occ > 0]) @ c.T

    def energy_elec(self, dm, h1e, vhf):
        e1 = torch.sum(dm * h1e).item()
        e2 = 0.5 * torch.sum(dm * vhf).item()
        return e1 + e2, e2

    def project_density(self, dm):
        """Nearest idempotent RHF density with the molecule's electron count:
        the nocc natural orbitals of largest occupation of ``dm`` (eigenvectors
        of X^T S D S X), each doubly occupied.  Turns a predicted density,
        which is neither idempotent nor of exact trace, into one whose
        orbital gradient the DIIS error vector measures."""
        X = self._X
        s1e = self.get_ovlp()
        dm = torch.as_tensor(dm, device='cuda', dtype=torch.float64)
        p = X.T @ s1e @ dm @ s1e @ X
        w, u = torch.linalg.eigh(0.5 * (p + p.T))
        nocc = self.mol.nelectron // 2
        c = X @ u[:, -nocc:]
        return 2. * c @ c.T

    def get_init_guess(self, mol=None, key=None):
        from . import guess
        key = (key or self.init_guess).lower()
        if key in ('minao', 'atom', 'sad'):
            dm = guess.sad_density(self.mol)
            return torch.as_tensor(dm, device='cuda')
        if key == 'learned':
            if self.guess_model is None:
                raise ValueError("init_guess='learned' needs RHF.guess_model")
            return self.project_density(self.guess_model.predict_density(self.mol))
        if key in ('1e', 'hcore', 'core'):
            h = self.get_hcore()
            e, c = self.eig(h)
            occ = self.get_occ(e, c)
            return self.make_rdm1(c, occ)
        raise ValueError('unknown init_guess %s' % key)

    # -- driver ----------------------------------------------------------------
    def kernel(self, dm0=None):
        return self.scf(dm0)

    def scf(self, dm0=None):
        if self.mol.nelectron % 2:
            raise ValueError('RHF needs an even number of electrons')
        t0 = time.perf_counter()
        h1e = self.get_hcore()
        s1e = self.get_ovlp()
        X = self._X
        enuc = self.energy_nuc()
        if dm0 is None:
            dm = self.get_init_guess()
        else:
            dm = torch.as_tensor(dm0, device='cuda', dtype=torch.float64)
        tol_grad = self.conv_tol_grad or math.sqrt(self.conv_tol)
        vhf = self.get_veff(dm=dm)
        e_tot = self.energy_elec(dm, h1e, vhf)[0] + enuc
        diis = CDIIS(self.diis_space)
        self.converged = False
        dm_last = vhf_last = None
        nbuild = 1
        fock_prev = None
        for cycle in range(self.max_cycle):
            fock = h1e + vhf
            err = X.T @ (fock @ dm @ s1e - s1e @ dm @ fock) @ X
            # the reference's rule (gpu4pyscf/scf/hf.py:176-179, cycles
            # counted from 0): damping before the DIIS start, DIIS from
            # cycle diis_start_cycle on, so the Fock matrix of the initial
            # guess (not idempotent, its commutator no measure of the
            # error) never enters the DIIS subspace
            if cycle < self.damp_cycles and fock_prev is not None and self.damp > 0:
                fock = (1 - self.damp) * fock + self.damp * fock_prev
            elif cycle >= self.diis_start_cycle:
                fock = diis.update(fock, err)
            fock_prev = fock
            if self.level_shift > 0 and (self.level_shift_cycles is None or cycle < self.level_shift_cycles):
                # shift the virtual space: F + shift (S - S D S / 2)
                fock = fock + self.level_shift * (s1e - 0.5 * s1e @ dm @ s1e)
            mo_e, mo_c = self.eig(fock)
            mo_occ = self.get_occ(mo_e, mo_c)
            dm_last, vhf_last, e_last = dm, vhf, e_tot
            dm = self.make_rdm1(mo_c, mo_occ)
            vhf = self.get_veff(dm=dm, dm_last=dm_last, vhf_last=vhf_last)
            nbuild += 1
            e_tot = self.energy_elec(dm, h1e, vhf)[0] + enuc
            fock = h1e + vhf
            # orbital gradient: occupied-virtual block of the MO Fock matrix
            f_mo = mo_c.T @ fock @ mo_c
            occ = mo_occ > 0
            g = f_mo[~occ][:, occ]
            gnorm = float(torch.linalg.norm(g).item()) * 2.
            if self.verbose:
                print('cycle %d E=%.12f dE=%.3e |g|=%.3e  %.2f s' % (cycle + 1, e_tot, e_tot - e_last, gnorm,
                                                                   time.perf_counter() - t0),
                      file=sys.stderr, flush=True)
            if abs(e_tot - e_last) < self.conv_tol and gnorm < tol_grad:
                self.converged = True
                break
        self.cycles = cycle + 1
        self.e_tot = e_tot
        self.mo_energy, self.mo_coeff, self.mo_occ = mo_e, mo_c, mo_occ
        self.dm = dm
        self.scf_summary = {'cycles': self.cycles, 'jk_builds': nbuild, 'wall_s': time.perf_counter() - t0,
                            'converged': self.converged, 'e_tot': e_tot}
        return e_tot
