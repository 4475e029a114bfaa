"""Closed-shell Hartree-Fock for many molecules in lockstep.

The reference runs one SCF per molecule (gpu4pyscf/scf/hf.py:206-341), each
cycle one J/K build over that molecule's classes.  ``BatchRHF`` advances many
molecules together: every cycle builds the incremental J/K of all molecules
that have not converged in one batched build (``BatchJK``: one launch per
angular class serves every molecule), then runs each molecule's CDIIS,
diagonalisation and convergence test exactly as ``RHF.scf`` does, so every
molecule takes the same cycles and reaches the same energy as its own
``RHF``.  Diagonalisations of molecules with the same basis size go through
one batched ``torch.linalg.eigh``.  Converged molecules carry a zero density
change, which the density screening of the batched build drops.
"""

import math
import time

import torch

from . import hf
from .jk_batch import BatchJK


class BatchRHF:
    def __init__(self, mols, conv_tol=1e-9, max_cycle=50, precision='fp64', split_thresh=1e-6,
                 direct_scf_tol=1e-13):
        self.mols = list(mols)
        self.conv_tol = conv_tol
        self.conv_tol_grad = None
        self.max_cycle = max_cycle
        self.diis_space = 8
        self.diis_start_cycle = 1
        self.precision = precision
        self.split_thresh = split_thresh
        self.direct_scf_tol = direct_scf_tol
        self.verbose = 0
        self.jk = BatchJK(self.mols, direct_scf_tol)
        # per-molecule one-electron integrals, orthogonaliser and SAD guess
        # come from the single-molecule driver
        self.single = [hf.RHF(m) for m in self.mols]
        for mf in self.single:
            mf.direct_scf_tol = direct_scf_tol

    def _veff(self, dms, dms_last, vhfs_last, active):
        """J - K/2 of every molecule from its density change (zero for the
        inactive ones), one batched build."""
        ddm = []
        for m, d in enumerate(dms):
            if dms_last is None:
                ddm.append(d)
            elif active[m]:
                ddm.append(d - dms_last[m])
            else:
                ddm.append(torch.zeros_like(d))
        self.jk.precision, self.jk.split_thresh = self.precision, self.split_thresh
        js, ks = self.jk.get_jk([x[None] for x in ddm], hermi=1)
        out = []
        for m, (j, k) in enumerate(zip(js, ks)):
            v = j[0] - 0.5 * k[0]
            out.append(v if vhfs_last is None else vhfs_last[m] + v)
        return out

    def _eig_all(self, focks, idx):
        """Eigenpairs of the orthogonalised Fock matrices of molecules idx;
        equal sizes share one batched eigh."""
        res = {}
        groups = {}
        for m in idx:
            groups.setdefault(self.single[m]._X.shape[1], []).append(m)
        for ms in groups.values():
            Xs = [self.single[m]._X for m in ms]
            A = torch.stack([X.T @ focks[m] @ X for m, X in zip(ms, Xs)])
            e, c = torch.linalg.eigh(A)
            for k, m in enumerate(ms):
                res[m] = (e[k], Xs[k] @ c[k])
        return res

    def kernel(self, dm0s=None):
        """Runs all SCFs; returns the list of total energies.  dm0s: None
        (SAD for every molecule) or a list of user-basis densities (None
        entries take SAD)."""
        t0 = time.perf_counter()
        n = len(self.mols)
        for mol in self.mols:
            if mol.nelectron % 2:
                raise ValueError('RHF needs an even number of electrons')
        h1e = [mf.get_hcore() for mf in self.single]
        s1e = [mf.get_ovlp() for mf in self.single]
        enuc = [mf.energy_nuc() for mf in self.single]
        dms = []
        for m, mf in enumerate(self.single):
            d0 = None if dm0s is None else dm0s[m]
            dms.append(mf.get_init_guess() if d0 is None
                       else torch.as_tensor(d0, device='cuda', dtype=torch.float64))
        tol_grad = self.conv_tol_grad or math.sqrt(self.conv_tol)
        active = [True] * n
        vhf = self._veff(dms, None, None, active)
        e_tot = [self.single[m].energy_elec(dms[m], h1e[m], vhf[m])[0] + enuc[m] for m in range(n)]
        diis = [hf.CDIIS(self.diis_space) for _ in range(n)]
        cycles = [0] * n
        converged = [False] * n
        mo = [None] * n
        nbuild = 1
        for cycle in range(self.max_cycle):
            idx = [m for m in range(n) if active[m]]
            if not idx:
                break
            focks = {}
            for m in idx:
                X = self.single[m]._X
                fock = h1e[m] + vhf[m]
                if cycle >= self.diis_start_cycle:   # as RHF.scf
                    err = X.T @ (fock @ dms[m] @ s1e[m] - s1e[m] @ dms[m] @ fock) @ X
                    fock = diis[m].update(fock, err)
                focks[m] = fock
            eig = self._eig_all(focks, idx)
            dms_last = list(dms)
            e_last = list(e_tot)
            for m in idx:
                mo_e, mo_c = eig[m]
                occ = self.single[m].get_occ(mo_e, mo_c)
                mo[m] = (mo_e, mo_c, occ)
                dms[m] = self.single[m].make_rdm1(mo_c, occ)
            vhf = self._veff(dms, dms_last, vhf, active)
            nbuild += 1
            for m in idx:
                mf = self.single[m]
                e_tot[m] = mf.energy_elec(dms[m], h1e[m], vhf[m])[0] + enuc[m]
                mo_e, mo_c, occ = mo[m]
                f_mo = mo_c.T @ (h1e[m] + vhf[m]) @ mo_c
                o = occ > 0
                gnorm = float(torch.linalg.norm(f_mo[~o][:, o]).item()) * 2.
                cycles[m] = cycle + 1
                if abs(e_tot[m] - e_last[m]) < self.conv_tol and gnorm < tol_grad:
                    converged[m] = True
                    active[m] = False
            if self.verbose:
                print('batch cycle %d: %d of %d molecules still running, %.2f s'
                      % (cycle + 1, sum(active), n, time.perf_counter() - t0), flush=True)
        self.e_tot = e_tot
        self.cycles = cycles
        self.converged = converged
        self.dms = dms
        self.mo = mo
        self.summary = {'jk_builds': nbuild, 'wall_s': time.perf_counter() - t0}
        return e_tot
