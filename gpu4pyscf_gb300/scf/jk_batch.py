"""J/K for many molecules at once.

The reference computes J/K one molecule at a time (a Python loop over
``get_jk`` calls, each looping over angular classes, gpu4pyscf/scf/jk.py:
492-641).  ``BatchJK`` merges the sorted bases of all molecules into one
optimizer (``jk_opt_create_batch``): every angular class of every molecule is
served by one launch of that class's persistent kernel, whose warps steal
work units from all molecules.  Densities of different counts per molecule
(1-4 here) are padded to the largest count with zero densities, which the
density screening drops.  The whole build -- basis transforms into the sorted
basis, packing, the class launches, unpacking and back-transforms -- can be
captured once into a CUDA graph and replayed (``capture`` / ``replay``).
"""

import ctypes

import numpy as np
import torch

from ..gto.sorted_basis import SortedBasis
from ..lib import libjk
from .jk import LMAX


class BatchJK:
    def __init__(self, mols, direct_scf_tol=1e-13, diffuse_cutoff=None):
        self.mols = list(mols)
        self.direct_scf_tol = direct_scf_tol
        self.diffuse_cutoff = diffuse_cutoff
        self.precision = 'fp64'
        self.split_thresh = 1e-6
        self._handle = None
        self._graph = None
        self.build()

    def build(self):
        self.sorted = [SortedBasis(m, self.diffuse_cutoff) for m in self.mols]
        for sb in self.sorted:
            if sb.lmax > LMAX:
                raise NotImplementedError('shells with l > %d are not supported' % LMAX)
        atm, bas, env, smol, sao = [], [], [], [], []
        env_off = 0
        atm_off = 0
        for m, sb in enumerate(self.sorted):
            a = np.array(sb._atm, dtype=np.int32, copy=True)
            b = np.array(sb._bas, dtype=np.int32, copy=True)
            a[:, 1] += env_off
            a[:, 3] += env_off
            b[:, 0] += atm_off
            b[:, 5] += env_off
            b[:, 6] += env_off
            atm.append(a)
            bas.append(b)
            env.append(np.asarray(sb._env, dtype=np.float64))
            smol.append(np.full(sb.nbas, m, dtype=np.int32))
            sao.append(np.asarray(sb.ao_loc[:-1], dtype=np.int32))
            env_off += len(sb._env)
            atm_off += len(a)
        atm = np.concatenate(atm)
        bas = np.concatenate(bas)
        env = np.concatenate(env)
        smol = np.concatenate(smol)
        sao = np.concatenate(sao)
        order = np.argsort(bas[:, 1], kind='stable')
        self._atm = np.ascontiguousarray(atm)
        self._bas = np.ascontiguousarray(bas[order])
        self._env = np.ascontiguousarray(env)
        self._smol = np.ascontiguousarray(smol[order])
        self._sao = np.ascontiguousarray(sao[order])
        self.mol_nao = np.array([sb.nao for sb in self.sorted], dtype=np.int32)
        self.mol_base = np.append(0, np.cumsum(self.mol_nao.astype(np.int64) ** 2))
        self.ntot = int(self.mol_base[-1])
        lib = libjk.load()
        h = ctypes.c_void_p()
        torch.cuda.current_device()
        err = lib.jk_opt_create_batch(self._atm.ctypes.data, len(self._atm), self._bas.ctypes.data,
                                      len(self._bas), self._env.ctypes.data, len(self._env),
                                      self._smol.ctypes.data, self._sao.ctypes.data, len(self.mols),
                                      self.mol_nao.ctypes.data, float(self.direct_scf_tol), 0,
                                      ctypes.byref(h))
        libjk.check(err, 'jk_opt_create_batch')
        self._handle = h
        self._coeff = [torch.as_tensor(sb.coeff, device='cuda') for sb in self.sorted]
        return self

    def __del__(self):
        if self._handle is not None:
            try:
                libjk.load().jk_opt_destroy(self._handle)
            except Exception:
                pass
            self._handle = None

    # -- packed sorted-basis densities -------------------------------------
    def pack(self, dms_sorted, n_dm):
        out = torch.zeros((n_dm, self.ntot), dtype=torch.float64, device='cuda')
        for m, d in enumerate(dms_sorted):
            n = int(self.mol_nao[m])
            b = int(self.mol_base[m])
            out[:d.shape[0], b:b + n * n] = d.reshape(d.shape[0], n * n)
        return out

    def unpack(self, packed, counts):
        res = []
        for m, k in enumerate(counts):
            n = int(self.mol_nao[m])
            b = int(self.mol_base[m])
            res.append(packed[:k, b:b + n * n].reshape(k, n, n))
        return res

    def build_sorted(self, packed, hermi=1, with_j=True, with_k=True, stats=False):
        n_dm = packed.shape[0]
        vj = torch.empty_like(packed) if with_j else None
        vk = torch.empty_like(packed) if with_k else None
        prec = libjk.PRECISIONS[self.precision]
        st = libjk.JKStats() if stats else None
        err = libjk.load().jk_build_batch(self._handle, packed.data_ptr(), n_dm, int(hermi), int(with_j),
                                          int(with_k), prec, float(self.split_thresh),
                                          vj.data_ptr() if with_j else None, vk.data_ptr() if with_k else None,
                                          torch.cuda.current_stream().cuda_stream,
                                          ctypes.byref(st) if stats else None)
        libjk.check(err, 'jk_build_batch')
        if stats:
            self.last_stats = st.as_dict()
        return vj, vk

    def get_jk(self, dms, hermi=1, stats=False):
        """dms: list (one per molecule) of (n_dm_m, nao_m, nao_m) user-basis
        densities (numpy or torch).  Returns lists of J and K (torch)."""
        dms = [torch.as_tensor(np.asarray(d) if not isinstance(d, torch.Tensor) else d,
                               dtype=torch.float64, device='cuda') for d in dms]
        dms = [d if d.ndim == 3 else d[None] for d in dms]
        counts = [d.shape[0] for d in dms]
        n_dm = max(counts)
        self._set_counts(counts)
        ds = [C @ d @ C.T for C, d in zip(self._coeff, dms)]
        vj, vk = self.build_sorted(self.pack(ds, n_dm), hermi, stats=stats)
        js = [C.T @ v @ C for C, v in zip(self._coeff, self.unpack(vj, counts))]
        ks = [C.T @ v @ C for C, v in zip(self._coeff, self.unpack(vk, counts))]
        return js, ks

    def _set_counts(self, counts):
        counts = tuple(int(c) for c in counts)
        if getattr(self, '_counts', None) != counts:
            arr = np.asarray(counts, dtype=np.int32)
            libjk.check(libjk.load().jk_opt_set_mol_ndm(self._handle, arr.ctypes.data), 'jk_opt_set_mol_ndm')
            self._counts = counts

    def variants(self):
        """Current launch choice (alt, grid) of every (class, precision)."""
        lib = libjk.load()
        out = []
        a, g = ctypes.c_int(), ctypes.c_int()
        for q in range(lib.jk_n_quartet_classes()):
            for prec in (0, 1):
                libjk.check(lib.jk_opt_get_variant(self._handle, q, prec, ctypes.byref(a), ctypes.byref(g)),
                            'jk_opt_get_variant')
                out.append((q, prec, a.value, g.value))
        return out

    def set_variants(self, variants):
        lib = libjk.load()
        for q, prec, a, g in variants:
            libjk.check(lib.jk_opt_set_variant(self._handle, q, prec, a, g), 'jk_opt_set_variant')

    def tune(self, dms, hermi=1, reps=3):
        """Autotune the launch of every class on these densities
        (jk_opt_tune); later builds use the choices."""
        dms = [torch.as_tensor(np.asarray(d) if not isinstance(d, torch.Tensor) else d,
                               dtype=torch.float64, device='cuda') for d in dms]
        dms = [d if d.ndim == 3 else d[None] for d in dms]
        n_dm = max(d.shape[0] for d in dms)
        self._set_counts([d.shape[0] for d in dms])
        packed = self.pack([C @ d @ C.T for C, d in zip(self._coeff, dms)], n_dm)
        err = libjk.load().jk_opt_tune(self._handle, packed.data_ptr(), n_dm, int(hermi),
                                       libjk.PRECISIONS[self.precision], float(self.split_thresh),
                                       torch.cuda.current_stream().cuda_stream, int(reps))
        libjk.check(err, 'jk_opt_tune')
        return self

    # -- CUDA graph -----------------------------------------------------------
    def capture(self, dms, hermi=1):
        """Record the whole batched build for densities shaped like ``dms``
        into one CUDA graph; ``replay`` then reruns it on new values."""
        self._static_in = [torch.as_tensor(np.asarray(d) if not isinstance(d, torch.Tensor) else d,
                                           dtype=torch.float64, device='cuda').clone() for d in dms]
        self._static_in = [d if d.ndim == 3 else d[None] for d in self._static_in]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        self._set_counts([d.shape[0] for d in self._static_in])
        with torch.cuda.stream(s):
            for _ in range(2):  # allocate the workspace before capture
                self.get_jk(self._static_in, hermi)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._static_out = self.get_jk(self._static_in, hermi)
        self._graph = g
        return self

    def replay(self, dms=None):
        if dms is not None:
            for dst, src in zip(self._static_in, dms):
                src = torch.as_tensor(src, dtype=torch.float64, device='cuda')
                dst.copy_(src if src.ndim == 3 else src[None])
        self._graph.replay()
        return self._static_out
