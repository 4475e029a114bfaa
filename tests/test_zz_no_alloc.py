"""The allocation-free J/K entry point, called through the C ABI.

jk_build_noalloc serves callers that may not allocate device memory once
they are running: a process held to a fixed device-memory budget after
start-up, or a host application whose own framework owns every device
allocation and forbids a library from calling cudaMalloc.  Its results must
equal those of jk_build, call after call, although every call reuses the
same fixed scratch array.  This file is collected last on purpose, so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(basis='syn-def2-svp'):
    import torch
    from gpu4pyscf_gb300 import gto
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk
    lib = libjk.load()
    lib.jk_build_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.jk_build_noalloc.restype = ctypes.c_int
    lib.jk_noalloc_scratch_bytes.restype = ctypes.c_int
    mol = gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696; C 0 2.2 0.3', basis=basis)
    opt = jk._VHFOpt(mol).build()
    return torch, lib, libjk, opt


def _noalloc(torch, lib, libjk, opt, dms, hermi, prec=None, split=0.):
    prec = libjk.JK_PREC_FP64 if prec is None else prec
    vj = torch.full_like(dms, float('nan'))
    vk = torch.full_like(dms, float('nan'))
    err = lib.jk_build_noalloc(opt._handle, dms.data_ptr(), dms.shape[0], dms.shape[-1], hermi, 1, 1,
                               prec, split, vj.data_ptr(), vk.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    libjk.check(err, 'jk_build_noalloc')
    return vj, vk


@pytest.mark.parametrize('hermi', [1, 0])
def test_noalloc_matches_jk_build_twice(hermi):
    torch, lib, libjk, opt = _setup()
    rng = np.random.default_rng(11)
    n = opt.sorted_mol.nao
    for call in range(2):
        d = rng.random((2, n, n)) - .4
        if hermi == 1:
            d = d + d.transpose(0, 2, 1)
        dms = torch.as_tensor(d, device='cuda')
        ref_j, ref_k = opt._build(dms, hermi, True, True)
        vj, vk = _noalloc(torch, lib, libjk, opt, dms, hermi)
        torch.cuda.synchronize()
        assert abs(vj - ref_j).max().item() < 1e-10, call
        assert abs(vk - ref_k).max().item() < 1e-10, call


@pytest.mark.parametrize('precision', ['mixed', 'mixed-fp32roots'])
def test_noalloc_mixed_matches_jk_build_twice(precision):
    """Mixed FP32/FP64 builds through the allocation-free entry point agree
    with jk_build's mixed builds (the same quartets in the same precision;
    only the order of the FP64 atomic additions differs)."""
    torch, lib, libjk, opt = _setup('syn-def2-tzvp')
    rng = np.random.default_rng(12)
    n = opt.sorted_mol.nao
    opt.precision, opt.split_thresh = precision, 1e-4
    for call in range(2):
        d = rng.random((1, n, n)) - .4
        d = d + d.transpose(0, 2, 1)
        dms = torch.as_tensor(d, device='cuda')
        ref_j, ref_k = opt._build(dms, 1, True, True)
        vj, vk = _noalloc(torch, lib, libjk, opt, dms, 1, libjk.PRECISIONS[precision], 1e-4)
        torch.cuda.synchronize()
        assert abs(vj - ref_j).max().item() < 1e-10, call
        assert abs(vk - ref_k).max().item() < 1e-10, call
    opt.precision = 'fp64'


def test_noalloc_rejects_oversize_request():
    torch, lib, libjk, opt = _setup()
    n = opt.sorted_mol.nao
    limit = lib.jk_noalloc_scratch_bytes()
    n_dm = limit // (8 * n * n * 4) + 2
    dms = torch.zeros((1, n, n), dtype=torch.float64, device='cuda')
    out = torch.zeros_like(dms)
    err = lib.jk_build_noalloc(opt._handle, dms.data_ptr(), n_dm, n, 1, 1, 1, libjk.JK_PREC_FP64, 0.,
                               out.data_ptr(), out.data_ptr(), None)
    assert err == -5
    assert b'scratch' in lib.jk_last_error()
