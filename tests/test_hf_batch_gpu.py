"""Batched RHF (many molecules in lockstep, one batched J/K build per cycle)
against the single-molecule RHF driver: same converged energies and the
same cycle counts, since every molecule runs the same CDIIS iterations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mols():
    from gpu4pyscf_gb300 import gto
    from gpu4pyscf_gb300.scf import learned_guess as lg
    out = [gto.M(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-6-31g*')]
    confs = lg.make_conformers(2, 2, 'syn-def2-svp', seed=5)
    out += [cs[0] for cs in confs] + [confs[0][1]]
    return out


def test_batch_rhf_matches_single():
    from gpu4pyscf_gb300.scf import hf, hf_batch
    mols = _mols()
    b = hf_batch.BatchRHF(mols, conv_tol=1e-9)
    es = b.kernel()
    assert all(b.converged)
    for m, e, cyc in zip(mols, es, b.cycles):
        mf = hf.RHF(m)
        mf.conv_tol = 1e-9
        e1 = mf.kernel()
        assert mf.converged
        assert abs(e - e1) < 1e-8, (e, e1)
        assert abs(cyc - mf.cycles) <= 1, (cyc, mf.cycles)


def test_batch_rhf_from_given_densities():
    """Converged densities as the start: every molecule stops after one or
    two cycles at the same energy."""
    from gpu4pyscf_gb300.scf import hf_batch
    mols = _mols()[1:]
    a = hf_batch.BatchRHF(mols, conv_tol=1e-9)
    ea = a.kernel()
    b = hf_batch.BatchRHF(mols, conv_tol=1e-9)
    eb = b.kernel(dm0s=[d.cpu().numpy() for d in a.dms])
    assert all(b.converged)
    assert max(b.cycles) <= 2
    assert np.allclose(ea, eb, atol=1e-8)
