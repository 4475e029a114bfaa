"""Learned initial guess end to end on a small set: converged densities from
the engine's RHF, training on the network kernels, held-out SCF from the
predicted density versus the superposition-of-atoms guess."""
import pytest

pytestmark = pytest.mark.gpu


def test_learned_guess_small():
    from gpu4pyscf_gb300.scf import hf, learned_guess as lg
    confsets = lg.make_conformers(2, 10, 'syn-def2-svp', seed=3)
    nblock = max(b - a for cs in confsets for (a, b) in lg.block_slices(cs[0]))
    data = lg.generate(confsets, holdout=2)
    model = lg.train(data, nblock, epochs=80, batch=1024)
    assert model.loss_history[-1] < 0.5 * model.loss_history[0]
    held = [m for cs in confsets for m in cs[-2:]]
    res = lg.evaluate(model, held, n_raw=0)
    assert res['all_converged']
    # unchanged converged energy
    assert res['max_abs_dE'] < 1e-7
    # what the trained network gains over the method without it: a guess
    # closer to the converged density than SAD on every held-out conformer
    for r in res['rows']:
        assert r['rms_learned'] < r['rms_sad'], r
    assert res['mean_cycles_learned'] <= res['mean_cycles_sad']
    mf = hf.RHF(held[0])
    mf.init_guess = 'learned'
    mf.guess_model = model
    mf.conv_tol = 1e-8
    mf.kernel()
    assert mf.converged
