"""The SCF driver's commutator-DIIS extrapolation (scf/hf.py CDIIS) on CPU
tensors: for a linear fixed-point map x -> A x + b, DIIS over the iterates
and their residuals is a Krylov method and solves an n-dimensional problem
in about n + 1 steps, where plain iteration only contracts by the spectral
radius of A per step."""
import numpy as np
import torch

from gpu4pyscf_gb300.scf.hf import CDIIS


def _problem(n=6, seed=0):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    A = Q @ np.diag(np.linspace(0.3, 0.9, n)) @ Q.T
    b = rng.normal(size=n)
    x_star = np.linalg.solve(np.eye(n) - A, b)
    return torch.as_tensor(A), torch.as_tensor(b), torch.as_tensor(x_star)


def test_linear_fixed_point():
    A, b, x_star = _problem()
    n = len(b)
    diis = CDIIS(space=n + 2)
    x = torch.zeros_like(b)
    for it in range(n + 2):
        fx = A @ x + b
        x = diis.update(fx, fx - x)
    assert float((x - x_star).abs().max()) < 1e-8
    # plain iteration after the same number of steps is still far off
    y = torch.zeros_like(b)
    for _ in range(n + 2):
        y = A @ y + b
    assert float((y - x_star).abs().max()) > 1e-2


def test_space_limit_keeps_last_vectors():
    A, b, _ = _problem(seed=1)
    diis = CDIIS(space=3)
    x = torch.zeros_like(b)
    for _ in range(6):
        fx = A @ x + b
        x = diis.update(fx, fx - x)
        assert len(diis.fs) <= 3 and len(diis.es) == len(diis.fs)
