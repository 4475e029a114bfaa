"""The learned-guess network: oracle gradients pinned by finite
differences (CPU), GPU kernels against the oracle (GPU)."""
import numpy as np
import pytest

from oracle import mlp_ref


def _params(sizes, seed=0):
    rng = np.random.default_rng(seed)
    W = [rng.normal(size=(i, o)) * np.sqrt(2. / i) for i, o in zip(sizes[:-1], sizes[1:])]
    b = [rng.normal(size=o) * .1 for o in sizes[1:]]
    return W, b


def test_oracle_gradients_finite_difference():
    sizes = [7, 11, 9, 5]
    W, b = _params(sizes)
    rng = np.random.default_rng(1)
    X = rng.normal(size=(6, 7))
    T = rng.normal(size=(6, 5))
    mask = (rng.random((6, 5)) > .3).astype(float)
    gW, gb, gX = mlp_ref.grads(W, b, X, T, mask)
    h = 1e-6
    for l in range(len(W)):
        for idx in [(0, 0), (W[l].shape[0] - 1, W[l].shape[1] - 1), (1, 2)]:
            Wp = [w.copy() for w in W]
            Wm = [w.copy() for w in W]
            Wp[l][idx] += h
            Wm[l][idx] -= h
            fd = (mlp_ref.loss(Wp, b, X, T, mask) - mlp_ref.loss(Wm, b, X, T, mask)) / (2 * h)
            assert abs(fd - gW[l][idx]) < 1e-7 * max(1., abs(fd))
        bp = [x.copy() for x in b]
        bm = [x.copy() for x in b]
        bp[l][0] += h
        bm[l][0] -= h
        fd = (mlp_ref.loss(W, bp, X, T, mask) - mlp_ref.loss(W, bm, X, T, mask)) / (2 * h)
        assert abs(fd - gb[l][0]) < 1e-7 * max(1., abs(fd))


@pytest.mark.gpu
def test_gpu_forward_backward_vs_oracle():
    import torch
    from gpu4pyscf_gb300.scf import mlp
    sizes = [80, 256, 256, 256, 196]
    net = mlp.DenseMLP(sizes, seed=3)
    W = [w.cpu().double().numpy() for w in net.W]
    rng = np.random.default_rng(2)
    b = [rng.normal(size=o) * .1 for o in sizes[1:]]
    net.b = [torch.as_tensor(x, dtype=torch.float32, device='cuda') for x in b]
    b = [x.astype(np.float32).astype(np.float64) for x in b]
    X = rng.normal(size=(333, 80)).astype(np.float32)
    T = rng.normal(size=(333, 196)).astype(np.float32)
    mask = (rng.random((333, 196)) > .4).astype(np.float32)
    y = net.forward(torch.as_tensor(X, device='cuda'))
    yref, _ = mlp_ref.forward(W, b, X.astype(np.float64))
    assert np.abs(y.cpu().numpy() - yref).max() < 2e-4 * max(1., np.abs(yref).max())
    loss, g = mlp.mse(y, torch.as_tensor(T, device='cuda'), torch.as_tensor(mask, device='cuda'))
    assert abs(loss.item() - mlp_ref.loss(W, b, X, T, mask)) < 1e-4 * mlp_ref.loss(W, b, X, T, mask)
    gX = net.backward(g)
    gW, gb, gXref = mlp_ref.grads(W, b, X.astype(np.float64), T.astype(np.float64), mask.astype(np.float64))
    for l in range(len(W)):
        scale = max(1e-6, np.abs(gW[l]).max())
        assert np.abs(net.gW[l].cpu().numpy() - gW[l]).max() < 2e-3 * scale, l
        assert np.abs(net.gb[l].cpu().numpy() - gb[l]).max() < 2e-3 * max(1e-6, np.abs(gb[l]).max()), l
    assert np.abs(gX.cpu().numpy() - gXref).max() < 2e-3 * np.abs(gXref).max()


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    import torch
    from gpu4pyscf_gb300.scf import mlp
    rng = np.random.default_rng(0)
    X = torch.as_tensor(rng.normal(size=(512, 16)).astype(np.float32), device='cuda')
    T = torch.sin(X[:, :4] * 2.) + X[:, 4:8] ** 2
    net = mlp.DenseMLP([16, 64, 64, 4], seed=1)
    first = None
    for it in range(300):
        y = net.forward(X)
        loss, g = mlp.mse(y, T)
        net.backward(g)
        net.adam_step(lr=3e-3)
        if first is None:
            first = loss.item()
    assert loss.item() < 0.1 * first
