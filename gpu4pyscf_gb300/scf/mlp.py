"""Dense FP32 network on the hand-written kernels of include/gb300mlp.h.

``DenseMLP(sizes)`` is a stack of dense layers with SiLU between them and a
linear output layer.  ``forward`` keeps what ``backward`` needs; ``backward``
returns the input gradient and fills the parameter gradients; ``adam_step``
updates the parameters.  Every product runs in ``mlp_gemm`` (operands
addressed by strides, so X^T dZ and dZ W^T need no transposed copies); the
SiLU derivative, bias gradients, loss and optimizer are kernels of the same
library.  ``MLPFunction`` wraps forward/backward as a torch autograd
Function for callers that want autograd.
"""

import ctypes
import math

import numpy as np
import torch

from ..lib import libjk

_sigs_done = False


def _lib():
    global _sigs_done
    lib = libjk.load()
    if not _sigs_done:
        vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
        lib.mlp_gemm.argtypes = [i32, i32, i32, vp, i64, i64, vp, i64, i64, vp, i32, f32, vp, vp, vp]
        lib.mlp_gemm.restype = i32
        lib.mlp_silu_backward.argtypes = [i64, vp, vp, vp, vp]
        lib.mlp_silu_backward.restype = i32
        lib.mlp_colsum.argtypes = [i32, i32, vp, vp, vp]
        lib.mlp_colsum.restype = i32
        lib.mlp_mse.argtypes = [i64, vp, vp, vp, f32, vp, vp, vp]
        lib.mlp_mse.restype = i32
        lib.mlp_adam.argtypes = [i64, vp, vp, vp, vp, f32, f32, f32, f32, i32, vp]
        lib.mlp_adam.restype = i32
        lib.mlp_last_error.argtypes = []
        lib.mlp_last_error.restype = ctypes.c_char_p
        _sigs_done = True
    return lib


def _check(err, what):
    if err:
        raise RuntimeError('%s failed (%d): %s' % (what, err, _lib().mlp_last_error().decode()))


def _st():
    return torch.cuda.current_stream().cuda_stream


def _p(t):
    return t.data_ptr() if t is not None else None


def gemm(A, B, transA=False, transB=False, bias=None, act=0, Z=None, out=None, beta=0.):
    """out = op(A) op(B) (+beta out) (+bias), SiLU if act=1 (pre-activation in Z)."""
    A = A.contiguous()
    B = B.contiguous()
    if transA:
        K, M = A.shape
        sam, sak = 1, M
    else:
        M, K = A.shape
        sam, sak = K, 1
    if transB:
        N, K2 = B.shape
        sbk, sbn = 1, K2
    else:
        K2, N = B.shape
        sbk, sbn = N, 1
    assert K == K2
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device='cuda')
    _check(_lib().mlp_gemm(M, N, K, _p(A), sam, sak, _p(B), sbk, sbn, _p(bias), act, float(beta),
                           _p(Z), _p(out), _st()), 'mlp_gemm')
    return out


class DenseMLP:
    def __init__(self, sizes, seed=0):
        self.sizes = list(sizes)
        g = torch.Generator(device='cpu').manual_seed(seed)
        self.W, self.b = [], []
        for i, o in zip(sizes[:-1], sizes[1:]):
            w = torch.randn((i, o), generator=g, dtype=torch.float32) * math.sqrt(2. / i)
            self.W.append(w.cuda())
            self.b.append(torch.zeros(o, dtype=torch.float32, device='cuda'))
        self.gW = [torch.zeros_like(w) for w in self.W]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step = 0
        self._cache = None

    @property
    def nlayers(self):
        return len(self.W)

    def forward(self, X, keep=True):
        X = X.contiguous().float()
        xs, zs = [X], []
        h = X
        for l in range(self.nlayers):
            last = l == self.nlayers - 1
            Z = None if last else torch.empty((h.shape[0], self.sizes[l + 1]), dtype=torch.float32, device='cuda')
            h = gemm(h, self.W[l], bias=self.b[l], act=0 if last else 1, Z=Z)
            if not last:
                zs.append(Z)
                xs.append(h)
        if keep:
            self._cache = (xs, zs)
        return h

    def backward(self, dY):
        xs, zs = self._cache
        g = dY.contiguous().float()
        for l in reversed(range(self.nlayers)):
            if l < self.nlayers - 1:
                dz = torch.empty_like(g)
                _check(_lib().mlp_silu_backward(g.numel(), _p(g), _p(zs[l]), _p(dz), _st()), 'mlp_silu_backward')
                g = dz
            X = xs[l]
            gemm(X, g, transA=True, out=self.gW[l])          # dW = X^T dZ
            _check(_lib().mlp_colsum(g.shape[0], g.shape[1], _p(g), _p(self.gb[l]), _st()), 'mlp_colsum')
            g = gemm(g, self.W[l], transB=True)                # dX = dZ W^T
        return g

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        lib = _lib()
        for p, gr, m, v in zip(self.W + self.b, self.gW + self.gb, self.mW + self.mb, self.vW + self.vb):
            _check(lib.mlp_adam(p.numel(), _p(p), _p(gr), _p(m), _p(v), lr, b1, b2, eps, self.step, _st()),
                   'mlp_adam')

    def state(self):
        return {'sizes': self.sizes, 'W': [w.cpu().numpy() for w in self.W], 'b': [b.cpu().numpy() for b in self.b]}

    def load(self, st):
        self.W = [torch.as_tensor(w, device='cuda') for w in st['W']]
        self.b = [torch.as_tensor(b, device='cuda') for b in st['b']]
        return self


def mse(y, t, mask=None):
    """Masked mean-squared error and its gradient (loss as a device scalar)."""
    n = y.numel()
    count = float(mask.sum().item()) if mask is not None else float(n)
    grad = torch.empty_like(y)
    loss = torch.zeros(1, dtype=torch.float32, device='cuda')
    _check(_lib().mlp_mse(n, _p(y), _p(t.contiguous()), _p(mask), 1. / max(count, 1.), _p(grad), _p(loss), _st()),
           'mlp_mse')
    return loss, grad


class MLPFunction(torch.autograd.Function):
    """Autograd wrapper: forward/backward through the network's kernels."""

    @staticmethod
    def forward(ctx, X, net):
        ctx.net = net
        return net.forward(X, keep=True)

    @staticmethod
    def backward(ctx, dY):
        return ctx.net.backward(dY), None
