"""The Rys root/weight tables the kernels use (csrc/rys_tables.inc), checked
on the CPU against the defining property of Rys quadrature: the n-point rule
at parameter T integrates t^(2k), so sum_r w_r u_r^k = F_k(T) (Boys function,
from the oracle) for k = 0 .. 2n-1.  The FP64 table (degree 9 on intervals
of width 1/2) must hold this to ~1e-13 relative, the FP32 table (degree 8 on
intervals of width 2, stored in float) to a few FP32 ulps; the Gauss-Hermite
asymptote beyond T_asym(n) = 40 + 6n is checked the same way.
"""
import os
import re

import numpy as np
import pytest

from oracle import oracle as orc

INC = os.path.join(os.path.dirname(__file__), '..', 'gpu4pyscf_gb300', 'csrc', 'rys_tables.inc')


def _parse():
    text = open(INC).read()
    defs = dict((m.group(1), int(m.group(2))) for m in re.finditer(r'#define (RYS_\w+) (\d+)\n', text))
    nint = [int(x) for x in re.search(r'rys_nint_host\[[^]]*\] = \{([^}]*)\}', text).group(1).split(',')]
    nint_f = [int(x) for x in re.search(r'rys_nint_f_host\[[^]]*\] = \{([^}]*)\}', text).group(1).split(',')]

    def block(name, conv):
        body = re.search(name + r'\[[A-Z_]+\] = \{\n(.*?)\n\};', text, re.S).group(1)
        return np.array([conv(v) for v in body.replace('\n', ' ').split(',') if v.strip()])

    tab = block('rys_coef_host', lambda v: float.fromhex(v.strip()))
    tab_f = block('rys_coef_f_host', lambda v: float(v.strip().rstrip('f'))).astype(np.float32)
    asym_x2 = np.array([float.fromhex(v) for v in re.search(r'#define RYS_ASYM_X2_LIST (.*)\n', text).group(1).split(',')])
    asym_w = np.array([float.fromhex(v) for v in re.search(r'#define RYS_ASYM_W_LIST (.*)\n', text).group(1).split(',')])
    return defs, nint, nint_f, tab, tab_f, asym_x2, asym_w


def _offsets(nint, deg):
    offs = [0, 0]
    for n in range(1, len(nint) - 1):
        offs.append(offs[-1] + nint[n] * (deg + 1) * 2 * n)
    return offs


def _eval(tab, off, deg, n, T, dtype, width):
    k = int(T / width)
    x = dtype(T - (k + 0.5) * width)
    c = tab[off + k * (deg + 1) * 2 * n: off + (k + 1) * (deg + 1) * 2 * n].reshape(deg + 1, 2 * n).astype(dtype)
    a = c[deg].copy()
    for i in range(deg - 1, -1, -1):
        a = a * x + c[i]
    return a[:n].astype(np.float64), a[n:].astype(np.float64)


def _moments_err(u, w, T, n):
    F = orc.boys(2 * n - 1, T)
    m = np.array([np.sum(w * u ** k) for k in range(2 * n)])
    return np.max(np.abs(m - F) / np.abs(F))


DATA = _parse()


@pytest.mark.parametrize('n', range(1, 10))
def test_fp64_table(n):
    defs, nint, _, tab, _, _, _ = DATA
    off = _offsets(nint, defs['RYS_DEG'])[n]
    rng = np.random.default_rng(n)
    tmax = 40 + 6 * n
    assert nint[n] == tmax * defs['RYS_INV_WIDTH']
    for T in np.concatenate([[0., 1e-9, 0.25, 0.5, 1.999, 2.0, tmax - 1e-9], rng.uniform(0, tmax, 40)]):
        u, w = _eval(tab, off, defs['RYS_DEG'], n, T, np.float64, 1. / defs['RYS_INV_WIDTH'])
        assert _moments_err(u, w, T, n) < 5e-13, T


@pytest.mark.parametrize('n', range(1, 10))
def test_fp32_table(n):
    defs, _, nint, _, tab_f, _, _ = DATA
    off = _offsets(nint, defs['RYS_DEG_F'])[n]
    assert off == int(re.search(r'rys_offset_f_host\[[^]]*\] = \{([^}]*)\}', open(INC).read()).group(1).split(',')[n])
    rng = np.random.default_rng(100 + n)
    for T in np.concatenate([[0., 1e-6, 0.5, 1.999, 2.0], rng.uniform(0, 2 * nint[n], 40)]):
        u, w = _eval(tab_f, off, defs['RYS_DEG_F'], n, np.float32(T), np.float32, defs['RYS_WIDTH_F'])
        assert _moments_err(u, w, float(np.float32(T)), n) < 2e-6 * n, T


@pytest.mark.parametrize('n', range(1, 10))
def test_asymptote(n):
    defs, _, _, _, _, x2, wt = DATA
    o = n * (n - 1) // 2
    tmax = 40 + 6 * n
    for T in (tmax, tmax + 7.3, 400.):
        u = x2[o:o + n] / T
        w = wt[o:o + n] / np.sqrt(T)
        assert _moments_err(u, w, T, n) < 1e-14
