"""Generate the Rys root/weight interpolation tables (rys_tables.inc).

Method (this project's own tables; nothing is taken from other code):
* For n roots and parameter T the Rys quadrature is the n-point Gauss rule of
  the measure d mu(x) = exp(-T x) / (2 sqrt(x)) dx on [0, 1], whose moments
  are the Boys functions F_k(T) = 1F1(k+1/2; k+3/2; -T) / (2k+1).  Nodes and
  weights come from the moments by the Chebyshev algorithm (ordinary moments
  -> three-term recurrence), then Golub-Welsch on the Jacobi matrix, all in
  80-digit mpmath arithmetic.
* 0 <= T < T_asym(n): piecewise polynomials on intervals of width 1/2.  On
  each interval the 2n functions (u_1..u_n, w_1..w_n) are interpolated at
  the 10 Chebyshev points and the interpolant is re-expanded, in high
  precision, in monomials of x = T - centre (|x| <= 1/4), so the device
  evaluates 9 Horner steps per function (max relative error 4e-16).  On
  GB300 every FP64 instruction is precious and table loads are not: narrow
  intervals trade table size (1.1 MB) for FMAs.
* The FP32 quartets use a second table on intervals of width 2 with degree
  DEG_F = 8 (9 Chebyshev points), whose interpolation error (< 4e-9
  relative) is below FP32 rounding; it is staged in shared memory by the
  FP32 kernels, so it stays small.
* T >= T_asym(n): u_r = h_r^2 / T, w_r = W_r / sqrt(T), with h_r, W_r the
  positive nodes and weights of 2n-point Gauss-Hermite quadrature (the
  integral over [0, 1] extended to [0, inf)).  T_asym(n) = 40 + 6n is where
  that tail error falls below 3e-16 relative.

Run:  python gen_rys_tables.py   (needs mpmath; writes rys_tables.inc here)
"""

import os
import sys
import multiprocessing as mp_proc

NMAX = 9
DEG = 9
INV_WIDTH = 2     # FP64 table: intervals of width 1 / INV_WIDTH
DEG_F = 8
WIDTH_F = 2       # FP32 table: intervals of width WIDTH_F
DPS = 80


def t_asym(n):
    return 40 + 6 * n   # a multiple of both interval widths


def _mp():
    import mpmath
    mpmath.mp.dps = DPS
    return mpmath


def boys(mp, k, T):
    return mp.hyp1f1(k + mp.mpf(1) / 2, k + mp.mpf(3) / 2, -T) / (2 * k + 1)


def rys(mp, n, T):
    T = mp.mpf(T)
    mu = [boys(mp, k, T) for k in range(2 * n)]
    sig_prev = [mp.mpf(0)] * (2 * n)
    sig = mu[:]
    alpha = [mu[1] / mu[0]]
    beta = [mu[0]]
    for k in range(1, n):
        new = [mp.mpf(0)] * (2 * n)
        for l in range(k, 2 * n - k):
            new[l] = sig[l + 1] - alpha[k - 1] * sig[l] - beta[k - 1] * sig_prev[l]
        alpha.append(new[k + 1] / new[k] - sig[k] / sig[k - 1])
        beta.append(new[k] / sig[k - 1])
        sig_prev, sig = sig, new
    J = mp.matrix(n, n)
    for i in range(n):
        J[i, i] = alpha[i]
        if i + 1 < n:
            J[i, i + 1] = J[i + 1, i] = mp.sqrt(beta[i + 1])
    E, Q = mp.eigsy(J)
    idx = sorted(range(n), key=lambda i: E[i])
    return [E[i] for i in idx], [beta[0] * Q[0, i] ** 2 for i in idx]


def hermite(mp, m):
    J = mp.matrix(m, m)
    for i in range(m - 1):
        J[i, i + 1] = J[i + 1, i] = mp.sqrt(mp.mpf(i + 1) / 2)
    E, Q = mp.eigsy(J)
    idx = sorted(range(m), key=lambda i: E[i])
    return [E[i] for i in idx], [mp.sqrt(mp.pi) * Q[0, i] ** 2 for i in idx]


def fit_interval(args):
    """Monomial coefficients [deg+1][2n] in x = T - centre on interval k of
    width `width`."""
    n, k, deg, width = args
    mp = _mp()
    a = mp.mpf(k) * mp.mpf(width)
    half = mp.mpf(width) / 2
    c = a + half
    N = deg + 1
    nodes = [mp.cos(mp.pi * (j + mp.mpf(1) / 2) / N) for j in range(N)]
    vals = []
    for x in nodes:
        u, w = rys(mp, n, c + half * x)
        vals.append(u + w)
    out = []
    for f in range(2 * n):
        # Chebyshev coefficients in t = (T - c) / half
        cheb = []
        for m in range(N):
            s = mp.mpf(0)
            for j in range(N):
                s += vals[j][f] * mp.cos(m * mp.pi * (j + mp.mpf(1) / 2) / N)
            cheb.append(s * 2 / N)
        cheb[0] /= 2
        # Chebyshev -> monomials in t
        mono = [mp.mpf(0)] * N
        Tkm1 = [mp.mpf(1)] + [mp.mpf(0)] * (N - 1)
        Tk = [mp.mpf(0), mp.mpf(1)] + [mp.mpf(0)] * (N - 2)
        for i in range(N):
            mono[i] += cheb[0] * Tkm1[i] + (cheb[1] * Tk[i] if N > 1 else 0)
        for m in range(2, N):
            Tn = [mp.mpf(0)] * N
            for i in range(N):
                if i > 0:
                    Tn[i] += 2 * Tk[i - 1]
                Tn[i] -= Tkm1[i]
            for i in range(N):
                mono[i] += cheb[m] * Tn[i]
            Tkm1, Tk = Tk, Tn
        # t = x / half, so coefficient of x^i is mono[i] / half^i
        out.append([mono[i] / half ** i for i in range(N)])
    return n, k, [[float(out[f][i]) for f in range(2 * n)] for i in range(N)]


def check_interval(args):
    """Max relative error of a table (coefficients rounded to double) on one
    interval."""
    n, k, coef, deg, width = args
    mp = _mp()
    worst = 0.
    for frac in (0.07, 0.31, 0.5, 0.77, 0.96):
        T = (k + frac) * width
        u, w = rys(mp, n, T)
        ref = [float(v) for v in u + w]
        x = T - (k + 0.5) * width
        for f in range(2 * n):
            acc = coef[deg][f]
            for i in range(deg - 1, -1, -1):
                acc = acc * x + coef[i][f]
            worst = max(worst, abs(acc - ref[f]) / abs(ref[f]))
    return worst


def main():
    mp = _mp()
    w64 = 1. / INV_WIDTH
    jobs = [(n, k, DEG, w64) for n in range(1, NMAX + 1) for k in range(t_asym(n) * INV_WIDTH)]
    jobs_f = [(n, k, DEG_F, WIDTH_F) for n in range(1, NMAX + 1) for k in range(t_asym(n) // WIDTH_F)]
    ctx = mp_proc.get_context('spawn')
    with ctx.Pool(os.cpu_count()) as pool:
        res = pool.map(fit_interval, jobs, chunksize=4)
        table = {(n, k): c for n, k, c in res}
        errs = pool.map(check_interval, [(n, k, table[(n, k)], DEG, w64) for n, k, _, _ in jobs], chunksize=4)
        res_f = pool.map(fit_interval, jobs_f, chunksize=4)
        table_f = {(n, k): c for n, k, c in res_f}
        errs_f = pool.map(check_interval, [(n, k, table_f[(n, k)], DEG_F, WIDTH_F) for n, k, _, _ in jobs_f],
                          chunksize=4)
    worst, worst_f = {}, {}
    for (n, k, _, _), e in zip(jobs, errs):
        worst[n] = max(worst.get(n, 0.), e)
    for (n, k, _, _), e in zip(jobs_f, errs_f):
        worst_f[n] = max(worst_f.get(n, 0.), e)
    lines = []
    lines.append('// Generated by gen_rys_tables.py -- do not edit.')
    lines.append('// Rys roots/weights: piecewise degree-%d polynomials in x = T - centre on' % DEG)
    lines.append('// intervals of width 1/%d for T < T_asym(n) = 40 + 6n; Gauss-Hermite asymptote beyond.' % INV_WIDTH)
    lines.append('// Max relative error of the double table vs 80-digit reference, per n:')
    for n in range(1, NMAX + 1):
        lines.append('//   n=%d: %.2e' % (n, worst[n]))
    lines.append('// FP32 table (degree %d, intervals of width %d): max relative interpolation error per n '
                 '(coefficients then rounded to float):' % (DEG_F, WIDTH_F))
    for n in range(1, NMAX + 1):
        lines.append('//   n=%d: %.2e' % (n, worst_f[n]))
    lines.append('#define RYS_NMAX %d' % NMAX)
    lines.append('#define RYS_DEG %d' % DEG)
    lines.append('#define RYS_INV_WIDTH %d' % INV_WIDTH)
    lines.append('#define RYS_DEG_F %d' % DEG_F)
    lines.append('#define RYS_WIDTH_F %d' % WIDTH_F)
    nint = [0] + [t_asym(n) * INV_WIDTH for n in range(1, NMAX + 1)]
    nint_f = [0] + [t_asym(n) // WIDTH_F for n in range(1, NMAX + 1)]
    # offs[n] = first element of the block for n roots (offs[0] unused)
    offs = [0, 0]
    for n in range(1, NMAX):
        offs.append(offs[-1] + nint[n] * (DEG + 1) * 2 * n)
    total = offs[-1] + nint[NMAX] * (DEG + 1) * 2 * NMAX
    lines.append('#define RYS_TABLE_SIZE %d' % total)
    lines.append('static const int rys_nint_host[RYS_NMAX + 1] = {%s};' % ', '.join(map(str, nint)))
    lines.append('static const int rys_offset_host[RYS_NMAX + 1] = {%s};' % ', '.join(map(str, offs)))
    lines.append('// layout per n: [interval][power 0..DEG][u_1..u_n, w_1..w_n]')
    lines.append('static const double rys_coef_host[RYS_TABLE_SIZE] = {')
    for n in range(1, NMAX + 1):
        for k in range(nint[n]):
            c = table[(n, k)]
            for i in range(DEG + 1):
                lines.append('  ' + ', '.join(float.hex(v) for v in c[i]) + ',')
    lines.append('};')
    offs_f = [0, 0]
    for n in range(1, NMAX):
        offs_f.append(offs_f[-1] + nint_f[n] * (DEG_F + 1) * 2 * n)
    total_f = offs_f[-1] + nint_f[NMAX] * (DEG_F + 1) * 2 * NMAX
    lines.append('#define RYS_TABLE_F_SIZE %d' % total_f)
    lines.append('static const int rys_nint_f_host[RYS_NMAX + 1] = {%s};' % ', '.join(map(str, nint_f)))
    lines.append('static const int rys_offset_f_host[RYS_NMAX + 1] = {%s};' % ', '.join(map(str, offs_f)))
    lines.append('// FP32 layout per n: [interval][power 0..DEG_F][u_1..u_n, w_1..w_n]')
    lines.append('static const float rys_coef_f_host[RYS_TABLE_F_SIZE] = {')
    for n in range(1, NMAX + 1):
        for k in range(nint_f[n]):
            c = table_f[(n, k)]
            for i in range(DEG_F + 1):
                lines.append('  ' + ', '.join('%.9ef' % v for v in c[i]) + ',')
    lines.append('};')
    hx, hw = [], []
    for n in range(1, NMAX + 1):
        x, W = hermite(mp, 2 * n)
        hx.extend(float(v * v) for v in x[n:])
        hw.extend(float(v) for v in W[n:])
    lines.append('// Gauss-Hermite asymptote per n (offset n(n-1)/2): squared positive nodes and weights')
    lines.append('#define RYS_ASYM_SIZE %d' % len(hx))
    lines.append('#define RYS_ASYM_X2_LIST %s' % ', '.join(float.hex(v) for v in hx))
    lines.append('#define RYS_ASYM_W_LIST %s' % ', '.join(float.hex(v) for v in hw))
    # FP32 copies for the FP32 asymptote (no conversion instruction, which
    # would run on the FP64 pipe)
    lines.append('#define RYS_ASYM_X2_LIST_F %s' % ', '.join('%.9ef' % v for v in hx))
    lines.append('#define RYS_ASYM_W_LIST_F %s' % ', '.join('%.9ef' % v for v in hw))
    lines.append('static const double rys_asym_x2_host[RYS_ASYM_SIZE] = {RYS_ASYM_X2_LIST};')
    lines.append('static const double rys_asym_w_host[RYS_ASYM_SIZE] = {RYS_ASYM_W_LIST};')
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'rys_tables.inc')
    with open(out, 'w') as f:
        f.write('\n'.join(lines) + '\n')
    print('wrote', out, 'max rel err', max(worst.values()), 'fp32 table', max(worst_f.values()))


if __name__ == '__main__':
    sys.exit(main())
