// CPU oracle for the direct-SCF J/K path.  TEST INFRASTRUCTURE ONLY: this
// library is loaded by tests/, by __graft_entry__.smoke() as the checker and
// by bench.py's CPU-baseline leg.  The product (gpu4pyscf_gb300) never links
// or calls it.
//
// It restates, with an algorithm independent of the GPU engine, what
// PySCF's CPU get_jk (libcvhf + libcint) computes for gpu4pyscf's tests
// (gpu4pyscf/scf/tests/test_scf_jk.py:22,45 use pyscf.scf.hf.get_jk as the
// oracle):
//   vj[k,l] = sum_ij (ij|kl) D[j,i]      vk[i,l] = sum_jk (ij|kl) D[j,k]
// Electron-repulsion integrals use the McMurchie-Davidson scheme (Hermite
// expansion + Boys-function R_tuv recursion), not Rys quadrature, so that the
// oracle and the GPU kernels disagree only through real bugs.
//
// Screening follows gpu4pyscf/lib/gvhf-rys/create_tasks.cu:152-162 and
// gpu4pyscf/scf/jk.py:510-516: a shell quartet (ij|kl) is skipped when
//   q[i,j] * q[k,l] * max(dmc[i,j], dmc[k,l], dmc[i,k], dmc[i,l], dmc[j,k], dmc[j,l]) < tol
// with q[i,j] = sqrt(max |(ij|ij)|) and dmc the per-shell-block absmax of the
// densities (symmetrised for hermi=0).  tol = 0 disables screening.
//
// Inputs use the libcint layout (atm[natm][6], bas[nbas][8], env) in the
// Cartesian AO basis of the given shells (nctr contractions per shell).
//
// Range separation follows libcint's convention (env[8] = omega, the slot
// PySCF's mol.omega writes; gpu4pyscf/scf/jk.py:1122-1168): omega > 0 gives
// the long-range operator erf(omega r)/r, omega < 0 the short-range
// erfc(|omega| r)/r.  Writing 1/r = 2/sqrt(pi) int_0^inf exp(-s^2 r^2) ds,
// the long-range operator stops the integral at s = omega; for a primitive
// quartet with reduced exponent a = pq/(p+q) this turns the Hermite
// integrals R_tuv(a) into sqrt(theta) R_tuv(theta a) with
// theta = omega^2 / (omega^2 + a).  Short range = full - long range.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int ATOM_OF = 0, ANG_OF = 1, NPRIM_OF = 2, NCTR_OF = 3, PTR_EXP = 5, PTR_COEFF = 6;
constexpr int CHARGE_OF = 0, PTR_COORD = 1;
constexpr int PTR_RANGE_OMEGA = 8;
constexpr int LMAX = 7;

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Boys function F_m(t), m = 0..mmax, written into f[].
// t small: Taylor; t <= 35: series for F_mmax then downward recursion;
// t > 35: erf closed form for F_0 then upward recursion (stable for t > mmax).
void boys(int mmax, double t, double *f) {
    if (t < 1e-14) {
        for (int m = 0; m <= mmax; ++m) f[m] = 1.0 / (2 * m + 1) - t / (2 * m + 3);
        return;
    }
    double et = std::exp(-t);
    if (t <= 35.0 || t < mmax + 10.0) {
        double term = 1.0 / (2 * mmax + 1);
        double sum = term;
        for (int k = 1; k < 2000; ++k) {
            term *= 2.0 * t / (2 * mmax + 2 * k + 1);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        f[mmax] = et * sum;
        for (int m = mmax - 1; m >= 0; --m) f[m] = (2.0 * t * f[m + 1] + et) / (2 * m + 1);
    } else {
        double st = std::sqrt(t);
        f[0] = 0.5 * std::sqrt(M_PI) / st * std::erf(st);
        for (int m = 0; m < mmax; ++m) f[m + 1] = ((2 * m + 1) * f[m] - et) / (2.0 * t);
    }
}

struct Shell {
    int l, nprim, nctr;
    const double *exps;
    const double *coef;  // [nctr][nprim]
    double r[3];
    int ao0;             // first Cartesian AO index
    int atom;
};

std::vector<Shell> make_shells(const int *atm, const int *bas, int nbas, const double *env, int *nao_out) {
    std::vector<Shell> sh(nbas);
    int off = 0;
    for (int i = 0; i < nbas; ++i) {
        const int *b = bas + i * 8;
        Shell &s = sh[i];
        s.l = b[ANG_OF];
        s.nprim = b[NPRIM_OF];
        s.nctr = b[NCTR_OF];
        s.exps = env + b[PTR_EXP];
        s.coef = env + b[PTR_COEFF];
        const double *r = env + atm[b[ATOM_OF] * 6 + PTR_COORD];
        s.r[0] = r[0]; s.r[1] = r[1]; s.r[2] = r[2];
        s.ao0 = off;
        s.atom = b[ATOM_OF];
        off += ncart(s.l) * s.nctr;
    }
    *nao_out = off;
    return sh;
}

void cart_comps(int l, std::vector<int> &lx, std::vector<int> &ly, std::vector<int> &lz) {
    lx.clear(); ly.clear(); lz.clear();
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) { lx.push_back(x); ly.push_back(y); lz.push_back(l - x - y); }
}

// Hermite expansion coefficients for one axis: E[i][j][t], i<=la, j<=lb, t<=i+j
struct Eaxis {
    int la, lb;
    std::vector<double> e;  // (la+1)*(lb+1)*(la+lb+1)
    double &at(int i, int j, int t) { return e[(i * (lb + 1) + j) * (la + lb + 1) + t]; }
    double get(int i, int j, int t) const {
        if (t < 0 || t > i + j) return 0.0;
        return e[(i * (lb + 1) + j) * (la + lb + 1) + t];
    }
    void build(int la_, int lb_, double p, double xpa, double xpb) {
        la = la_; lb = lb_;
        int nt = la + lb + 1;
        e.assign((la + 1) * (lb + 1) * nt, 0.0);
        double h = 0.5 / p;
        at(0, 0, 0) = 1.0;
        for (int i = 0; i <= la; ++i) {
            if (i > 0) {
                for (int t = 0; t <= i; ++t) {
                    double v = xpa * get(i - 1, 0, t) + (t + 1) * get(i - 1, 0, t + 1);
                    if (t > 0) v += h * get(i - 1, 0, t - 1);
                    at(i, 0, t) = v;
                }
            }
            for (int j = 1; j <= lb; ++j) {
                for (int t = 0; t <= i + j; ++t) {
                    double v = xpb * get(i, j - 1, t) + (t + 1) * get(i, j - 1, t + 1);
                    if (t > 0) v += h * get(i, j - 1, t - 1);
                    at(i, j, t) = v;
                }
            }
        }
    }
};

// Hermite Coulomb integrals R_{tuv}(alpha, XYZ) for t+u+v <= L, stored
// densely in r[(t*(L+1)+u)*(L+1)+v].
struct Rtab {
    int L;
    std::vector<double> cur, nxt;
    double at(int t, int u, int v) const { return cur[(t * (L + 1) + u) * (L + 1) + v]; }
    void build(int L_, double alpha, double X, double Y, double Z, double prefac) {
        L = L_;
        int n1 = L + 1;
        size_t sz = (size_t)n1 * n1 * n1;
        cur.assign(sz, 0.0);
        nxt.assign(sz, 0.0);
        double f[4 * LMAX + 2];
        double T = alpha * (X * X + Y * Y + Z * Z);
        boys(L, T, f);
        // level n = L
        double m2a = -2.0 * alpha;
        double pw = prefac;
        std::vector<double> r000(L + 1);
        for (int n = 0; n <= L; ++n) { r000[n] = pw * f[n]; pw *= m2a; }
        // start with level L: only R_000
        nxt[0] = r000[L];
        for (int n = L - 1; n >= 0; --n) {
            int lim = L - n;
            // build level n into cur from level n+1 in nxt
            for (int t = 0; t <= lim; ++t)
                for (int u = 0; u <= lim - t; ++u)
                    for (int v = 0; v <= lim - t - u; ++v) {
                        double val;
                        if (t > 0) {
                            val = X * nxt[((t - 1) * n1 + u) * n1 + v];
                            if (t > 1) val += (t - 1) * nxt[((t - 2) * n1 + u) * n1 + v];
                        } else if (u > 0) {
                            val = Y * nxt[(t * n1 + u - 1) * n1 + v];
                            if (u > 1) val += (u - 1) * nxt[(t * n1 + u - 2) * n1 + v];
                        } else if (v > 0) {
                            val = Z * nxt[(t * n1 + u) * n1 + v - 1];
                            if (v > 1) val += (v - 1) * nxt[(t * n1 + u) * n1 + v - 2];
                        } else {
                            val = r000[n];
                        }
                        cur[(t * n1 + u) * n1 + v] = val;
                    }
            std::swap(cur, nxt);
        }
        std::swap(cur, nxt);
        if (L == 0) cur[0] = r000[0];
    }
};

// Contracted Cartesian ERI block (ij|kl), layout
// out[(((ci*nctr_j + cj)*nctr_k + ck)*nctr_l + cl)][a][b][c][d]
// with a,b,c,d running over Cartesian components.
void eri_block(const Shell &si, const Shell &sj, const Shell &sk, const Shell &sl, std::vector<double> &out,
               double omega = 0.0) {
    int la = si.l, lb = sj.l, lc = sk.l, ld = sl.l;
    int na = ncart(la), nb = ncart(lb), nc = ncart(lc), nd = ncart(ld);
    int nabcd = na * nb * nc * nd;
    int nctr = si.nctr * sj.nctr * sk.nctr * sl.nctr;
    out.assign((size_t)nabcd * nctr, 0.0);
    std::vector<int> ax, ay, az, bx, by, bz, cx, cy, cz, dx, dy, dz;
    cart_comps(la, ax, ay, az); cart_comps(lb, bx, by, bz);
    cart_comps(lc, cx, cy, cz); cart_comps(ld, dx, dy, dz);
    int lab = la + lb, lcd = lc + ld, L = lab + lcd;
    double AB[3], CD[3];
    for (int x = 0; x < 3; ++x) { AB[x] = si.r[x] - sj.r[x]; CD[x] = sk.r[x] - sl.r[x]; }
    double rab2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    double rcd2 = CD[0] * CD[0] + CD[1] * CD[1] + CD[2] * CD[2];
    Eaxis Eab[3], Ecd[3];
    Rtab R, Rlr;
    int nh = lab + 1;  // bra Hermite index range per axis
    std::vector<double> W((size_t)nh * nh * nh);
    std::vector<double> prim(nabcd);
    for (int pa = 0; pa < si.nprim; ++pa)
    for (int pb = 0; pb < sj.nprim; ++pb) {
        double a = si.exps[pa], b = sj.exps[pb];
        double p = a + b;
        double Kab = std::exp(-a * b / p * rab2);
        double P[3];
        for (int x = 0; x < 3; ++x) P[x] = (a * si.r[x] + b * sj.r[x]) / p;
        for (int x = 0; x < 3; ++x) Eab[x].build(la, lb, p, P[x] - si.r[x], P[x] - sj.r[x]);
        for (int pc = 0; pc < sk.nprim; ++pc)
        for (int pd = 0; pd < sl.nprim; ++pd) {
            double c = sk.exps[pc], d = sl.exps[pd];
            double q = c + d;
            double Kcd = std::exp(-c * d / q * rcd2);
            double Q[3];
            for (int x = 0; x < 3; ++x) Q[x] = (c * sk.r[x] + d * sl.r[x]) / q;
            for (int x = 0; x < 3; ++x) Ecd[x].build(lc, ld, q, Q[x] - sk.r[x], Q[x] - sl.r[x]);
            double alpha = p * q / (p + q);
            double pref = 2.0 * std::pow(M_PI, 2.5) / (p * q * std::sqrt(p + q)) * Kab * Kcd;
            if (omega > 0) {
                double theta = omega * omega / (omega * omega + alpha);
                R.build(L, alpha * theta, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], pref * std::sqrt(theta));
            } else {
                R.build(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], pref);
                if (omega < 0) {
                    double theta = omega * omega / (omega * omega + alpha);
                    Rlr.build(L, alpha * theta, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], pref * std::sqrt(theta));
                    for (size_t e = 0; e < R.cur.size(); ++e) R.cur[e] -= Rlr.cur[e];
                }
            }
            for (int ic = 0; ic < nc; ++ic)
            for (int id = 0; id < nd; ++id) {
                // W_tuv = sum_{tau,nu,phi} (-1)^(tau+nu+phi) Ecd R_{t+tau,u+nu,v+phi}
                int mx = cx[ic] + dx[id], my = cy[ic] + dy[id], mz = cz[ic] + dz[id];
                for (int t = 0; t <= lab; ++t)
                for (int u = 0; u <= lab - t; ++u)
                for (int v = 0; v <= lab - t - u; ++v) {
                    double s = 0.0;
                    for (int tau = 0; tau <= mx; ++tau) {
                        double ex = Ecd[0].get(cx[ic], dx[id], tau);
                        if (ex == 0.0) continue;
                        for (int nu = 0; nu <= my; ++nu) {
                            double ey = Ecd[1].get(cy[ic], dy[id], nu);
                            if (ey == 0.0) continue;
                            double exy = ex * ey;
                            for (int phi = 0; phi <= mz; ++phi) {
                                double ez = Ecd[2].get(cz[ic], dz[id], phi);
                                double sg = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
                                s += sg * exy * ez * R.at(t + tau, u + nu, v + phi);
                            }
                        }
                    }
                    W[(t * nh + u) * nh + v] = s;
                }
                for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib) {
                    int mxa = ax[ia] + bx[ib], mya = ay[ia] + by[ib], mza = az[ia] + bz[ib];
                    double s = 0.0;
                    for (int t = 0; t <= mxa; ++t) {
                        double ex = Eab[0].get(ax[ia], bx[ib], t);
                        for (int u = 0; u <= mya; ++u) {
                            double exy = ex * Eab[1].get(ay[ia], by[ib], u);
                            for (int v = 0; v <= mza; ++v)
                                s += exy * Eab[2].get(az[ia], bz[ib], v) * W[(t * nh + u) * nh + v];
                        }
                    }
                    prim[((ia * nb + ib) * nc + ic) * nd + id] = s;
                }
            }
            // contract
            for (int ci = 0; ci < si.nctr; ++ci)
            for (int cj = 0; cj < sj.nctr; ++cj)
            for (int ck = 0; ck < sk.nctr; ++ck)
            for (int cl = 0; cl < sl.nctr; ++cl) {
                double cc = si.coef[ci * si.nprim + pa] * sj.coef[cj * sj.nprim + pb]
                          * sk.coef[ck * sk.nprim + pc] * sl.coef[cl * sl.nprim + pd];
                if (cc == 0.0) continue;
                double *o = out.data() + (size_t)(((ci * sj.nctr + cj) * sk.nctr + ck) * sl.nctr + cl) * nabcd;
                for (int e = 0; e < nabcd; ++e) o[e] += cc * prim[e];
            }
        }
    }
}

int nthreads_of(int req) {
#ifdef _OPENMP
    return req > 0 ? req : omp_get_max_threads();
#else
    (void)req;
    return 1;
#endif
}

// AO index of (shell, contraction, component)
inline int aoidx(const Shell &s, int ctr, int comp) { return s.ao0 + ctr * ncart(s.l) + comp; }

}  // namespace

extern "C" {

// Boys function values F_0..F_mmax at t.
void oracle_boys(int mmax, double t, double *out) { boys(mmax, t, out); }

// Full Cartesian ERI tensor eri[nao^4] (small systems only).
int oracle_eri_full(const int *atm, int natm, const int *bas, int nbas, const double *env, double *eri) {
    (void)natm;
    int nao;
    auto sh = make_shells(atm, bas, nbas, env, &nao);
    std::vector<double> blk;
    size_t n = nao;
    for (int i = 0; i < nbas; ++i)
    for (int j = 0; j < nbas; ++j)
    for (int k = 0; k < nbas; ++k)
    for (int l = 0; l < nbas; ++l) {
        eri_block(sh[i], sh[j], sh[k], sh[l], blk, env[PTR_RANGE_OMEGA]);
        int na = ncart(sh[i].l), nb = ncart(sh[j].l), nc = ncart(sh[k].l), nd = ncart(sh[l].l);
        for (int ci = 0; ci < sh[i].nctr; ++ci)
        for (int cj = 0; cj < sh[j].nctr; ++cj)
        for (int ck = 0; ck < sh[k].nctr; ++ck)
        for (int cl = 0; cl < sh[l].nctr; ++cl) {
            const double *o = blk.data() + (size_t)(((ci * sh[j].nctr + cj) * sh[k].nctr + ck) * sh[l].nctr + cl) * na * nb * nc * nd;
            for (int a = 0; a < na; ++a)
            for (int b = 0; b < nb; ++b)
            for (int c = 0; c < nc; ++c)
            for (int d = 0; d < nd; ++d) {
                size_t I = aoidx(sh[i], ci, a), J = aoidx(sh[j], cj, b), K = aoidx(sh[k], ck, c), L = aoidx(sh[l], cl, d);
                eri[((I * n + J) * n + K) * n + L] = o[((a * nb + b) * nc + c) * nd + d];
            }
        }
    }
    return 0;
}

// Schwarz factors q[i*nbas+j] = sqrt(max |(ij|ij)|) over all components.
int oracle_qcond(const int *atm, int natm, const int *bas, int nbas, const double *env, double *q, int nthreads) {
    (void)natm;
    int nao;
    auto sh = make_shells(atm, bas, nbas, env, &nao);
    int nt = nthreads_of(nthreads);
#pragma omp parallel for schedule(dynamic) num_threads(nt)
    for (int ij = 0; ij < nbas * nbas; ++ij) {
        int i = ij / nbas, j = ij % nbas;
        if (j > i) continue;
        std::vector<double> blk;
        eri_block(sh[i], sh[j], sh[i], sh[j], blk, env[PTR_RANGE_OMEGA]);
        int na = ncart(sh[i].l) , nb = ncart(sh[j].l);
        int nctr = sh[i].nctr * sh[j].nctr;
        double m = 0.0;
        for (int c1 = 0; c1 < sh[i].nctr; ++c1)
        for (int c2 = 0; c2 < sh[j].nctr; ++c2) {
            const double *o = blk.data() + (size_t)(((c1 * sh[j].nctr + c2) * sh[i].nctr + c1) * sh[j].nctr + c2) * na * nb * na * nb;
            for (int a = 0; a < na; ++a)
            for (int b = 0; b < nb; ++b)
                m = std::max(m, std::fabs(o[((a * nb + b) * na + a) * nb + b]));
        }
        (void)nctr;
        q[i * nbas + j] = q[j * nbas + i] = std::sqrt(m);
    }
    return 0;
}

// J/K for n_dm Cartesian densities dm[n_dm][nao][nao].
// hermi: 0 general, 1 symmetric, 2 antisymmetric (J set to zero).
// stats (optional, int64[4]): quartets computed, quartets screened out,
// primitive quartets computed, shell pairs.
// bra_stride: if >1, only bra shell pairs whose index i*(i+1)/2+j is a
// multiple of it are computed (a representative bounded sample for timing).
int oracle_jk(const int *atm, int natm, const int *bas, int nbas, const double *env,
              const double *dm, int n_dm, int hermi, double tol, int with_j, int with_k,
              double *vj, double *vk, int nthreads, long long bra_stride, long long *stats) {
    (void)natm;
    int nao;
    auto sh = make_shells(atm, bas, nbas, env, &nao);
    size_t nn = (size_t)nao * nao;
    std::vector<double> q((size_t)nbas * nbas, 1.0);
    std::vector<double> dmc((size_t)nbas * nbas, 1.0);
    if (tol > 0) {
        oracle_qcond(atm, natm, bas, nbas, env, q.data(), nthreads);
        for (int i = 0; i < nbas; ++i)
        for (int j = 0; j < nbas; ++j) {
            double m = 0.0;
            int ni = ncart(sh[i].l) * sh[i].nctr, nj = ncart(sh[j].l) * sh[j].nctr;
            for (int d = 0; d < n_dm; ++d)
            for (int a = 0; a < ni; ++a)
            for (int b = 0; b < nj; ++b)
                m = std::max(m, std::fabs(dm[d * nn + (size_t)(sh[i].ao0 + a) * nao + sh[j].ao0 + b]));
            dmc[i * nbas + j] = m;
        }
        if (hermi == 0) {
            std::vector<double> t(dmc);
            for (int i = 0; i < nbas; ++i)
            for (int j = 0; j < nbas; ++j) dmc[i * nbas + j] = t[i * nbas + j] + t[j * nbas + i];
        }
    }
    int nt = nthreads_of(nthreads);
    std::vector<std::vector<double>> jbuf(nt), kbuf(nt);
    long long n_comp = 0, n_skip = 0, n_prim = 0;
    long long npair = (long long)nbas * (nbas + 1) / 2;
    long long stride = bra_stride > 1 ? bra_stride : 1;
    long long plimit = (npair + stride - 1) / stride;
#pragma omp parallel num_threads(nt) reduction(+:n_comp, n_skip, n_prim)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        std::vector<double> &J = jbuf[tid];
        std::vector<double> &K = kbuf[tid];
        if (with_j) J.assign(nn * n_dm, 0.0);
        if (with_k) K.assign(nn * n_dm, 0.0);
        std::vector<double> blk;
#pragma omp for schedule(dynamic)
        for (long long ijs = 0; ijs < plimit; ++ijs) {
            long long ij = ijs * stride;
            int i = (int)((std::sqrt(8.0 * ij + 1) - 1) / 2);
            while ((long long)i * (i + 1) / 2 > ij) --i;
            while ((long long)(i + 1) * (i + 2) / 2 <= ij) ++i;
            int j = (int)(ij - (long long)i * (i + 1) / 2);
            for (int k = 0; k <= i; ++k) {
                int lmax = (k == i) ? j : k;
                for (int l = 0; l <= lmax; ++l) {
                    if (tol > 0) {
                        double dmax = std::max({dmc[i * nbas + j], dmc[k * nbas + l], dmc[i * nbas + k],
                                                dmc[i * nbas + l], dmc[j * nbas + k], dmc[j * nbas + l]});
                        if (q[i * nbas + j] * q[k * nbas + l] * dmax < tol) { ++n_skip; continue; }
                    }
                    ++n_comp;
                    n_prim += (long long)sh[i].nprim * sh[j].nprim * sh[k].nprim * sh[l].nprim;
                    eri_block(sh[i], sh[j], sh[k], sh[l], blk, env[PTR_RANGE_OMEGA]);
                    double fac = 1.0;
                    if (i == j) fac *= 0.5;
                    if (k == l) fac *= 0.5;
                    if (i == k && j == l) fac *= 0.5;
                    const Shell *S[4] = {&sh[i], &sh[j], &sh[k], &sh[l]};
                    int nf[4] = {ncart(sh[i].l), ncart(sh[j].l), ncart(sh[k].l), ncart(sh[l].l)};
                    int nab = nf[0] * nf[1] * nf[2] * nf[3];
                    for (int ci = 0; ci < S[0]->nctr; ++ci)
                    for (int cj = 0; cj < S[1]->nctr; ++cj)
                    for (int ck = 0; ck < S[2]->nctr; ++ck)
                    for (int cl = 0; cl < S[3]->nctr; ++cl) {
                        const double *o = blk.data() + (size_t)(((ci * S[1]->nctr + cj) * S[2]->nctr + ck) * S[3]->nctr + cl) * nab;
                        for (int a = 0; a < nf[0]; ++a)
                        for (int b = 0; b < nf[1]; ++b)
                        for (int c = 0; c < nf[2]; ++c)
                        for (int d = 0; d < nf[3]; ++d) {
                            double e = fac * o[((a * nf[1] + b) * nf[2] + c) * nf[3] + d];
                            size_t I = aoidx(*S[0], ci, a), Jx = aoidx(*S[1], cj, b);
                            size_t Kx = aoidx(*S[2], ck, c), Lx = aoidx(*S[3], cl, d);
                            // the 8 index permutations (pq|rs) of this element
                            size_t perm[8][4] = {{I, Jx, Kx, Lx}, {Jx, I, Kx, Lx}, {I, Jx, Lx, Kx}, {Jx, I, Lx, Kx},
                                                 {Kx, Lx, I, Jx}, {Lx, Kx, I, Jx}, {Kx, Lx, Jx, I}, {Lx, Kx, Jx, I}};
                            for (int dd = 0; dd < n_dm; ++dd) {
                                const double *D = dm + dd * nn;
                                for (int pp = 0; pp < 8; ++pp) {
                                    size_t P = perm[pp][0], Q = perm[pp][1], Rr = perm[pp][2], Ss = perm[pp][3];
                                    // vj[r,s] += (pq|rs) D[q,p];  vk[p,s] += (pq|rs) D[q,r]
                                    if (with_j) J[dd * nn + Rr * nao + Ss] += e * D[Q * nao + P];
                                    if (with_k) K[dd * nn + P * nao + Ss] += e * D[Q * nao + Rr];
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    if (with_j) {
        std::memset(vj, 0, sizeof(double) * nn * n_dm);
        for (int t = 0; t < nt; ++t)
            if (!jbuf[t].empty())
                for (size_t x = 0; x < nn * n_dm; ++x) vj[x] += jbuf[t][x];
        if (hermi == 2) std::memset(vj, 0, sizeof(double) * nn * n_dm);
    }
    if (with_k) {
        std::memset(vk, 0, sizeof(double) * nn * n_dm);
        for (int t = 0; t < nt; ++t)
            if (!kbuf[t].empty())
                for (size_t x = 0; x < nn * n_dm; ++x) vk[x] += kbuf[t][x];
    }
    if (stats) { stats[0] = n_comp; stats[1] = n_skip; stats[2] = n_prim; stats[3] = npair; }
    return 0;
}

// Nuclear gradient of the two-electron energy of one symmetric density D
// (Cartesian AO basis of the shells) at fixed D,
//   E = j_factor/2 sum (ij|kl) D_ji D_lk - k_factor/4 sum (ij|kl) D_jk D_li,
// grad[A*3+x] = dE/dR_Ax.  This is what gpu4pyscf's RYS_per_atom_jk_ip1
// returns for an RHF density (gpu4pyscf/lib/gvhf-rys/rys_contract_jk_ip1.cu:
// 1747-1797, called by _jk_energy_per_atom, gpu4pyscf/grad/rhf.py:60-171;
// its own check is gpu4pyscf/scf/tests/test_scf_jk.py:388-413).
// With D symmetric the four centres of a quartet contribute alike, so
//   dE/dR_A = -4 sum_{i on A} sum_jkl (d/dr_i i j|kl) G_ijkl,
//   G_ijkl = j_factor/2 D_ji D_lk - k_factor/4 D_jk D_li,
// and the derivative of a Cartesian primitive x^a exp(-alpha r^2) along x is
// a x^(a-1) exp(..) - 2 alpha x^(a+1) exp(..): the ERIs of the shell raised
// by one (coefficients times 2 alpha) and lowered by one.  No screening.
int oracle_jk_grad(const int *atm, int natm, const int *bas, int nbas, const double *env,
                   const double *dm, double j_factor, double k_factor, double *grad, int nthreads) {
    int nao;
    auto sh = make_shells(atm, bas, nbas, env, &nao);
    const double omega = env[PTR_RANGE_OMEGA];
    for (int i = 0; i < natm * 3; ++i) grad[i] = 0.;
    int nt = nthreads_of(nthreads);
    std::vector<std::vector<double>> gbuf(nt, std::vector<double>((size_t)natm * 3, 0.));
#pragma omp parallel for schedule(dynamic) num_threads(nt)
    for (int ish = 0; ish < nbas; ++ish) {
#ifdef _OPENMP
        std::vector<double> &g = gbuf[omp_get_thread_num()];
#else
        std::vector<double> &g = gbuf[0];
#endif
        const Shell &I = sh[ish];
        // raised (coefficients x 2 alpha) and lowered copies of shell I
        std::vector<double> cplus((size_t)I.nctr * I.nprim);
        for (int c = 0; c < I.nctr; ++c)
            for (int p = 0; p < I.nprim; ++p) cplus[c * I.nprim + p] = I.coef[c * I.nprim + p] * 2. * I.exps[p];
        Shell Ip = I, Im = I;
        Ip.l = I.l + 1;
        Ip.coef = cplus.data();
        Im.l = I.l - 1;
        std::vector<int> ax, ay, az, px, py, pz, mx, my, mz;
        cart_comps(I.l, ax, ay, az);
        cart_comps(Ip.l, px, py, pz);
        if (I.l > 0) cart_comps(Im.l, mx, my, mz);
        auto find = [](const std::vector<int> &X, const std::vector<int> &Y, const std::vector<int> &Z,
                       int x, int y, int z) {
            for (size_t c = 0; c < X.size(); ++c)
                if (X[c] == x && Y[c] == y && Z[c] == z) return (int)c;
            return -1;
        };
        const int nfi = ncart(I.l), nfp = ncart(Ip.l), nfm = I.l > 0 ? ncart(Im.l) : 0;
        std::vector<double> bp, bm;
        for (int jsh = 0; jsh < nbas; ++jsh)
        for (int ksh = 0; ksh < nbas; ++ksh)
        for (int lsh = 0; lsh < nbas; ++lsh) {
            const Shell &J = sh[jsh], &K = sh[ksh], &L = sh[lsh];
            eri_block(Ip, J, K, L, bp, omega);
            if (I.l > 0) eri_block(Im, J, K, L, bm, omega);
            const int nfj = ncart(J.l), nfk = ncart(K.l), nfl = ncart(L.l);
            const int nrest = nfj * nfk * nfl;
            for (int ci = 0; ci < I.nctr; ++ci)
            for (int cj = 0; cj < J.nctr; ++cj)
            for (int ck = 0; ck < K.nctr; ++ck)
            for (int cl = 0; cl < L.nctr; ++cl) {
                const size_t cidx = ((ci * J.nctr + cj) * K.nctr + ck) * L.nctr + cl;
                const double *op = bp.data() + cidx * (size_t)nfp * nrest;
                const double *om = I.l > 0 ? bm.data() + cidx * (size_t)nfm * nrest : nullptr;
                for (int a = 0; a < nfi; ++a) {
                    const size_t Ia = aoidx(I, ci, a);
                    for (int x = 0; x < 3; ++x) {
                        const int d[3] = {x == 0, x == 1, x == 2};
                        const int up = find(px, py, pz, ax[a] + d[0], ay[a] + d[1], az[a] + d[2]);
                        const int na = x == 0 ? ax[a] : (x == 1 ? ay[a] : az[a]);
                        const int dn = na > 0 ? find(mx, my, mz, ax[a] - d[0], ay[a] - d[1], az[a] - d[2]) : -1;
                        double s = 0.;
                        for (int b = 0; b < nfj; ++b)
                        for (int c = 0; c < nfk; ++c)
                        for (int e = 0; e < nfl; ++e) {
                            const int r = (b * nfk + c) * nfl + e;
                            // d/dr of the bra function: a_x (a-1) - 2 alpha (a+1)
                            double deri = -op[(size_t)up * nrest + r];
                            if (dn >= 0) deri += na * om[(size_t)dn * nrest + r];
                            const size_t Jb = aoidx(J, cj, b), Kc = aoidx(K, ck, c), Le = aoidx(L, cl, e);
                            const double G = .5 * j_factor * dm[Jb * nao + Ia] * dm[Le * nao + Kc]
                                           - .25 * k_factor * dm[Jb * nao + Kc] * dm[Le * nao + Ia];
                            s += deri * G;
                        }
                        g[I.atom * 3 + x] -= 4. * s;
                    }
                }
            }
        }
    }
    for (int t = 0; t < nt; ++t)
        for (int i = 0; i < natm * 3; ++i) grad[i] += gbuf[t][i];
    return 0;
}

// One-electron Cartesian integrals: kind 0 overlap, 1 kinetic, 2 nuclear
// attraction (point charges of all atoms).
int oracle_int1e(const int *atm, int natm, const int *bas, int nbas, const double *env, int kind, double *out) {
    int nao;
    auto sh = make_shells(atm, bas, nbas, env, &nao);
    std::memset(out, 0, sizeof(double) * nao * nao);
#pragma omp parallel for schedule(dynamic)
    for (int ij = 0; ij < nbas * nbas; ++ij) {
        int i = ij / nbas, j = ij % nbas;
        const Shell &A = sh[i], &B = sh[j];
        std::vector<int> ax, ay, az, bx, by, bz;
        cart_comps(A.l, ax, ay, az);
        cart_comps(B.l, bx, by, bz);
        int na = ncart(A.l), nb = ncart(B.l);
        Eaxis E[3];
        Rtab R;
        double AB[3];
        for (int x = 0; x < 3; ++x) AB[x] = A.r[x] - B.r[x];
        double rab2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
        std::vector<double> prim(na * nb);
        for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = A.exps[pa], b = B.exps[pb], p = a + b;
            double K = std::exp(-a * b / p * rab2);
            double P[3];
            for (int x = 0; x < 3; ++x) P[x] = (a * A.r[x] + b * B.r[x]) / p;
            // kinetic needs lb+2
            int lbx = (kind == 1) ? B.l + 2 : B.l;
            for (int x = 0; x < 3; ++x) E[x].build(A.l, lbx, p, P[x] - A.r[x], P[x] - B.r[x]);
            double s0 = std::pow(M_PI / p, 1.5) * K;
            if (kind == 0) {
                for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib)
                    prim[ia * nb + ib] = s0 * E[0].get(ax[ia], bx[ib], 0) * E[1].get(ay[ia], by[ib], 0) * E[2].get(az[ia], bz[ib], 0);
            } else if (kind == 1) {
                // T = -1/2 <a|nabla^2|b>, d^2/dx^2 acting on x^l e^{-b x^2}:
                // l(l-1) x^{l-2} - 2b(2l+1) x^l + 4b^2 x^{l+2}
                for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib) {
                    int la3[3] = {ax[ia], ay[ia], az[ia]}, lb3[3] = {bx[ib], by[ib], bz[ib]};
                    double S1[3], D2[3];
                    for (int x = 0; x < 3; ++x) {
                        int l1 = la3[x], l2 = lb3[x];
                        S1[x] = E[x].get(l1, l2, 0);
                        double d = -2.0 * b * (2 * l2 + 1) * E[x].get(l1, l2, 0) + 4.0 * b * b * E[x].get(l1, l2 + 2, 0);
                        if (l2 >= 2) d += l2 * (l2 - 1) * E[x].get(l1, l2 - 2, 0);
                        D2[x] = d;
                    }
                    double t = D2[0] * S1[1] * S1[2] + S1[0] * D2[1] * S1[2] + S1[0] * S1[1] * D2[2];
                    prim[ia * nb + ib] = -0.5 * s0 * t;
                }
            } else {
                std::fill(prim.begin(), prim.end(), 0.0);
                int L = A.l + B.l;
                for (int c = 0; c < natm; ++c) {
                    const double *C = env + atm[c * 6 + PTR_COORD];
                    double Z = atm[c * 6 + CHARGE_OF];
                    R.build(L, p, P[0] - C[0], P[1] - C[1], P[2] - C[2], -Z * 2.0 * M_PI / p * K);
                    for (int ia = 0; ia < na; ++ia)
                    for (int ib = 0; ib < nb; ++ib) {
                        double s = 0.0;
                        for (int t = 0; t <= ax[ia] + bx[ib]; ++t)
                        for (int u = 0; u <= ay[ia] + by[ib]; ++u)
                        for (int v = 0; v <= az[ia] + bz[ib]; ++v)
                            s += E[0].get(ax[ia], bx[ib], t) * E[1].get(ay[ia], by[ib], u) * E[2].get(az[ia], bz[ib], v) * R.at(t, u, v);
                        prim[ia * nb + ib] += s;
                    }
                }
            }
            for (int ci = 0; ci < A.nctr; ++ci)
            for (int cj = 0; cj < B.nctr; ++cj) {
                double cc = A.coef[ci * A.nprim + pa] * B.coef[cj * B.nprim + pb];
                for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib)
                    out[(size_t)aoidx(A, ci, ia) * nao + aoidx(B, cj, ib)] += cc * prim[ia * nb + ib];
            }
        }
    }
    return 0;
}

}  // extern "C"
