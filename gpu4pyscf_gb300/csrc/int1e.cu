// One-electron integrals for the SCF driver: overlap, kinetic energy and
// nuclear attraction over the raw Cartesian functions of a sorted basis
// (the role of mol.intor('int1e_ovlp'/'int1e_kin'/'int1e_nuc') that
// gpu4pyscf's get_hcore / get_ovlp use, gpu4pyscf/scf/hf.py:138-155).
//
// One thread per (shell pair i >= j, Cartesian component a of i, b of j):
// overlap and kinetic from one-dimensional Obara-Saika recurrences, nuclear
// attraction by Rys quadrature over every nucleus (same root tables as the
// J/K kernels).  Not on the hot path: it runs once per SCF.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gb300jk.h"
#include "rys_roots.cuh"

namespace {

thread_local std::string g_err1e;

struct Sh1 { double x, y, z; int l, nprim, p0, ao; };

__device__ __forceinline__ void comp_xyz(int l, int c, int &x, int &y, int &z) {
    int idx = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            if (idx == c) { x = lx; y = ly; z = l - lx - ly; return; }
            ++idx;
        }
    x = y = z = 0;
}

constexpr int L1MAX = 3;

// 1D overlap table s[i][j], i <= la, j <= lb (lb up to la+... kinetic needs +2)
__device__ void ovlp1d(int la, int lb, double pa, double pb, double h, double s[L1MAX + 1][L1MAX + 3]) {
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) {
            double v;
            if (i == 0 && j == 0) v = 1.0;
            else if (i > 0) {
                v = pa * s[i - 1][j];
                if (i > 1) v += h * (i - 1) * s[i - 2][j];
                if (j > 0) v += h * j * s[i - 1][j - 1];
            } else {
                v = pb * s[i][j - 1];
                if (j > 1) v += h * (j - 1) * s[i][j - 2];
            }
            s[i][j] = v;
        }
}

template <int NR>
__device__ void nuc_roots(double T, const double *coef, double *u, double *w) {
    jk::rys_roots<NR>(T, coef, u, w);
}

__device__ void roots_n(int n, double T, const double *coef, double *u, double *w) {
    switch (n) {
        case 1: nuc_roots<1>(T, coef, u, w); break;
        case 2: nuc_roots<2>(T, coef, u, w); break;
        case 3: nuc_roots<3>(T, coef, u, w); break;
        default: nuc_roots<4>(T, coef, u, w); break;
    }
}

// 1D Rys integral for nuclear attraction: vertical up to la+lb, then transfer
__device__ double rys1d(int ia, int ib, double c00, double b10, double ab) {
    double v[2 * L1MAX + 1];
    int n = ia + ib;
    v[0] = 1.0;
    if (n > 0) v[1] = c00;
    for (int k = 1; k < n; ++k) v[k + 1] = c00 * v[k] + k * b10 * v[k - 1];
    // I(i, j+1) = I(i+1, j) + ab I(i, j), applied ib times
    for (int j = 0; j < ib; ++j)
        for (int i = 0; i < n - j; ++i) v[i] = v[i + 1] + ab * v[i];
    return v[ia];
}

__global__ void int1e_kernel(const Sh1 *sh, int nbas, const int2 *pairs, int npairs, const int *pair_off,
                             const double *exps, const double *coefs, const double4 *nuc, int natm,
                             const double *rys_coef, int nao, double *S, double *Tk, double *V) {
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    // binary search of the pair owning this element
    int total = pair_off[npairs];
    if (gid >= total) return;
    int lo = 0, hi = npairs;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (pair_off[mid] <= gid) lo = mid; else hi = mid;
    }
    int2 pr = pairs[lo];
    const Sh1 &A = sh[pr.x], &B = sh[pr.y];
    int nfb = (B.l + 1) * (B.l + 2) / 2;
    int e = gid - pair_off[lo];
    int ca = e / nfb, cb = e % nfb;
    int a3[3], b3[3];
    comp_xyz(A.l, ca, a3[0], a3[1], a3[2]);
    comp_xyz(B.l, cb, b3[0], b3[1], b3[2]);
    double Ac[3] = {A.x, A.y, A.z}, Bc[3] = {B.x, B.y, B.z};
    double AB2 = 0.;
    for (int x = 0; x < 3; ++x) AB2 += (Ac[x] - Bc[x]) * (Ac[x] - Bc[x]);
    double sval = 0., tval = 0., vval = 0.;
    int nroot = (A.l + B.l) / 2 + 1;
    for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = exps[A.p0 + pa], b = exps[B.p0 + pb];
            double cc = coefs[A.p0 + pa] * coefs[B.p0 + pb];
            double p = a + b, ip = 1.0 / p;
            double K = exp(-a * b * ip * AB2) * cc;
            double P[3], PA[3], PB[3];
            for (int x = 0; x < 3; ++x) {
                P[x] = (a * Ac[x] + b * Bc[x]) * ip;
                PA[x] = P[x] - Ac[x];
                PB[x] = P[x] - Bc[x];
            }
            double s1[3][L1MAX + 1][L1MAX + 3];
            double S1[3], D2[3];
            for (int x = 0; x < 3; ++x) {
                ovlp1d(a3[x], b3[x] + 2, PA[x], PB[x], 0.5 * ip, s1[x]);
                int l1 = a3[x], l2 = b3[x];
                S1[x] = s1[x][l1][l2];
                double d = -2.0 * b * (2 * l2 + 1) * s1[x][l1][l2] + 4.0 * b * b * s1[x][l1][l2 + 2];
                if (l2 >= 2) d += l2 * (l2 - 1) * s1[x][l1][l2 - 2];
                D2[x] = d;
            }
            double s0 = K * ip * sqrt(ip) * 5.5683279968317078453;  // pi^(3/2) p^(-3/2) K
            sval += s0 * S1[0] * S1[1] * S1[2];
            tval += -0.5 * s0 * (D2[0] * S1[1] * S1[2] + S1[0] * D2[1] * S1[2] + S1[0] * S1[1] * D2[2]);
            double vp = 0.;
            for (int c = 0; c < natm; ++c) {
                double4 C = nuc[c];
                double PC[3] = {P[0] - C.x, P[1] - C.y, P[2] - C.z};
                double T = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
                double u[4], w[4];
                roots_n(nroot, T, rys_coef, u, w);
                double acc = 0.;
                for (int r = 0; r < nroot; ++r) {
                    double b10 = 0.5 * ip * (1.0 - u[r]);
                    double prod = w[r];
                    for (int x = 0; x < 3; ++x)
                        prod *= rys1d(a3[x], b3[x], PA[x] - u[r] * PC[x], b10, Ac[x] - Bc[x]);
                    acc += prod;
                }
                vp -= C.w * acc;
            }
            vval += 2.0 * M_PI * ip * K * vp;
        }
    size_t i = A.ao + ca, j = B.ao + cb;
    S[i * nao + j] = sval; S[j * nao + i] = sval;
    Tk[i * nao + j] = tval; Tk[j * nao + i] = tval;
    V[i * nao + j] = vval; V[j * nao + i] = vval;
}

template <typename T>
cudaError_t up(T **d, const std::vector<T> &h) {
    cudaError_t e = cudaMalloc((void **)d, sizeof(T) * (h.empty() ? 1 : h.size()));
    if (e != cudaSuccess) return e;
    if (!h.empty()) e = cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return e;
}

}  // namespace

extern "C" const char *jk_int1e_last_error(void) { return g_err1e.c_str(); }

extern "C" int jk_int1e(const int32_t *atm, int natm, const int32_t *bas, int nbas, const double *env, int nenv,
                        double *S, double *T, double *V, void *stream) {
    if (!atm || !bas || !env || !S || !T || !V || natm <= 0 || nbas <= 0) { g_err1e = "invalid arguments"; return JK_ERR_ARG; }
    std::vector<Sh1> sh;
    std::vector<double> exps, coefs;
    int ao = 0;
    for (int i = 0; i < nbas; ++i) {
        const int32_t *b = bas + 8 * i;
        int ia = b[0], l = b[1], np = b[2], pe = b[5], pc = b[6];
        if (ia < 0 || ia >= natm || l < 0 || l > L1MAX || b[3] != 1 || np <= 0 || pe < 0 || pc < 0 ||
            pe + np > nenv || pc + np > nenv) {
            g_err1e = "invalid shell (sorted basis with l <= 3 and one contraction per shell expected)";
            return JK_ERR_ARG;
        }
        int pcd = atm[6 * ia + 1];
        if (pcd < 0 || pcd + 3 > nenv) { g_err1e = "bad coordinate pointer"; return JK_ERR_ARG; }
        Sh1 s{env[pcd], env[pcd + 1], env[pcd + 2], l, np, (int)exps.size(), ao};
        for (int p = 0; p < np; ++p) { exps.push_back(env[pe + p]); coefs.push_back(env[pc + p]); }
        sh.push_back(s);
        ao += (l + 1) * (l + 2) / 2;
    }
    std::vector<double4> nuc;
    for (int c = 0; c < natm; ++c) {
        int pcd = atm[6 * c + 1];
        if (pcd < 0 || pcd + 3 > nenv) { g_err1e = "bad coordinate pointer"; return JK_ERR_ARG; }
        nuc.push_back(make_double4(env[pcd], env[pcd + 1], env[pcd + 2], (double)atm[6 * c]));
    }
    std::vector<int2> pairs;
    std::vector<int> off{0};
    for (int i = 0; i < nbas; ++i)
        for (int j = 0; j <= i; ++j) {
            pairs.push_back(make_int2(i, j));
            off.push_back(off.back() + (sh[i].l + 1) * (sh[i].l + 2) / 2 * (sh[j].l + 1) * (sh[j].l + 2) / 2);
        }
    std::vector<double> tab(rys_coef_host, rys_coef_host + RYS_TABLE_SIZE);
    Sh1 *dsh = nullptr; int2 *dpairs = nullptr; int *doff = nullptr;
    double *dexp = nullptr, *dcoef = nullptr, *dtab = nullptr; double4 *dnuc = nullptr;
    cudaError_t e = up(&dsh, sh);
    if (e == cudaSuccess) e = up(&dpairs, pairs);
    if (e == cudaSuccess) e = up(&doff, off);
    if (e == cudaSuccess) e = up(&dexp, exps);
    if (e == cudaSuccess) e = up(&dcoef, coefs);
    if (e == cudaSuccess) e = up(&dtab, tab);
    if (e == cudaSuccess) e = up(&dnuc, nuc);
    cudaStream_t st = (cudaStream_t)stream;
    if (e == cudaSuccess) {
        int total = off.back();
        int1e_kernel<<<(total + 127) / 128, 128, 0, st>>>(dsh, nbas, dpairs, (int)pairs.size(), doff, dexp, dcoef,
                                                           dnuc, natm, dtab, ao, S, T, V);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(dsh); cudaFree(dpairs); cudaFree(doff); cudaFree(dexp); cudaFree(dcoef); cudaFree(dtab); cudaFree(dnuc);
    if (e != cudaSuccess) { g_err1e = std::string("jk_int1e: ") + cudaGetErrorString(e); return JK_ERR_CUDA; }
    return 0;
}
