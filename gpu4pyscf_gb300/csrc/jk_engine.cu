// Host driver of the GB300 J/K engine: the C ABI of include/gb300jk.h.
//
//   jk_opt_create: shell and primitive-pair data, Schwarz factors on the GPU
//     (diagonal quartets through the same class kernels), pruning and sorting
//     of the shell pairs of every (li, lj) class by Schwarz factor, planning
//     buffers.  Follows what gpu4pyscf's _VHFOpt.build and
//     _cache_q_cond_and_non0pairs prepare (gpu4pyscf/scf/jk.py:423-442,
//     984-1120), in this engine's own layout.
//   jk_build: densities -> screening table -> per-class work ranges (all on
//     the device, no host synchronisation) -> one launch per angular class
//     and precision -> symmetrisation into the caller's buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/gb300jk.h"
#include "jk_device.cuh"
#include "jk_registry.h"
#include "rys_tables.inc"

using namespace jk;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(JK_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

ClassEntry g_tab[NQCLASS];
std::once_flag g_tab_once;

void init_registry() {
    std::memset(g_tab, 0, sizeof(g_tab));
    register_bra_class_0(g_tab);
    register_bra_class_1(g_tab);
    register_bra_class_2(g_tab);
    register_bra_class_3(g_tab);
    register_bra_class_4(g_tab);
    register_bra_class_5(g_tab);
    register_bra_class_6(g_tab);
    register_bra_class_7(g_tab);
    register_bra_class_8(g_tab);
    register_bra_class_9(g_tab);
    register_generic(g_tab);
}

template <typename T>
int dalloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return fail(JK_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return 0;
}

template <typename T>
int upload(T **p, const std::vector<T> &h) {
    int err = dalloc(p, h.size());
    if (err) return err;
    if (!h.empty()) {
        cudaError_t e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(JK_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    }
    return 0;
}

inline int ncart_h(int l) { return (l + 1) * (l + 2) / 2; }

// ---------------------------------------------------------------------------
// small device kernels: densities, screening table, planning, epilogue
// ---------------------------------------------------------------------------

// Packed block layout of densities and J/K: one square block per molecule.
struct Layout {
    int nmol;
    long long ntot;              // elements per density
    const long long *mol_base;   // [nmol] first element of each block
    const int *mol_nao;          // [nmol] block size
};

// element r of a density -> index of the transposed element
__device__ __forceinline__ size_t transposed(const Layout &L, size_t r) {
    int lo = 0, hi = L.nmol;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if ((size_t)__ldg(L.mol_base + mid) <= r) lo = mid; else hi = mid;
    }
    const size_t base = (size_t)__ldg(L.mol_base + lo);
    const size_t n = (size_t)__ldg(L.mol_nao + lo);
    const size_t t = r - base;
    return base + (t % n) * n + t / n;
}

__global__ void prep_dm_kernel(const double *dm, int n_dm, Layout L, int hermi, int mixed,
                               double *dmj, double *dmk, float *dmj_f, float *dmk_f) {
    const size_t nn = (size_t)L.ntot;
    const size_t total = nn * n_dm;
    for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        size_t idm = x / nn, r = x % nn;
        double a = dm[x], at = dm[idm * nn + transposed(L, r)];
        double js = a + at;
        dmj[x] = js;
        dmk[x] = a;
        if (hermi == 0) dmk[(n_dm + idm) * nn + r] = at;
        if (mixed) {
            dmj_f[x] = (float)js;
            dmk_f[x] = (float)a;
            if (hermi == 0) dmk_f[(n_dm + idm) * nn + r] = (float)at;
        }
    }
}

// per shell pair: log of the largest |D| over its block in every density
// (symmetrised for hermi=0); shells of different molecules get -690
__global__ void dm_cond_kernel(const double *dm, int n_dm, Layout L, const ShellDev *sh, int nbas,
                               int hermi, float *dm_cond) {
    int ij = blockIdx.x * blockDim.x + threadIdx.x;
    if (ij >= nbas * nbas) return;
    int i = ij / nbas, j = ij % nbas;
    if (sh[i].mol != sh[j].mol) { dm_cond[ij] = -690.f; return; }
    const size_t base = (size_t)L.mol_base[sh[i].mol];
    const size_t nao = (size_t)L.mol_nao[sh[i].mol];
    int ni = (sh[i].l + 1) * (sh[i].l + 2) / 2, nj = (sh[j].l + 1) * (sh[j].l + 2) / 2;
    const size_t nn = (size_t)L.ntot;
    double mij = 0., mji = 0.;
    for (int d = 0; d < n_dm; ++d)
        for (int a = 0; a < ni; ++a)
            for (int b = 0; b < nj; ++b) {
                mij = fmax(mij, fabs(dm[d * nn + base + (size_t)(sh[i].ao + a) * nao + sh[j].ao + b]));
                mji = fmax(mji, fabs(dm[d * nn + base + (size_t)(sh[j].ao + b) * nao + sh[i].ao + a]));
            }
    double v = hermi == 0 ? mij + mji : fmax(mij, mji);
    dm_cond[ij] = (float)log(v + 1e-300);
}

__global__ void max_kernel(const float *x, int n, float *out) {
    __shared__ float red[1024];
    float m = -1e30f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, x[i]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

// Density part of the gradient screening bound over every quartet: twice
// the largest log|D| block plus the larger of the J and K weight logs.
__global__ void grad_bound_kernel(const float *dm_max, float log_j, float log_k, float *out) {
    out[0] = 2.f * dm_max[0] + fmaxf(log_j, log_k);
}

struct PlanClass {
    const float *bra_logq;
    const float *ket_logq;
    const int *ket_bstart;  // bucket boundaries of the ket list
    const int *ket_mb0;     // [nmol] first ket bucket of each molecule
    const int *ket_mbn;     // [nmol] ket buckets of each molecule
    const int2 *bra_ij;
    const ShellDev *shells;
    int nbra, nket, nbk, same, qb64, qb32;
    int *kb64, *ke64, *cnt64, *kb32, *ke32, *cnt32;  // [nbra * nbk]
    int start;  // offset in the flattened (class, bra, bucket) index space
};

// number of entries of the descending array q[0..n) with q[k] >= thr
__device__ int count_ge(const float *q, int n, float thr) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (q[mid] >= thr) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Per (ket bucket, bra pair): the ket range that can pass
// q_ij q_kl max|D| >= tol with the largest density block, and in mixed mode
// the two overlapping ranges the FP64 and FP32 launches scan: kets before
// beg32 reach the split even with the bra's own density block (FP64 for
// sure), kets from mid on stay below it even with the largest block (FP32
// for sure); in between the kernels decide per quartet from its own six
// blocks.  The counts are the work units of each range, scanned into unit
// offsets.
__global__ void plan_kernel(const PlanClass *pcs, int npc, int total, const float *dm_max,
                            const float *dm_cond, int nbas, float log_cut, float log_split, int mixed) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = npc;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (pcs[mid].start <= g) lo = mid; else hi = mid;
    }
    const PlanClass &p = pcs[lo];
    int x = g - p.start;
    if (x >= p.nbra * p.nbk) return;
    int ib = x % p.nbra, kl = x / p.nbra;  // ket-bucket major
    // kets of the bra's molecule only: kl-th bucket of that molecule
    const int mol = p.shells[p.bra_ij[ib].x].mol;
    if (kl >= p.ket_mbn[mol]) {
        p.kb64[x] = p.ke64[x] = p.kb32[x] = p.ke32[x] = 0;
        p.cnt64[x] = p.cnt32[x] = 0;
        return;
    }
    const int k = p.ket_mb0[mol] + kl;
    int b0 = p.ket_bstart[k], b1 = p.ket_bstart[k + 1];
    // The kernels decide each quartet from the bound they compute
    // themselves (pair_passes); these ranges only have to contain every
    // quartet a kernel would take.  Float sums of logs associate differently
    // here and there, so a bound at a threshold can round to opposite sides
    // of it: every range is widened by PLAN_MARGIN in log space (a quartet
    // dropped at the split would lose a contribution of the split's size).
    constexpr float PLAN_MARGIN = 1e-3f;
    float base = p.bra_logq[ib] + dm_max[0];
    int end = b0 + count_ge(p.ket_logq + b0, b1 - b0, log_cut - base - PLAN_MARGIN);
    int mid = end, beg32 = end;
    if (mixed) {
        mid = min(end, b0 + count_ge(p.ket_logq + b0, b1 - b0, log_split - base - PLAN_MARGIN));
        const int2 ij = p.bra_ij[ib];
        const float own = p.bra_logq[ib] + dm_cond[(size_t)ij.x * nbas + ij.y];
        beg32 = min(end, b0 + count_ge(p.ket_logq + b0, b1 - b0, log_split - own + PLAN_MARGIN));
    }
    if (p.same) {
        end = max(b0, min(end, ib + 1));
        mid = max(b0, min(mid, ib + 1));
        beg32 = max(b0, min(beg32, ib + 1));
    }
    p.kb64[x] = b0;
    p.ke64[x] = mid;
    p.cnt64[x] = (mid - b0 + JK_KCHUNK - 1) / JK_KCHUNK;
    p.kb32[x] = beg32;
    p.ke32[x] = end;
    p.cnt32[x] = mixed ? (end - beg32 + JK_KCHUNK - 1) / JK_KCHUNK : 0;
}

struct ScanJob { const int *cnt; int *off; int n; };

// exclusive prefix sum, one block per job; off[n] = total
__global__ void scan_kernel(const ScanJob *jobs) {
    const ScanJob jb = jobs[blockIdx.x];
    __shared__ int buf[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < jb.n; base += 1024) {
        int i = base + threadIdx.x;
        int v = i < jb.n ? jb.cnt[i] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int s = 1; s < 1024; s <<= 1) {
            int t = threadIdx.x >= s ? buf[threadIdx.x - s] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < jb.n) jb.off[i] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) jb.off[jb.n] = carry;
}

// fixed-point pairs (a, b) of the deterministic mode -> a 2^-24 + b 2^-56
__global__ void fx_to_double_kernel(const unsigned long long *fx, size_t n, double *out) {
    for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x)
        out[x] = (double)(long long)fx[2 * x] * (1. / JK_FX_HI) + (double)(long long)fx[2 * x + 1] * (1. / JK_FX_LO);
}

// Products with the sparse map C between the user and the sorted basis
// (each row holds the few coefficients of one Cartesian component: a
// Cartesian-to-spherical block or a scale factor), S given as compressed
// rows (ptr, idx, val):
//   right: out[i][r][m] = sum_p in[i][r][idx[p]] val[p],  p in row m of S
//   left:  out[i][r][m] = sum_p val[p] in[i][idx[p]][m],  p in row r of S
// so that C D C^T is right then left with S = C, and C^T V C right then
// left with S = C^T.  A dense product spends O(nao^3) FP64 operations on
// zeros (GB300's FP64 rate makes that milliseconds at nao ~ 700); these
// spend a few per element.
__global__ void sparse_right_kernel(const int *ptr, const int *idx, const double *val, long long total, int K, int M,
                                    const double *in, double *out) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(x % M);
        const double *row = in + (x / M) * K;
        double s = 0.;
        for (int p = __ldg(ptr + m); p < __ldg(ptr + m + 1); ++p) s = fma(row[__ldg(idx + p)], __ldg(val + p), s);
        out[x] = s;
    }
}

__global__ void sparse_left_kernel(const int *ptr, const int *idx, const double *val, long long total, int R, int K,
                                   int M, const double *in, double *out) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(x % M);
        const long long ir = x / M;
        const int r = (int)(ir % R);
        const double *blk = in + (ir / R) * K * (long long)M;
        double s = 0.;
        for (int p = __ldg(ptr + r); p < __ldg(ptr + r + 1); ++p) s = fma(__ldg(val + p), blk[(long long)__ldg(idx + p) * M + m], s);
        out[x] = s;
    }
}

__global__ void epilogue_kernel(const double *jt, const double *kt, int n_dm, Layout L, int hermi,
                                int with_j, int with_k, double *vj, double *vk) {
    const size_t nn = (size_t)L.ntot;
    const size_t total = nn * n_dm;
    for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        size_t idm = x / nn, r = x % nn;
        size_t xt = idm * nn + transposed(L, r);
        if (with_j) vj[x] = hermi == 2 ? 0. : jt[x] + jt[xt];
        if (with_k) {
            if (hermi == 1) vk[x] = kt[x] + kt[xt];
            else if (hermi == 2) vk[x] = kt[x] - kt[xt];
            else vk[x] = kt[x] + kt[n_dm * nn + xt];
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// optimizer object
// ---------------------------------------------------------------------------

struct HostPairList {
    std::vector<int2> ij;
    std::vector<float> logq;
    std::vector<int> prim_off;
    std::vector<int> prim_cnt;
};

struct jk_opt {
    int device = 0;
    int sm_count = 0;
    int nbas = 0, nao = 0;
    double tol = 1e-13;
    std::vector<ShellDev> shells_h;
    std::vector<double> exps_h, coefs_h;  // per shell primitive data
    std::vector<int> prim0_h;              // first primitive of each shell
    ShellDev *shells = nullptr;
    d4 *pp_a = nullptr, *pp_b = nullptr;
    double *pp_ip = nullptr;
    float4 *pp_af = nullptr, *pp_bf = nullptr;
    float *pp_ipf = nullptr;
    double2 *pp_e = nullptr;   // primitive exponents of every primitive pair (gradients)
    int natm = 0;
    int lmax = 0;              // highest shell angular momentum
    int *shell_atom = nullptr;
    float *grad_max = nullptr; // screening bound of a gradient build (device scalar)
    double *rys_coef = nullptr;
    float *rys_coef_f = nullptr;
    // sorted pair lists per pair class
    int npairs[NPAIRCLASS] = {0};
    int2 *pl_ij[NPAIRCLASS] = {nullptr};
    float *pl_logq[NPAIRCLASS] = {nullptr};
    int *pl_prim[NPAIRCLASS] = {nullptr};
    int *pl_cnt[NPAIRCLASS] = {nullptr};     // primitive pairs kept per pair
    int nbk[NPAIRCLASS] = {0};           // ket buckets per molecule (max over molecules)
    int *pl_bstart[NPAIRCLASS] = {nullptr};  // bucket boundaries (molecule, primitive count)
    int *pl_mb0[NPAIRCLASS] = {nullptr};     // [nmol] first bucket of each molecule
    int *pl_mbn[NPAIRCLASS] = {nullptr};     // [nmol] buckets of each molecule
    // molecules: packed block layout of densities and J/K
    int nmol = 1;
    long long ntot = 0;
    std::vector<long long> mol_base_h;
    std::vector<int> mol_nao_h;
    long long *mol_base = nullptr;
    int *mol_nao = nullptr;
    int *mol_ndm = nullptr;      // device copy of the per-molecule density counts
    bool use_mol_ndm = false;
    std::vector<double> qcond_h;  // [nbas*nbas]
    // planning buffers per quartet class
    int *kb64[NQCLASS] = {nullptr}, *ke64[NQCLASS] = {nullptr}, *cnt64[NQCLASS] = {nullptr}, *off64[NQCLASS] = {nullptr};
    int *kb32[NQCLASS] = {nullptr}, *ke32[NQCLASS] = {nullptr}, *cnt32[NQCLASS] = {nullptr}, *off32[NQCLASS] = {nullptr};
    PlanClass *plan_dev = nullptr;
    ScanJob *scan_dev = nullptr;
    int nplan = 0, nscan = 0, plan_total = 0;
    std::vector<int> plan_classes;  // quartet classes with work
    // workspace
    float *dm_cond = nullptr, *dm_max = nullptr;
    int ws_ndm = 0;
    double *dmj = nullptr, *dmk = nullptr, *jt = nullptr, *kt = nullptr;
    // deterministic accumulation: fixed-point sums of J and K (see jk_add)
    bool det = false;
    int fx_ndm = 0;
    unsigned long long *jfx = nullptr, *kfx = nullptr;
    float *dmj_f = nullptr, *dmk_f = nullptr;
    unsigned long long *counters = nullptr;
    // per-launch quartet counts of the last two builds (launch sizing from
    // history); qhist_cur selects the half the next build writes
    unsigned long long *qhist = nullptr;
    int qhist_cur = 0;
    bool qhist_valid = false;
    int *work = nullptr;                 // [2 passes][NQCLASS][2 precisions] unit counters of the class launches
    std::vector<void *> owned;
    // side streams: class kernels of one build run concurrently on them,
    // forked from and joined back into the caller's stream with events
    static constexpr int NSIDE = 4;
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[NSIDE] = {};
    // autotuned launch variant per (class, precision): kernel family
    // (0 default, 1 alternative) and grid size in blocks per SM (0: default)
    int variant_alt[2 * NQCLASS] = {0};
    int variant_grid[2 * NQCLASS] = {0};
    // per-class timing (diagnostics)
    bool time_classes = false;
    std::vector<cudaEvent_t> ev;        // pairs of events
    std::vector<int> ev_slot;           // 2*q + precision of each pair
    std::vector<int64_t> last_flops, last_quartets;  // [2*NQCLASS]
};

namespace {

void free_all(jk_opt *o) {
    for (void *p : o->owned) cudaFree(p);
    o->owned.clear();
    for (cudaEvent_t e : o->ev) cudaEventDestroy(e);
    o->ev.clear();
    for (int i = 0; i < jk_opt::NSIDE; ++i) {
        if (o->side[i]) cudaStreamDestroy(o->side[i]);
        if (o->join_ev[i]) cudaEventDestroy(o->join_ev[i]);
        o->side[i] = nullptr;
        o->join_ev[i] = nullptr;
    }
    if (o->fork_ev) cudaEventDestroy(o->fork_ev);
    o->fork_ev = nullptr;
}

__global__ void probe_fma_kernel(double *out, int iters, int fp32) {
    double a[8];
    float af[8];
    for (int k = 0; k < 8; ++k) { a[k] = 1.0 + 1e-3 * (threadIdx.x + k); af[k] = (float)a[k]; }
    const double m = 0.999999, c = 1e-7;
    const float mf = 0.999999f, cf = 1e-7f;
    if (fp32) {
        for (int i = 0; i < iters; ++i)
#pragma unroll
            for (int k = 0; k < 8; ++k) af[k] = fmaf(af[k], mf, cf);
        float s = 0.f;
        for (int k = 0; k < 8; ++k) s += af[k];
        if (s == 12345.f) out[0] = s;
    } else {
        for (int i = 0; i < iters; ++i)
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
        double s = 0.;
        for (int k = 0; k < 8; ++k) s += a[k];
        if (s == 12345.) out[0] = s;
    }
}

template <typename T>
int own_alloc(jk_opt *o, T **p, size_t n) {
    int e = dalloc(p, n);
    if (!e) o->owned.push_back((void *)*p);
    return e;
}

template <typename T>
int own_upload(jk_opt *o, T **p, const std::vector<T> &h) {
    int e = upload(p, h);
    if (!e) o->owned.push_back((void *)*p);
    return e;
}

struct PrimPairHost {
    std::vector<d4> a, b;
    std::vector<double> ip;
    std::vector<double2> e;   // exponents (a, b) (gradient kernels)
};

// Primitive pairs of shell pair (i, j).  With prune, pairs whose Gaussian
// product is negligible, |K_ab| (pi/p)^(3/2) < 1e-18 (the overlap of the two
// primitives; every integral of the pair is bounded by a small multiple of
// it), are left out -- tight primitives on different atoms decay to nothing
// -- but the largest one is always kept.  Returns the number added.
constexpr double PRIM_PRUNE = 1e-18;
const double SQRT_TWO_PI25 = std::sqrt(2. * std::pow(M_PI, 2.5));

inline double prim_weight(double a, double b, double ca, double cb, double AB2) {
    double p = a + b;
    return std::fabs(std::exp(-a * b / p * AB2) * ca * cb) * std::pow(M_PI / p, 1.5);
}

int add_prim_pairs(const jk_opt *o, int i, int j, PrimPairHost &pp, bool prune = false) {
    const ShellDev &A = o->shells_h[i], &B = o->shells_h[j];
    double AB2 = (A.x - B.x) * (A.x - B.x) + (A.y - B.y) * (A.y - B.y) + (A.z - B.z) * (A.z - B.z);
    double wmax = 0.;
    int kmax = 0;
    if (prune) {
        for (int pa = 0; pa < A.nprim; ++pa)
            for (int pb = 0; pb < B.nprim; ++pb) {
                double w = prim_weight(o->exps_h[o->prim0_h[i] + pa], o->exps_h[o->prim0_h[j] + pb],
                                       o->coefs_h[o->prim0_h[i] + pa], o->coefs_h[o->prim0_h[j] + pb], AB2);
                if (w > wmax) { wmax = w; kmax = pa * B.nprim + pb; }
            }
    }
    int added = 0;
    for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = o->exps_h[o->prim0_h[i] + pa], b = o->exps_h[o->prim0_h[j] + pb];
            double ca = o->coefs_h[o->prim0_h[i] + pa], cb = o->coefs_h[o->prim0_h[j] + pb];
            if (prune && pa * B.nprim + pb != kmax && prim_weight(a, b, ca, cb, AB2) < PRIM_PRUNE) continue;
            double p = a + b;
            // K_ab c_a c_b / p times sqrt(2 pi^(5/2)): the product of a bra's
            // and a ket's value times 1/sqrt(p+q) is the ERI prefactor
            // 2 pi^(5/2) K_ab K_cd c_a c_b c_c c_d / (p q sqrt(p+q))
            double K = std::exp(-a * b / p * AB2) * ca * cb * SQRT_TWO_PI25 / p;
            double Px = (a * A.x + b * B.x) / p, Py = (a * A.y + b * B.y) / p, Pz = (a * A.z + b * B.z) / p;
            pp.a.push_back(d4{p, Px, Py, Pz});
            pp.b.push_back(d4{Px - A.x, Py - A.y, Pz - A.z, K});
            pp.ip.push_back(1.0 / p);
            pp.e.push_back(make_double2(a, b));
            ++added;
        }
    return added;
}

int count_prim_pairs(const jk_opt *o, int i, int j) {
    PrimPairHost tmp;
    return add_prim_pairs(o, i, j, tmp, true);
}

int launch_class(const void *func, int grid, int smem, const EngineDev &d, const ClassDev &c, int ntiles,
                 cudaStream_t st, int threads = JK_THREADS) {
    void *args[] = {(void *)&d, (void *)&c, (void *)&ntiles};
    CK(cudaLaunchKernel(func, dim3(grid), dim3(threads), args, (size_t)smem, st));
    return 0;
}

// Dynamic shared memory limit of every kernel: the largest any class
// launching it needs (the generic kernel serves several classes).
int set_smem_attrs() {
    std::vector<std::pair<const void *, int>> need;
    auto add = [&](const void *k, int bytes) {
        if (!k) return;
        for (auto &p : need)
            if (p.first == k) { p.second = std::max(p.second, bytes); return; }
        need.emplace_back(k, bytes);
    };
    for (int q = 0; q < NQCLASS; ++q) {
        const ClassEntry &e = g_tab[q];
        add(e.k64, e.smem64);
        add(e.k32, e.smem32);
        add(e.kdiag, e.smemdiag);
        add(e.k64_alt, e.smem64_alt);
        add(e.k32_alt, e.smem32_alt);
    }
    for (auto &p : need) CK(cudaFuncSetAttribute(p.first, cudaFuncAttributeMaxDynamicSharedMemorySize, p.second));
    return 0;
}

EngineDev base_engine(const jk_opt *o) {
    EngineDev d;
    std::memset(&d, 0, sizeof(d));
    d.shells = o->shells;
    d.pp_a = o->pp_a; d.pp_b = o->pp_b; d.pp_ip = o->pp_ip;
    d.pp_af = o->pp_af; d.pp_bf = o->pp_bf; d.pp_ipf = o->pp_ipf;
    d.rys_coef = o->rys_coef; d.rys_coef_f = o->rys_coef_f;
    d.nbas = o->nbas; d.nao = o->nao;
    d.ntot = o->ntot; d.mol_base = o->mol_base; d.mol_nao = o->mol_nao;
    d.mol_ndm = o->use_mol_ndm ? o->mol_ndm : nullptr;
    d.op_scale = 1.; d.op_scale_f = 1.f;
    return d;
}

Layout layout_of(const jk_opt *o) {
    return Layout{o->nmol, o->ntot, o->mol_base, o->mol_nao};
}

int grid_for(const jk_opt *o, long long upper_tiles, int lean = 0) {
    long long g = (long long)o->sm_count * (lean ? 8 : 2);
    if (upper_tiles < g) g = upper_tiles;
    return (int)std::max<long long>(g, 1);
}

// Launch the class kernel of (q, prec) with the optimizer's current variant.
int launch_variant(const jk_opt *o, int q, int prec, long long upper, const EngineDev &d, const ClassDev &c,
                   cudaStream_t st) {
    const ClassEntry &e = g_tab[q];
    const int alt = o->variant_alt[2 * q + prec] && (prec ? e.k32_alt : e.k64_alt);
    const void *k = prec ? (alt ? e.k32_alt : e.k32) : (alt ? e.k64_alt : e.k64);
    const int smem = prec ? (alt ? e.smem32_alt : e.smem32) : (alt ? e.smem64_alt : e.smem64);
    const int threads = alt ? e.threads_alt : (prec ? e.threads32 : e.threads64);
    const int lean = alt ? 0 : (prec ? e.lean32 : e.lean64);
    int grid;
    if (o->variant_grid[2 * q + prec] > 0)
        grid = (int)std::max<long long>(1, std::min<long long>(upper, (long long)o->sm_count * o->variant_grid[2 * q + prec]));
    else
        grid = grid_for(o, upper, lean);
    return launch_class(k, grid, smem, d, c, 0, st, threads);
}


}  // namespace

// Algorithmic FLOP model of one angular class: per primitive quartet
// n*(3*nf + 9*g) for the recurrences and the gx*gy*gz products plus
// C_root(n) = 52*n + 30 for the roots, weights and prefactors; per contracted
// quartet 12*nf*n_dm for the six density contractions.
static int64_t jk_flop_model(int li, int lj, int lk, int ll, int64_t nquart, int64_t nprim, int n_dm) {
    int n = (li + lj + lk + ll) / 2 + 1;
    int64_t nf = (int64_t)ncart_h(li) * ncart_h(lj) * ncart_h(lk) * ncart_h(ll);
    int64_t g = (int64_t)(li + 1) * (lj + 1) * (lk + 1) * (ll + 1);
    return nprim * (n * (3 * nf + 9 * g) + 52 * n + 30) + nquart * 12 * nf * n_dm;
}

extern "C" {

const char *jk_last_error(void) { return g_last_error.c_str(); }

int jk_n_quartet_classes(void) { return NQCLASS; }

int jk_opt_time_classes(jk_opt *opt, int enable) {
    if (!opt) return fail(JK_ERR_ARG, "null optimizer");
    opt->time_classes = enable != 0;
    return 0;
}

int jk_opt_class_times(jk_opt *opt, double *ms, int64_t *flops, int64_t *quartets,
                       int32_t *li, int32_t *lj, int32_t *lk, int32_t *ll) {
    if (!opt || !ms) return fail(JK_ERR_ARG, "null argument");
    std::call_once(g_tab_once, init_registry);
    for (int k = 0; k < 2 * NQCLASS; ++k) {
        ms[k] = 0.;
        if (flops) flops[k] = opt->last_flops.empty() ? 0 : opt->last_flops[k];
        if (quartets) quartets[k] = opt->last_quartets.empty() ? 0 : opt->last_quartets[k];
    }
    for (size_t k = 0; k < opt->ev_slot.size(); ++k) {
        float t = 0.f;
        CK(cudaEventSynchronize(opt->ev[2 * k + 1]));
        CK(cudaEventElapsedTime(&t, opt->ev[2 * k], opt->ev[2 * k + 1]));
        ms[opt->ev_slot[k]] += t;
    }
    for (int q = 0; q < NQCLASS; ++q) {
        if (li) li[q] = g_tab[q].li;
        if (lj) lj[q] = g_tab[q].lj;
        if (lk) lk[q] = g_tab[q].lk;
        if (ll) ll[q] = g_tab[q].ll;
    }
    return 0;
}

int jk_probe_fma(double *out, int blocks, int iters, int fp32, void *stream) {
    if (!out || blocks <= 0 || iters <= 0) return fail(JK_ERR_ARG, "jk_probe_fma: invalid arguments");
    probe_fma_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, fp32);
    CK(cudaGetLastError());
    return 0;
}

int jk_opt_nao(const jk_opt *opt) { return opt ? opt->nao : -1; }

int jk_opt_npairs(const jk_opt *opt) {
    if (!opt) return -1;
    int n = 0;
    for (int c = 0; c < NPAIRCLASS; ++c) n += opt->npairs[c];
    return n;
}

int jk_opt_get_qcond(const jk_opt *opt, double *q) {
    if (!opt || !q) return fail(JK_ERR_ARG, "null argument");
    std::memcpy(q, opt->qcond_h.data(), sizeof(double) * opt->qcond_h.size());
    return 0;
}

void jk_opt_destroy(jk_opt *opt) {
    if (!opt) return;
    free_all(opt);
    delete opt;
}

// shell_mol / shell_ao / mol_nao: molecule of each shell, its first AO
// within the molecule, AOs per molecule (all null for one molecule).
static int create_impl(const int32_t *atm, int natm, const int32_t *bas, int nbas, const double *env, int nenv,
                       const int32_t *shell_mol, const int32_t *shell_ao, int nmol, const int32_t *mol_nao,
                       double tol, jk_opt **out) {
    if (!atm || !bas || !env || !out || natm <= 0 || nbas <= 0 || nenv <= 0 || !(tol >= 0) || nmol <= 0)
        return fail(JK_ERR_ARG, "jk_opt_create: invalid arguments");
    std::call_once(g_tab_once, init_registry);
    jk_opt *o = new jk_opt();
    *out = nullptr;
    auto bail = [&](int code) { free_all(o); delete o; return code; };
    CK(cudaGetDevice(&o->device));
    CK(cudaDeviceGetAttribute(&o->sm_count, cudaDevAttrMultiProcessorCount, o->device));
    if (int e = set_smem_attrs()) return bail(e);
    if (int e = grad_set_smem_attrs())
        return bail(fail(JK_ERR_CUDA, std::string("gradient kernels: ") + cudaGetErrorString((cudaError_t)e)));
    CK(cudaEventCreateWithFlags(&o->fork_ev, cudaEventDisableTiming));
    for (int i = 0; i < jk_opt::NSIDE; ++i) {
        CK(cudaStreamCreateWithFlags(&o->side[i], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&o->join_ev[i], cudaEventDisableTiming));
    }
    o->nbas = nbas;
    o->natm = natm;
    o->tol = tol;
    std::vector<int> shell_atom_h;
    int ao = 0, prev_l = -1;
    for (int i = 0; i < nbas; ++i) {
        const int32_t *b = bas + 8 * i;
        int ia = b[0], l = b[1], np = b[2], nctr = b[3], pe = b[5], pc = b[6];
        if (ia < 0 || ia >= natm) return bail(fail(JK_ERR_ARG, "shell atom index out of range"));
        if (l < 0 || l > JK_LMAX) return bail(fail(JK_ERR_LMAX, "shell angular momentum above the GPU limit (g)"));
        if (nctr != 1) return bail(fail(JK_ERR_ARG, "sorted basis must have one contraction per shell"));
        if (np <= 0 || pe < 0 || pc < 0 || pe + np > nenv || pc + np > nenv)
            return bail(fail(JK_ERR_ARG, "shell primitive data out of range"));
        if (l < prev_l) return bail(fail(JK_ERR_ARG, "shells must be sorted by angular momentum"));
        prev_l = l;
        o->lmax = std::max(o->lmax, l);
        shell_atom_h.push_back(ia);
        int pcoord = atm[6 * ia + 1];
        if (pcoord < 0 || pcoord + 3 > nenv) return bail(fail(JK_ERR_ARG, "atom coordinate pointer out of range"));
        ShellDev s;
        s.x = env[pcoord]; s.y = env[pcoord + 1]; s.z = env[pcoord + 2];
        if (!std::isfinite(s.x) || !std::isfinite(s.y) || !std::isfinite(s.z))
            return bail(fail(JK_ERR_ARG, "non-finite coordinates"));
        s.l = l; s.nprim = np; s.ao = ao; s.mol = 0;
        if (shell_mol) {
            s.mol = shell_mol[i];
            s.ao = shell_ao[i];
            if (s.mol < 0 || s.mol >= nmol || s.ao < 0 || s.ao + ncart_h(l) > mol_nao[s.mol])
                return bail(fail(JK_ERR_ARG, "shell molecule or AO offset out of range"));
        }
        ao += ncart_h(l);
        o->prim0_h.push_back((int)o->exps_h.size());
        for (int p = 0; p < np; ++p) {
            if (!(env[pe + p] > 0) || !std::isfinite(env[pc + p]))
                return bail(fail(JK_ERR_ARG, "invalid exponent or coefficient"));
            o->exps_h.push_back(env[pe + p]);
            o->coefs_h.push_back(env[pc + p]);
        }
        o->shells_h.push_back(s);
    }
    o->nao = shell_mol ? 0 : ao;
    o->nmol = nmol;
    o->ntot = 0;
    for (int m = 0; m < nmol; ++m) {
        int n = shell_mol ? mol_nao[m] : ao;
        if (n <= 0) return bail(fail(JK_ERR_ARG, "molecule without AOs"));
        o->mol_base_h.push_back(o->ntot);
        o->mol_nao_h.push_back(n);
        o->ntot += (long long)n * n;
    }
    if (int e = own_upload(o, &o->mol_base, o->mol_base_h)) return bail(e);
    if (int e = own_upload(o, &o->mol_nao, o->mol_nao_h)) return bail(e);
    if (int e = own_alloc(o, &o->mol_ndm, (size_t)nmol)) return bail(e);
    if (int e = own_upload(o, &o->shells, o->shells_h)) return bail(e);
    if (int e = own_upload(o, &o->shell_atom, shell_atom_h)) return bail(e);
    {
        std::vector<double> t(rys_coef_host, rys_coef_host + RYS_TABLE_SIZE);
        std::vector<float> tf(rys_coef_f_host, rys_coef_f_host + RYS_TABLE_F_SIZE);
        if (int e = own_upload(o, &o->rys_coef, t)) return bail(e);
        if (int e = own_upload(o, &o->rys_coef_f, tf)) return bail(e);
    }

    // candidate pairs per class (i >= j), skipping pairs whose every
    // primitive product decays below exp(-60)
    std::vector<HostPairList> cand(NPAIRCLASS);
    PrimPairHost cpp;
    for (int i = 0; i < nbas; ++i)
        for (int j = 0; j <= i; ++j) {
            const ShellDev &A = o->shells_h[i], &B = o->shells_h[j];
            if (A.mol != B.mol) continue;
            double AB2 = (A.x - B.x) * (A.x - B.x) + (A.y - B.y) * (A.y - B.y) + (A.z - B.z) * (A.z - B.z);
            double best = 1e300;
            for (int pa = 0; pa < A.nprim; ++pa)
                for (int pb = 0; pb < B.nprim; ++pb) {
                    double a = o->exps_h[o->prim0_h[i] + pa], b = o->exps_h[o->prim0_h[j] + pb];
                    best = std::min(best, a * b / (a + b) * AB2);
                }
            if (best > 60.) continue;
            int pc = pair_class(A.l, B.l);
            cand[pc].ij.push_back(int2{i, j});
            cand[pc].prim_off.push_back((int)cpp.a.size());
            cand[pc].prim_cnt.push_back(add_prim_pairs(o, i, j, cpp));
        }
    // Schwarz factors on the GPU
    {
        d4 *ca = nullptr, *cb = nullptr;
        double *cip = nullptr;
        if (int e = upload(&ca, cpp.a)) return bail(e);
        if (int e = upload(&cb, cpp.b)) { cudaFree(ca); return bail(e); }
        if (int e = upload(&cip, cpp.ip)) { cudaFree(ca); cudaFree(cb); return bail(e); }
        std::vector<int2 *> dij(NPAIRCLASS, nullptr);
        std::vector<int *> dpo(NPAIRCLASS, nullptr);
        std::vector<int *> dpc(NPAIRCLASS, nullptr);
        std::vector<float *> dq(NPAIRCLASS, nullptr);
        int err = 0;
        EngineDev d = base_engine(o);
        d.pp_a = ca; d.pp_b = cb; d.pp_ip = cip;
        for (int pc = 0; pc < NPAIRCLASS && !err; ++pc) {
            int n = (int)cand[pc].ij.size();
            if (n == 0) continue;
            if ((err = upload(&dij[pc], cand[pc].ij))) break;
            if ((err = upload(&dpo[pc], cand[pc].prim_off))) break;
            if ((err = upload(&dpc[pc], cand[pc].prim_cnt))) break;
            if ((err = dalloc(&dq[pc], n))) break;
            const ClassEntry &e = g_tab[quartet_class(pc, pc)];
            ClassDev c;
            std::memset(&c, 0, sizeof(c));
            c.bra.n = c.ket.n = n;
            c.bra.ij = c.ket.ij = dij[pc];
            c.bra.prim_off = c.ket.prim_off = dpo[pc];
            c.bra.prim_cnt = c.ket.prim_cnt = dpc[pc];
            c.same = 1;
            c.class_id = quartet_class(pc, pc);
            c.li = c.lk = pc_li(pc);
            c.lj = c.ll = pc_lj(pc);
            d.qout = dq[pc];
            int ntiles = (n + e.qbdiag - 1) / e.qbdiag;
            err = launch_class(e.kdiag, grid_for(o, ntiles), e.smemdiag, d, c, ntiles, 0);
        }
        if (!err) {
            cudaError_t ce = cudaDeviceSynchronize();
            if (ce != cudaSuccess) err = fail(JK_ERR_CUDA, std::string("Schwarz kernels: ") + cudaGetErrorString(ce));
        }
        std::vector<std::vector<float>> qh(NPAIRCLASS);
        for (int pc = 0; pc < NPAIRCLASS && !err; ++pc) {
            qh[pc].resize(cand[pc].ij.size());
            if (!qh[pc].empty() &&
                cudaMemcpy(qh[pc].data(), dq[pc], qh[pc].size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
                err = fail(JK_ERR_CUDA, "copy of Schwarz factors");
        }
        for (int pc = 0; pc < NPAIRCLASS; ++pc) { cudaFree(dij[pc]); cudaFree(dpo[pc]); cudaFree(dpc[pc]); cudaFree(dq[pc]); }
        cudaFree(ca); cudaFree(cb); cudaFree(cip);
        if (err) return bail(err);
        // sort; every pair with a nonzero Schwarz factor is kept whatever
        // the densities of later builds (the per-build plan cuts the ket
        // ranges by the actual density maxima)
        o->qcond_h.assign((size_t)nbas * nbas, 0.);
        PrimPairHost fpp;
        for (int pc = 0; pc < NPAIRCLASS; ++pc) {
            std::vector<int> idx;
            for (int k = 0; k < (int)qh[pc].size(); ++k) {
                const int2 &p = cand[pc].ij[k];
                o->qcond_h[(size_t)p.x * nbas + p.y] = o->qcond_h[(size_t)p.y * nbas + p.x] = qh[pc][k];
                if (qh[pc][k] > 0) idx.push_back(k);
            }
            std::vector<int> pruned(qh[pc].size(), 0);
            for (int k : idx) pruned[k] = count_prim_pairs(o, cand[pc].ij[k].x, cand[pc].ij[k].y);
            auto npp = [&](int k) { return pruned[k]; };
            auto molp = [&](int k) { return o->shells_h[cand[pc].ij[k].x].mol; };
            // order: molecule, primitive count (descending), Schwarz factor (descending)
            std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
                int ma = molp(a), mb = molp(b);
                if (ma != mb) return ma < mb;
                int na = npp(a), nb = npp(b);
                if (na != nb) return na > nb;
                return qh[pc][a] > qh[pc][b];
            });
            // buckets: runs of equal (molecule, primitive count)
            std::vector<int> bstart{0}, bmol;
            for (size_t t = 0; t < idx.size(); ++t) {
                if (t > 0 && (npp(idx[t]) != npp(idx[t - 1]) || molp(idx[t]) != molp(idx[t - 1])))
                    bstart.push_back((int)t);
                if (bmol.size() < bstart.size()) bmol.push_back(molp(idx[t]));
            }
            bstart.push_back((int)idx.size());
            if (idx.empty()) { bstart = {0, 0}; bmol = {0}; }
            std::vector<int> mb0(nmol, 0), mbn(nmol, 0);
            for (int k = (int)bmol.size() - 1; k >= 0; --k) {
                if (idx.empty()) break;
                mb0[bmol[k]] = k;
                mbn[bmol[k]] += 1;
            }
            int maxb = 0;
            for (int m = 0; m < nmol; ++m) maxb = std::max(maxb, mbn[m]);
            o->nbk[pc] = std::max(maxb, 1);
            if (int e = own_upload(o, &o->pl_bstart[pc], bstart)) return bail(e);
            if (int e = own_upload(o, &o->pl_mb0[pc], mb0)) return bail(e);
            if (int e = own_upload(o, &o->pl_mbn[pc], mbn)) return bail(e);
            HostPairList fin;
            for (int k : idx) {
                const int2 &p = cand[pc].ij[k];
                fin.ij.push_back(p);
                fin.logq.push_back(std::log(qh[pc][k]));
                fin.prim_off.push_back((int)fpp.a.size());
                fin.prim_cnt.push_back(add_prim_pairs(o, p.x, p.y, fpp, true));
            }
            o->npairs[pc] = (int)fin.ij.size();
            if (int e = own_upload(o, &o->pl_ij[pc], fin.ij)) return bail(e);
            if (int e = own_upload(o, &o->pl_logq[pc], fin.logq)) return bail(e);
            if (int e = own_upload(o, &o->pl_prim[pc], fin.prim_off)) return bail(e);
            if (int e = own_upload(o, &o->pl_cnt[pc], fin.prim_cnt)) return bail(e);
        }
        std::vector<float4> af, bf;
        std::vector<float> ipf;
        for (size_t k = 0; k < fpp.a.size(); ++k) {
            af.push_back(make_float4((float)fpp.a[k].x, (float)fpp.a[k].y, (float)fpp.a[k].z, (float)fpp.a[k].w));
            bf.push_back(make_float4((float)fpp.b[k].x, (float)fpp.b[k].y, (float)fpp.b[k].z, (float)fpp.b[k].w));
            ipf.push_back((float)fpp.ip[k]);
        }
        if (int e = own_upload(o, &o->pp_a, fpp.a)) return bail(e);
        if (int e = own_upload(o, &o->pp_b, fpp.b)) return bail(e);
        if (int e = own_upload(o, &o->pp_ip, fpp.ip)) return bail(e);
        if (int e = own_upload(o, &o->pp_af, af)) return bail(e);
        if (int e = own_upload(o, &o->pp_bf, bf)) return bail(e);
        if (int e = own_upload(o, &o->pp_ipf, ipf)) return bail(e);
        if (int e = own_upload(o, &o->pp_e, fpp.e)) return bail(e);
    }
    // planning buffers
    std::vector<PlanClass> plan;
    std::vector<ScanJob> scans;
    int total = 0;
    for (int a = 0; a < NPAIRCLASS; ++a)
        for (int b = 0; b <= a; ++b) {
            int q = quartet_class(a, b);
            int nb = o->npairs[a], nk = o->npairs[b];
            if (nb == 0 || nk == 0) continue;
            const ClassEntry &e = g_tab[q];
            int nx = nb * o->nbk[b];
            if (int er = own_alloc(o, &o->kb64[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->ke64[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->cnt64[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->off64[q], nx + 1)) return bail(er);
            if (int er = own_alloc(o, &o->kb32[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->ke32[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->cnt32[q], nx)) return bail(er);
            if (int er = own_alloc(o, &o->off32[q], nx + 1)) return bail(er);
            PlanClass p;
            p.bra_logq = o->pl_logq[a];
            p.ket_logq = o->pl_logq[b];
            p.ket_bstart = o->pl_bstart[b];
            p.ket_mb0 = o->pl_mb0[b];
            p.ket_mbn = o->pl_mbn[b];
            p.bra_ij = o->pl_ij[a];
            p.shells = o->shells;
            p.nbra = nb; p.nket = nk; p.nbk = o->nbk[b]; p.same = (a == b);
            p.qb64 = e.qb64; p.qb32 = e.qb32;
            p.kb64 = o->kb64[q]; p.ke64 = o->ke64[q]; p.cnt64 = o->cnt64[q];
            p.kb32 = o->kb32[q]; p.ke32 = o->ke32[q]; p.cnt32 = o->cnt32[q];
            p.start = total;
            total += nx;
            plan.push_back(p);
            scans.push_back(ScanJob{o->cnt64[q], o->off64[q], nx});
            scans.push_back(ScanJob{o->cnt32[q], o->off32[q], nx});
            o->plan_classes.push_back(q);
        }
    o->nplan = (int)plan.size();
    o->nscan = (int)scans.size();
    o->plan_total = total;
    if (int e = own_upload(o, &o->plan_dev, plan)) return bail(e);
    if (int e = own_upload(o, &o->scan_dev, scans)) return bail(e);
    if (int e = own_alloc(o, &o->dm_cond, (size_t)nbas * nbas)) return bail(e);
    if (int e = own_alloc(o, &o->dm_max, 1)) return bail(e);
    if (int e = own_alloc(o, &o->grad_max, 1)) return bail(e);
    if (int e = own_alloc(o, &o->counters, 4 * NQCLASS)) return bail(e);
    if (int e = own_alloc(o, &o->qhist, 4 * NQCLASS)) return bail(e);
    if (int e = own_alloc(o, &o->work, 4 * NQCLASS)) return bail(e);
    *out = o;
    return 0;
}

int jk_opt_create(const int32_t *atm, int natm, const int32_t *bas, int nbas, const double *env, int nenv,
                  double tol, int flags, jk_opt **out) {
    (void)flags;
    return create_impl(atm, natm, bas, nbas, env, nenv, nullptr, nullptr, 1, nullptr, tol, out);
}

int jk_opt_create_batch(const int32_t *atm, int natm, const int32_t *bas, int nbas, const double *env, int nenv,
                        const int32_t *shell_mol, const int32_t *shell_ao, int nmol, const int32_t *mol_nao,
                        double tol, int flags, jk_opt **out) {
    (void)flags;
    if (!shell_mol || !shell_ao || !mol_nao) return fail(JK_ERR_ARG, "jk_opt_create_batch: null molecule arrays");
    return create_impl(atm, natm, bas, nbas, env, nenv, shell_mol, shell_ao, nmol, mol_nao, tol, out);
}

static int ensure_workspace(jk_opt *o, int n_dm) {
    if (n_dm <= o->ws_ndm) return 0;
    for (void *p : {(void *)o->dmj, (void *)o->dmk, (void *)o->jt, (void *)o->kt, (void *)o->dmj_f, (void *)o->dmk_f}) {
        if (!p) continue;
        auto it = std::find(o->owned.begin(), o->owned.end(), p);
        if (it != o->owned.end()) o->owned.erase(it);
        cudaFree(p);
    }
    size_t nn = (size_t)o->ntot;
    if (int e = own_alloc(o, &o->dmj, nn * n_dm)) return e;
    if (int e = own_alloc(o, &o->dmk, nn * 2 * n_dm)) return e;
    if (int e = own_alloc(o, &o->jt, nn * n_dm)) return e;
    if (int e = own_alloc(o, &o->kt, nn * 2 * n_dm)) return e;
    if (int e = own_alloc(o, &o->dmj_f, nn * n_dm)) return e;
    if (int e = own_alloc(o, &o->dmk_f, nn * 2 * n_dm)) return e;
    o->ws_ndm = n_dm;
    return 0;
}

static int ensure_fx(jk_opt *o, int n_dm) {
    if (n_dm <= o->fx_ndm) return 0;
    for (void *p : {(void *)o->jfx, (void *)o->kfx}) {
        if (!p) continue;
        auto it = std::find(o->owned.begin(), o->owned.end(), p);
        if (it != o->owned.end()) o->owned.erase(it);
        cudaFree(p);
    }
    size_t nn = (size_t)o->ntot;
    if (int e = own_alloc(o, &o->jfx, nn * 2 * n_dm)) return e;
    if (int e = own_alloc(o, &o->kfx, nn * 2 * 2 * n_dm)) return e;
    o->fx_ndm = n_dm;
    return 0;
}

// Operator passes of a build: lr * erf(|omega| r)/r + sr * erfc(|omega| r)/r
// = sr * (1/r) + (lr - sr) * erf(|omega| r)/r, one pass per nonzero term.
struct OpPass { double omega2, scale; };

static int op_passes(double omega, double lr, double sr, OpPass *out) {
    int n = 0;
    if (omega == 0.) {
        if (lr != sr) return -1;
        out[n++] = OpPass{0., sr};
        return n;
    }
    if (sr != 0.) out[n++] = OpPass{0., sr};
    if (lr != sr) out[n++] = OpPass{omega * omega, lr - sr};
    return n;
}

static int build_impl(jk_opt *o, const double *dm, int n_dm, int hermi, int with_j, int with_k, int precision,
                      double split_thresh, double *vj, double *vk, void *stream, jk_stats *stats,
                      double omega = 0., double lr_factor = 1., double sr_factor = 1.) {
    OpPass passes[2];
    const int npass = op_passes(omega, lr_factor, sr_factor, passes);
    if (npass < 0 || !std::isfinite(omega) || !std::isfinite(lr_factor) || !std::isfinite(sr_factor))
        return fail(JK_ERR_ARG, "jk_build: omega = 0 needs lr_factor == sr_factor");
    if (npass == 0) return fail(JK_ERR_ARG, "jk_build: lr_factor = sr_factor = 0 gives no operator");
    if (!o || !dm || n_dm <= 0 || hermi < 0 || hermi > 2 || (!with_j && !with_k))
        return fail(JK_ERR_ARG, "jk_build: invalid arguments");
    if ((with_j && !vj) || (with_k && !vk)) return fail(JK_ERR_ARG, "jk_build: missing output buffer");
    if (precision != JK_PREC_FP64 && precision != JK_PREC_MIXED && precision != JK_PREC_MIXED_FP32ROOTS)
        return fail(JK_ERR_ARG, "jk_build: bad precision");
    if (precision != JK_PREC_FP64 && !(split_thresh > 0)) return fail(JK_ERR_ARG, "jk_build: split_thresh must be > 0");
    cudaStream_t st = (cudaStream_t)stream;
    if (int e = ensure_workspace(o, n_dm)) return e;
    if (o->det)
        if (int e = ensure_fx(o, n_dm)) return e;
    const int mixed = precision != JK_PREC_FP64;
    const size_t nn = (size_t)o->ntot;
    const Layout L = layout_of(o);
    const int n_dmk = hermi == 0 ? 2 * n_dm : n_dm;
    int launches = 0;
    {
        int grid = (int)std::min<size_t>((nn * n_dm + 255) / 256, (size_t)o->sm_count * 8);
        prep_dm_kernel<<<grid, 256, 0, st>>>(dm, n_dm, L, hermi, mixed, o->dmj, o->dmk, o->dmj_f, o->dmk_f);
        int nb2 = o->nbas * o->nbas;
        dm_cond_kernel<<<(nb2 + 255) / 256, 256, 0, st>>>(dm, n_dm, L, o->shells, o->nbas, hermi, o->dm_cond);
        max_kernel<<<1, 1024, 0, st>>>(o->dm_cond, nb2, o->dm_max);
        launches += 3;
    }
    if (o->nplan > 0) {
        float log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
        float log_split = mixed ? (float)std::log(split_thresh) : 0.f;
        plan_kernel<<<(o->plan_total + 255) / 256, 256, 0, st>>>(o->plan_dev, o->nplan, o->plan_total, o->dm_max,
                                                                 o->dm_cond, o->nbas, log_cut, log_split, mixed);
        scan_kernel<<<o->nscan, 1024, 0, st>>>(o->scan_dev);
        launches += 2;
    }
    CK(cudaGetLastError());
    if (with_j) CK(cudaMemsetAsync(o->jt, 0, sizeof(double) * nn * n_dm, st));
    if (with_k) CK(cudaMemsetAsync(o->kt, 0, sizeof(double) * nn * n_dmk, st));
    if (o->det) {
        CK(cudaMemsetAsync(o->jfx, 0, sizeof(unsigned long long) * 2 * nn * n_dm, st));
        CK(cudaMemsetAsync(o->kfx, 0, sizeof(unsigned long long) * 2 * nn * n_dmk, st));
    }
    CK(cudaMemsetAsync(o->work, 0, sizeof(int) * 4 * NQCLASS, st));
    const bool want_stats = stats != nullptr;
    if (want_stats) CK(cudaMemsetAsync(o->counters, 0, sizeof(unsigned long long) * 4 * NQCLASS, st));
    unsigned long long *qnow = o->qhist + o->qhist_cur * 2 * NQCLASS;
    const unsigned long long *qprev = o->qhist_valid ? o->qhist + (1 - o->qhist_cur) * 2 * NQCLASS : nullptr;
    CK(cudaMemsetAsync(qnow, 0, sizeof(unsigned long long) * 2 * NQCLASS, st));

    EngineDev d = base_engine(o);
    d.dm_cond = o->dm_cond;
    d.dmj = o->dmj; d.dmk = o->dmk; d.dmj_f = o->dmj_f; d.dmk_f = o->dmk_f;
    d.vj = o->jt; d.vk = o->kt;
    d.n_dm = n_dm; d.n_dmk = n_dmk;
    d.with_j = with_j && hermi != 2;
    d.with_k = with_k;
    d.log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
    d.log_split = mixed ? (float)std::log(split_thresh) : 0.f;
    d.fp32_asym = precision == JK_PREC_MIXED_FP32ROOTS;
    d.qprev = qprev;
    d.qnow = qnow;
    d.vj_fx = o->det ? o->jfx : nullptr;
    d.vk_fx = o->det ? o->kfx : nullptr;
    o->qhist_cur ^= 1;
    o->qhist_valid = true;
    o->ev_slot.clear();
    if (o->time_classes) {
        size_t need = 4 * o->plan_classes.size() * npass;
        while (o->ev.size() < need) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            o->ev.push_back(e);
        }
    }
    // Class kernels are independent (they only add into the accumulators), so
    // unless per-class timing is on they run concurrently on the side
    // streams, heaviest (highest angular momentum) classes first.
    const bool concurrent = !o->time_classes;
    if (concurrent) {
        CK(cudaEventRecord(o->fork_ev, st));
        for (int i = 0; i < jk_opt::NSIDE; ++i) CK(cudaStreamWaitEvent(o->side[i], o->fork_ev, 0));
    }
    int nlaunched = 0;
    for (int ip = 0; ip < npass; ++ip) {
        d.omega2 = passes[ip].omega2; d.omega2_f = (float)passes[ip].omega2;
        d.op_scale = passes[ip].scale; d.op_scale_f = (float)passes[ip].scale;
        int *work = o->work + ip * 2 * NQCLASS;
        for (auto it = o->plan_classes.rbegin(); it != o->plan_classes.rend(); ++it) {
            const int q = *it;
            const ClassEntry &e = g_tab[q];
            int a = 0;
            while ((a + 1) * (a + 2) / 2 <= q) ++a;
            int b = q - a * (a + 1) / 2;
            ClassDev c;
            std::memset(&c, 0, sizeof(c));
            c.bra = PairList{o->npairs[a], o->pl_ij[a], o->pl_logq[a], o->pl_prim[a], o->pl_cnt[a]};
            c.ket = PairList{o->npairs[b], o->pl_ij[b], o->pl_logq[b], o->pl_prim[b], o->pl_cnt[b]};
            c.same = a == b;
            c.nbk = o->nbk[b];
            c.nx = o->npairs[a] * o->nbk[b];
            c.li = e.li; c.lj = e.lj; c.lk = e.lk; c.ll = e.ll;
            long long upper = (long long)o->npairs[a] * ((o->npairs[b] + e.qb64 - 1) / e.qb64 + o->nbk[b]);
            if (!d.with_j && !d.with_k) break;
            cudaStream_t ls = concurrent ? o->side[nlaunched++ % jk_opt::NSIDE] : st;
            c.class_id = q;
            d.counters = want_stats ? o->counters : nullptr;
            c.work = work + 2 * q;
            c.q_off = o->off64[q]; c.ket_begin = o->kb64[q]; c.ket_end = o->ke64[q];
            c.split_mode = mixed ? SPLIT_HIGH : SPLIT_ALL;
            if (o->time_classes) { o->ev_slot.push_back(2 * q); CK(cudaEventRecord(o->ev[2 * (o->ev_slot.size() - 1)], st)); }
            if (int er = launch_variant(o, q, 0, upper, d, c, ls)) return er;
            if (o->time_classes) CK(cudaEventRecord(o->ev[2 * (o->ev_slot.size() - 1) + 1], st));
            ++launches;
            if (mixed) {
                c.class_id = NQCLASS + q;  // FP32 counters in the second half
                c.work = work + 2 * q + 1;
                c.q_off = o->off32[q]; c.ket_begin = o->kb32[q]; c.ket_end = o->ke32[q];
                c.split_mode = SPLIT_LOW;
                long long up32 = (long long)o->npairs[a] * ((o->npairs[b] + e.qb32 - 1) / e.qb32 + o->nbk[b]);
                if (o->time_classes) { o->ev_slot.push_back(2 * q + 1); CK(cudaEventRecord(o->ev[2 * (o->ev_slot.size() - 1)], st)); }
                cudaStream_t ls32 = concurrent ? o->side[nlaunched++ % jk_opt::NSIDE] : st;
                if (int er = launch_variant(o, q, 1, up32, d, c, ls32)) return er;
                if (o->time_classes) CK(cudaEventRecord(o->ev[2 * (o->ev_slot.size() - 1) + 1], st));
                ++launches;
            }
        }
    }  // passes
    if (concurrent) {
        for (int i = 0; i < jk_opt::NSIDE; ++i) {
            CK(cudaEventRecord(o->join_ev[i], o->side[i]));
            CK(cudaStreamWaitEvent(st, o->join_ev[i], 0));
        }
    }
    {
        int grid = (int)std::min<size_t>((nn * n_dm + 255) / 256, (size_t)o->sm_count * 8);
        if (o->det) {
            int g2 = (int)std::min<size_t>((nn * n_dmk + 255) / 256, (size_t)o->sm_count * 8);
            if (with_j) fx_to_double_kernel<<<grid, 256, 0, st>>>(o->jfx, nn * n_dm, o->jt);
            if (with_k) fx_to_double_kernel<<<g2, 256, 0, st>>>(o->kfx, nn * n_dmk, o->kt);
            launches += 2;
        }
        epilogue_kernel<<<grid, 256, 0, st>>>(o->jt, o->kt, n_dm, L, hermi, with_j, with_k, vj, vk);
        ++launches;
    }
    CK(cudaGetLastError());
    if (want_stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::vector<unsigned long long> cnt(4 * NQCLASS);
        o->last_flops.assign(2 * NQCLASS, 0);
        o->last_quartets.assign(2 * NQCLASS, 0);
        CK(cudaStreamSynchronize(st));
        CK(cudaMemcpy(cnt.data(), o->counters, sizeof(unsigned long long) * cnt.size(), cudaMemcpyDeviceToHost));
        for (int q = 0; q < NQCLASS; ++q) {
            const ClassEntry &e = g_tab[q];
            for (int prec = 0; prec < 2; ++prec) {
                int64_t nq = (int64_t)cnt[2 * (q + prec * NQCLASS)];
                int64_t np = (int64_t)cnt[2 * (q + prec * NQCLASS) + 1];
                int64_t fl = jk_flop_model(e.li, e.lj, e.lk, e.ll, nq, np, n_dm);
                o->last_flops[2 * q + prec] = fl;
                o->last_quartets[2 * q + prec] = nq;
                if (prec == 0) { stats->quartets_fp64 += nq; stats->prim_quartets_fp64 += np; stats->flops_fp64 += fl; }
                else { stats->quartets_fp32 += nq; stats->prim_quartets_fp32 += np; stats->flops_fp32 += fl; }
            }
        }
        stats->kernel_launches = launches;
        stats->n_classes = (int)o->plan_classes.size();
    }
    return 0;
}

int jk_build(jk_opt *o, const double *dm, int n_dm, int nao, int hermi, int with_j, int with_k, int precision,
             double split_thresh, double *vj, double *vk, void *stream, jk_stats *stats) {
    if (!o || o->nmol != 1 || nao != o->nao) return fail(JK_ERR_ARG, "jk_build: invalid arguments");
    return build_impl(o, dm, n_dm, hermi, with_j, with_k, precision, split_thresh, vj, vk, stream, stats);
}

int jk_build_batch(jk_opt *o, const double *dm, int n_dm, int hermi, int with_j, int with_k, int precision,
                   double split_thresh, double *vj, double *vk, void *stream, jk_stats *stats) {
    return build_impl(o, dm, n_dm, hermi, with_j, with_k, precision, split_thresh, vj, vk, stream, stats);
}

int jk_build_rsh(jk_opt *o, const double *dm, int n_dm, int nao, int hermi, int with_j, int with_k, double omega,
                 double lr_factor, double sr_factor, int precision, double split_thresh, double *vj, double *vk,
                 void *stream, jk_stats *stats) {
    if (!o || o->nmol != 1 || nao != o->nao) return fail(JK_ERR_ARG, "jk_build_rsh: invalid arguments");
    return build_impl(o, dm, n_dm, hermi, with_j, with_k, precision, split_thresh, vj, vk, stream, stats, omega,
                      lr_factor, sr_factor);
}

long long jk_opt_ntot(const jk_opt *o) { return o ? o->ntot : -1; }

// Nuclear gradient of the J/K energy through the dedicated derivative
// kernels (jk_grad.cu), with the optimizer's pair lists and its plan of
// work units.  The plan runs with the gradient's bound (products of two
// density blocks) in place of the J/K build's; the class kernels add their
// per-atom sums into ejk on the side streams.
int jk_energy_grad(jk_opt *o, const double *dm, int n_dm, int nao, double j_factor, double k_factor,
                   double omega, double lr_factor, double sr_factor, double *ejk, void *stream,
                   jk_stats *stats) {
    if (!o || !dm || !ejk || n_dm < 1 || n_dm > 2 || o->nmol != 1 || nao != o->nao)
        return fail(JK_ERR_ARG, "jk_energy_grad: invalid arguments");
    if (!std::isfinite(j_factor) || !std::isfinite(k_factor))
        return fail(JK_ERR_ARG, "jk_energy_grad: non-finite factors");
    if (o->lmax > GRAD_LMAX)
        return fail(JK_ERR_LMAX, "jk_energy_grad: shells above f are not supported by the gradient kernels");
    OpPass passes[2];
    const int npass = op_passes(omega, lr_factor, sr_factor, passes);
    if (npass < 0 || !std::isfinite(omega) || !std::isfinite(lr_factor) || !std::isfinite(sr_factor))
        return fail(JK_ERR_ARG, "jk_energy_grad: omega = 0 needs lr_factor == sr_factor");
    cudaStream_t st = (cudaStream_t)stream;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    CK(cudaMemsetAsync(ejk, 0, sizeof(double) * 3 * o->natm, st));
    if (npass == 0 || (j_factor == 0. && k_factor == 0.)) return 0;
    // weights of the density products (the reference's convention): 8-fold
    // permutation symmetry and the 1/2 of the Coulomb energy give 4 j_factor;
    // K takes (D_jk D_li + D_jl D_ki), and an RHF density (one matrix)
    // carries both spins, which halves k_factor
    const double jfac = 4. * j_factor;
    const double kfac = -2. * (n_dm == 1 ? .5 : 1.) * k_factor;
    const float log_j = jfac != 0. ? (float)(std::log(std::fabs(jfac)) + 2. * std::log((double)n_dm)) : -1e30f;
    const float log_k = kfac != 0. ? (float)(std::log(2. * std::fabs(kfac) * n_dm)) : -1e30f;
    const Layout L = layout_of(o);
    const int nb2 = o->nbas * o->nbas;
    dm_cond_kernel<<<(nb2 + 255) / 256, 256, 0, st>>>(dm, n_dm, L, o->shells, o->nbas, 1, o->dm_cond);
    max_kernel<<<1, 1024, 0, st>>>(o->dm_cond, nb2, o->dm_max);
    grad_bound_kernel<<<1, 1, 0, st>>>(o->dm_max, log_j, log_k, o->grad_max);
    const float log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
    if (o->nplan > 0) {
        plan_kernel<<<(o->plan_total + 255) / 256, 256, 0, st>>>(o->plan_dev, o->nplan, o->plan_total, o->grad_max,
                                                                 o->dm_cond, o->nbas, log_cut, 0.f, 0);
        scan_kernel<<<o->nscan, 1024, 0, st>>>(o->scan_dev);
    }
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(o->work, 0, sizeof(int) * 4 * NQCLASS, st));
    if (stats) CK(cudaMemsetAsync(o->counters, 0, sizeof(unsigned long long) * 4 * NQCLASS, st));
    EngineDev d = base_engine(o);
    d.dm_cond = o->dm_cond;
    d.log_cut = log_cut;
    d.counters = stats ? o->counters : nullptr;
    GradDev g;
    std::memset(&g, 0, sizeof(g));
    g.pp_e = o->pp_e;
    g.shell_atom = o->shell_atom;
    g.dm = dm;
    g.n_dm = n_dm;
    g.nao = nao;
    g.jfac = jfac;
    g.kfac = kfac;
    g.log_j = log_j;
    g.log_k = log_k;
    g.grad = ejk;
    CK(cudaEventRecord(o->fork_ev, st));
    for (int i = 0; i < jk_opt::NSIDE; ++i) CK(cudaStreamWaitEvent(o->side[i], o->fork_ev, 0));
    int nlaunched = 0;
    for (int ip = 0; ip < npass; ++ip) {
        d.omega2 = passes[ip].omega2;
        d.op_scale = passes[ip].scale;
        int *work = o->work + ip * 2 * NQCLASS;
        for (auto it = o->plan_classes.rbegin(); it != o->plan_classes.rend(); ++it) {
            const int q = *it;
            const ClassEntry &e = g_tab[q];
            int a = 0;
            while ((a + 1) * (a + 2) / 2 <= q) ++a;
            const int b = q - a * (a + 1) / 2;
            GradClass gc;
            if (grad_class(e.li, e.lj, e.lk, e.ll, &gc))
                return fail(JK_ERR_LMAX, "jk_energy_grad: class above the gradient kernels");
            ClassDev c;
            std::memset(&c, 0, sizeof(c));
            c.bra = PairList{o->npairs[a], o->pl_ij[a], o->pl_logq[a], o->pl_prim[a], o->pl_cnt[a]};
            c.ket = PairList{o->npairs[b], o->pl_ij[b], o->pl_logq[b], o->pl_prim[b], o->pl_cnt[b]};
            c.same = a == b;
            c.nbk = o->nbk[b];
            c.nx = o->npairs[a] * o->nbk[b];
            c.li = e.li; c.lj = e.lj; c.lk = e.lk; c.ll = e.ll;
            c.class_id = q;
            c.work = work + 2 * q;
            c.q_off = o->off64[q]; c.ket_begin = o->kb64[q]; c.ket_end = o->ke64[q];
            c.split_mode = SPLIT_ALL;
            g.qb = gc.qb;
            // one block per work unit at most; resident blocks of every SM
            const long long upper = (long long)o->npairs[a] * ((o->npairs[b] + JK_KCHUNK - 1) / JK_KCHUNK + o->nbk[b]);
            int per_sm = 0;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gc.kernel, JK_THREADS, (size_t)gc.smem));
            const int grid = (int)std::max<long long>(1, std::min<long long>(upper, (long long)o->sm_count * std::max(per_sm, 1)));
            cudaStream_t ls = o->side[nlaunched++ % jk_opt::NSIDE];
            void *args[] = {(void *)&d, (void *)&c, (void *)&g};
            CK(cudaLaunchKernel(gc.kernel, dim3(grid), dim3(JK_THREADS), args, (size_t)gc.smem, ls));
        }
    }
    for (int i = 0; i < jk_opt::NSIDE; ++i) {
        CK(cudaEventRecord(o->join_ev[i], o->side[i]));
        CK(cudaStreamWaitEvent(st, o->join_ev[i], 0));
    }
    CK(cudaGetLastError());
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::vector<unsigned long long> cnt(4 * NQCLASS);
        CK(cudaStreamSynchronize(st));
        CK(cudaMemcpy(cnt.data(), o->counters, sizeof(unsigned long long) * cnt.size(), cudaMemcpyDeviceToHost));
        for (int q = 0; q < NQCLASS; ++q) {
            stats->quartets_fp64 += (int64_t)cnt[2 * q];
            stats->prim_quartets_fp64 += (int64_t)cnt[2 * q + 1];
        }
        // density maxima (2), bound, plan and scan, and the class launches
        stats->kernel_launches = 3 + (o->nplan > 0 ? 2 : 0) + npass * (int)o->plan_classes.size();
        stats->n_classes = (int)o->plan_classes.size();
    }
    return 0;
}

int jk_opt_natm(const jk_opt *opt) { return opt ? opt->natm : -1; }

int jk_sparse_mm(int side, const int *ptr, const int *idx, const double *val, int n, int R, int K, int M,
                 const double *in, double *out, void *stream) {
    if ((side != 0 && side != 1) || !ptr || !idx || !val || !in || !out || n <= 0 || R <= 0 || K <= 0 || M <= 0)
        return fail(JK_ERR_ARG, "jk_sparse_mm: invalid arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const long long total = (long long)n * R * M;
    const int grid = (int)std::min<long long>((total + 255) / 256, 4096);
    if (side == 0)
        sparse_right_kernel<<<grid, 256, 0, st>>>(ptr, idx, val, total, K, M, in, out);
    else
        sparse_left_kernel<<<grid, 256, 0, st>>>(ptr, idx, val, total, R, K, M, in, out);
    CK(cudaGetLastError());
    return 0;
}

int jk_opt_set_mol_ndm(jk_opt *o, const int32_t *ndm) {
    if (!o) return fail(JK_ERR_ARG, "jk_opt_set_mol_ndm: null optimizer");
    if (!ndm) { o->use_mol_ndm = false; return 0; }
    for (int m = 0; m < o->nmol; ++m)
        if (ndm[m] < 0) return fail(JK_ERR_ARG, "jk_opt_set_mol_ndm: negative count");
    CK(cudaMemcpy(o->mol_ndm, ndm, sizeof(int) * o->nmol, cudaMemcpyHostToDevice));
    o->use_mol_ndm = true;
    return 0;
}

int jk_opt_set_deterministic(jk_opt *o, int enable) {
    if (!o) return fail(JK_ERR_ARG, "jk_opt_set_deterministic: null optimizer");
    o->det = enable != 0;
    return 0;
}

int jk_opt_set_variant(jk_opt *o, int q, int prec, int alt, int grid_per_sm) {
    if (!o || q < 0 || q >= NQCLASS || prec < 0 || prec > 1 || alt < 0 || alt > 1 || grid_per_sm < 0 || grid_per_sm > 64)
        return fail(JK_ERR_ARG, "jk_opt_set_variant: invalid arguments");
    o->variant_alt[2 * q + prec] = alt;
    o->variant_grid[2 * q + prec] = grid_per_sm;
    return 0;
}

int jk_opt_get_variant(const jk_opt *o, int q, int prec, int *alt, int *grid_per_sm) {
    if (!o || q < 0 || q >= NQCLASS || prec < 0 || prec > 1 || !alt || !grid_per_sm)
        return fail(JK_ERR_ARG, "jk_opt_get_variant: invalid arguments");
    *alt = o->variant_alt[2 * q + prec];
    *grid_per_sm = o->variant_grid[2 * q + prec];
    return 0;
}

// Autotuner: one regular build prepares the screening tables and work
// ranges for the caller's densities; then every class kernel is relaunched
// alone for each candidate (kernel family x grid of 1, 2, 4, 8 blocks per
// SM), timed with CUDA events (best of reps), and the fastest is kept.
// The internal accumulators are overwritten meanwhile; the caller's data is
// not touched.  Returns the number of (class, precision) entries tuned.
int jk_opt_tune(jk_opt *o, const double *dm, int n_dm, int hermi, int precision, double split_thresh,
                void *stream, int reps) {
    if (!o || !dm || n_dm <= 0 || reps <= 0) return fail(JK_ERR_ARG, "jk_opt_tune: invalid arguments");
    cudaStream_t st = (cudaStream_t)stream;
    double *vj = nullptr, *vk = nullptr;
    if (int e = dalloc(&vj, (size_t)o->ntot * n_dm)) return e;
    if (int e = dalloc(&vk, (size_t)o->ntot * n_dm)) { cudaFree(vj); return e; }
    const bool saved_timing = o->time_classes;
    o->time_classes = false;
    int err = build_impl(o, dm, n_dm, hermi, 1, 1, precision, split_thresh, vj, vk, stream, nullptr);
    o->time_classes = saved_timing;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int tuned = 0;
    if (!err && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        err = fail(JK_ERR_CUDA, "jk_opt_tune: event creation");
    const int mixed = precision != JK_PREC_FP64;
    EngineDev d = base_engine(o);
    d.dm_cond = o->dm_cond;
    d.dmj = o->dmj; d.dmk = o->dmk; d.dmj_f = o->dmj_f; d.dmk_f = o->dmk_f;
    d.vj = o->jt; d.vk = o->kt;
    d.n_dm = n_dm; d.n_dmk = hermi == 0 ? 2 * n_dm : n_dm;
    d.with_j = hermi != 2;
    d.with_k = 1;
    d.log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
    d.log_split = mixed ? (float)std::log(split_thresh) : 0.f;
    d.fp32_asym = precision == JK_PREC_MIXED_FP32ROOTS;
    static const int grids[4] = {1, 2, 4, 8};
    for (size_t t = 0; !err && t < o->plan_classes.size(); ++t) {
        const int q = o->plan_classes[t];
        const ClassEntry &e = g_tab[q];
        int a = 0;
        while ((a + 1) * (a + 2) / 2 <= q) ++a;
        const int b = q - a * (a + 1) / 2;
        ClassDev c;
        std::memset(&c, 0, sizeof(c));
        c.bra = PairList{o->npairs[a], o->pl_ij[a], o->pl_logq[a], o->pl_prim[a], o->pl_cnt[a]};
        c.ket = PairList{o->npairs[b], o->pl_ij[b], o->pl_logq[b], o->pl_prim[b], o->pl_cnt[b]};
        c.same = a == b;
        c.nbk = o->nbk[b];
        c.nx = o->npairs[a] * o->nbk[b];
        c.li = e.li; c.lj = e.lj; c.lk = e.lk; c.ll = e.ll;
        const long long upper = (long long)o->npairs[a] * ((o->npairs[b] + 127) / 128 + o->nbk[b]);
        for (int prec = 0; prec <= mixed && !err; ++prec) {
            c.class_id = prec ? NQCLASS + q : q;
            c.work = o->work + 2 * q + prec;
            c.q_off = prec ? o->off32[q] : o->off64[q];
            c.ket_begin = prec ? o->kb32[q] : o->kb64[q];
            c.ket_end = prec ? o->ke32[q] : o->ke64[q];
            c.split_mode = !mixed ? SPLIT_ALL : prec ? SPLIT_LOW : SPLIT_HIGH;
            float best = 1e30f;
            int best_alt = 0, best_grid = 0;
            for (int alt = 0; alt <= ((prec ? e.k32_alt : e.k64_alt) ? 1 : 0) && !err; ++alt)
                for (int gi = 0; gi < 4 && !err; ++gi) {
                    o->variant_alt[2 * q + prec] = alt;
                    o->variant_grid[2 * q + prec] = grids[gi];
                    float tmin = 1e30f;
                    for (int r = 0; r < reps && !err; ++r) {
                        float ms = 0.f;
                        if (cudaMemsetAsync(c.work, 0, sizeof(int), st) != cudaSuccess ||
                            cudaEventRecord(e0, st) != cudaSuccess) { err = fail(JK_ERR_CUDA, "jk_opt_tune: record"); break; }
                        if ((err = launch_variant(o, q, prec, upper, d, c, st))) break;
                        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { err = fail(JK_ERR_CUDA, "jk_opt_tune: timing"); break; }
                        tmin = std::min(tmin, ms);
                    }
                    if (tmin < best) { best = tmin; best_alt = alt; best_grid = grids[gi]; }
                }
            o->variant_alt[2 * q + prec] = best_alt;
            o->variant_grid[2 * q + prec] = best_grid;
            ++tuned;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(st);
    cudaFree(vj);
    cudaFree(vk);
    return err ? err : 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free J/K build.
//
// Some callers cannot call cudaMalloc at the moment they need a J/K build: a
// process running under a strict device-memory budget that forbids growth
// after start-up, or a plugin inside a host application whose own framework
// owns every device allocation.  jk_build grows its
// per-call workspace on demand; jk_build_noalloc instead takes every
// per-call buffer (density copies, J/K accumulators, screening table) from
// the fixed device array below, which each GPU that loads this library holds
// for the life of the process.  The optimizer itself must still be created
// beforehand with jk_opt_create, which does allocate.
// ---------------------------------------------------------------------------

#define JK_NOALLOC_SCRATCH_BYTES (32u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[JK_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int JK_NOALLOC_MAX_DEVICES = 64;
void *g_noalloc_addr[JK_NOALLOC_MAX_DEVICES] = {nullptr};
std::mutex g_noalloc_mu;

// Device address of the scratch array for the current device.  The host
// symbol g_noalloc_scratch is only a stand-in: its address must be resolved
// once per device, with that device current.
int noalloc_scratch(void **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= JK_NOALLOC_MAX_DEVICES) return fail(JK_ERR_ARG, "jk_build_noalloc: device index too large");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(JK_ERR_CUDA, std::string("jk_build_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return 0;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" int jk_noalloc_scratch_bytes(void) { return (int)JK_NOALLOC_SCRATCH_BYTES; }

extern "C" int jk_build_noalloc(jk_opt *o, const double *dm, int n_dm, int nao, int hermi, int with_j, int with_k,
                                int precision, double split_thresh, double *vj, double *vk, void *stream) {
    if (!o || !dm || n_dm <= 0 || o->nmol != 1 || nao != o->nao || hermi < 0 || hermi > 2 || (!with_j && !with_k))
        return fail(JK_ERR_ARG, "jk_build_noalloc: invalid arguments");
    if ((with_j && !vj) || (with_k && !vk)) return fail(JK_ERR_ARG, "jk_build_noalloc: missing output buffer");
    if (precision != JK_PREC_FP64 && precision != JK_PREC_MIXED && precision != JK_PREC_MIXED_FP32ROOTS)
        return fail(JK_ERR_ARG, "jk_build_noalloc: bad precision");
    if (precision != JK_PREC_FP64 && !(split_thresh > 0))
        return fail(JK_ERR_ARG, "jk_build_noalloc: split_thresh must be > 0");
    const int mixed = precision != JK_PREC_FP64;
    const size_t nn = (size_t)nao * nao;
    const int n_dmk = hermi == 0 ? 2 * n_dm : n_dm;
    // carve the scratch: dmj, dmk, jt, kt, [dmj_f, dmk_f], dm_cond, dm_max
    size_t off_dmj = 0;
    size_t off_dmk = off_dmj + align256(sizeof(double) * nn * n_dm);
    size_t off_jt = off_dmk + align256(sizeof(double) * nn * n_dmk);
    size_t off_kt = off_jt + align256(sizeof(double) * nn * n_dm);
    size_t off_dmjf = off_kt + align256(sizeof(double) * nn * n_dmk);
    size_t off_dmkf = off_dmjf + (mixed ? align256(sizeof(float) * nn * n_dm) : 0);
    size_t off_cond = off_dmkf + (mixed ? align256(sizeof(float) * nn * n_dmk) : 0);
    size_t off_max = off_cond + align256(sizeof(float) * (size_t)o->nbas * o->nbas);
    size_t off_work = off_max + 256;
    size_t need = off_work + align256(sizeof(int) * 2 * NQCLASS);
    if (need > JK_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "jk_build_noalloc: needs %zu bytes of scratch for nao=%d n_dm=%d, above the fixed %u bytes; "
                      "use jk_build", need, nao, n_dm, (unsigned)JK_NOALLOC_SCRATCH_BYTES);
        return fail(JK_ERR_OVERFLOW, msg);
    }
    void *base = nullptr;
    if (int e = noalloc_scratch(&base)) return e;
    unsigned char *b = (unsigned char *)base;
    double *dmj = (double *)(b + off_dmj), *dmk = (double *)(b + off_dmk);
    double *jt = (double *)(b + off_jt), *kt = (double *)(b + off_kt);
    float *dmj_f = mixed ? (float *)(b + off_dmjf) : nullptr;
    float *dmk_f = mixed ? (float *)(b + off_dmkf) : nullptr;
    float *dm_cond = (float *)(b + off_cond), *dm_max = (float *)(b + off_max);
    int *work = (int *)(b + off_work);
    cudaStream_t st = (cudaStream_t)stream;
    {
        int grid = (int)std::min<size_t>((nn * n_dm + 255) / 256, (size_t)o->sm_count * 8);
        prep_dm_kernel<<<grid, 256, 0, st>>>(dm, n_dm, layout_of(o), hermi, mixed, dmj, dmk, dmj_f, dmk_f);
        int nb2 = o->nbas * o->nbas;
        dm_cond_kernel<<<(nb2 + 255) / 256, 256, 0, st>>>(dm, n_dm, layout_of(o), o->shells, o->nbas, hermi, dm_cond);
        max_kernel<<<1, 1024, 0, st>>>(dm_cond, nb2, dm_max);
    }
    if (o->nplan > 0) {
        float log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
        float log_split = mixed ? (float)std::log(split_thresh) : 0.f;
        plan_kernel<<<(o->plan_total + 255) / 256, 256, 0, st>>>(o->plan_dev, o->nplan, o->plan_total, dm_max,
                                                                 dm_cond, o->nbas, log_cut, log_split, mixed);
        scan_kernel<<<o->nscan, 1024, 0, st>>>(o->scan_dev);
    }
    CK(cudaGetLastError());
    // the accumulators keep the previous call's contents: clear them
    CK(cudaMemsetAsync(jt, 0, sizeof(double) * nn * n_dm, st));
    CK(cudaMemsetAsync(kt, 0, sizeof(double) * nn * n_dmk, st));
    CK(cudaMemsetAsync(work, 0, sizeof(int) * 2 * NQCLASS, st));
    EngineDev d = base_engine(o);
    d.dm_cond = dm_cond;
    d.dmj = dmj; d.dmk = dmk; d.dmj_f = dmj_f; d.dmk_f = dmk_f;
    d.vj = jt; d.vk = kt;
    d.n_dm = n_dm; d.n_dmk = n_dmk;
    d.with_j = with_j && hermi != 2;
    d.with_k = with_k;
    d.log_cut = o->tol > 0 ? (float)std::log(o->tol) : -1e30f;
    d.log_split = mixed ? (float)std::log(split_thresh) : 0.f;
    d.fp32_asym = precision == JK_PREC_MIXED_FP32ROOTS;
    d.counters = nullptr;
    if (d.with_j || d.with_k) {
        // the optimizer's launch variants (autotuned or set), one class after
        // another on the caller's stream
        for (int q : o->plan_classes) {
            const ClassEntry &e = g_tab[q];
            int a = 0;
            while ((a + 1) * (a + 2) / 2 <= q) ++a;
            int bcls = q - a * (a + 1) / 2;
            ClassDev c;
            std::memset(&c, 0, sizeof(c));
            c.bra = PairList{o->npairs[a], o->pl_ij[a], o->pl_logq[a], o->pl_prim[a], o->pl_cnt[a]};
            c.ket = PairList{o->npairs[bcls], o->pl_ij[bcls], o->pl_logq[bcls], o->pl_prim[bcls], o->pl_cnt[bcls]};
            c.same = a == bcls;
            c.nbk = o->nbk[bcls];
            c.nx = o->npairs[a] * o->nbk[bcls];
            c.li = e.li; c.lj = e.lj; c.lk = e.lk; c.ll = e.ll;
            c.class_id = q;
            c.work = work + 2 * q;
            c.q_off = o->off64[q]; c.ket_begin = o->kb64[q]; c.ket_end = o->ke64[q];
            c.split_mode = mixed ? SPLIT_HIGH : SPLIT_ALL;
            long long upper = (long long)o->npairs[a] * ((o->npairs[bcls] + e.qb64 - 1) / e.qb64 + o->nbk[bcls]);
            if (int er = launch_variant(o, q, 0, upper, d, c, st)) return er;
            if (mixed) {
                c.class_id = NQCLASS + q;
                c.work = work + 2 * q + 1;
                c.q_off = o->off32[q]; c.ket_begin = o->kb32[q]; c.ket_end = o->ke32[q];
                c.split_mode = SPLIT_LOW;
                long long up32 = (long long)o->npairs[a] * ((o->npairs[bcls] + e.qb32 - 1) / e.qb32 + o->nbk[bcls]);
                if (int er = launch_variant(o, q, 1, up32, d, c, st)) return er;
            }
        }
    }
    {
        int grid = (int)std::min<size_t>((nn * n_dm + 255) / 256, (size_t)o->sm_count * 8);
        epilogue_kernel<<<grid, 256, 0, st>>>(jt, kt, n_dm, layout_of(o), hermi, with_j, with_k, vj, vk);
    }
    CK(cudaGetLastError());
    return 0;
}
