// Device side of the GB300 Rys J/K engine: data layout shared by the host
// driver and the per-class kernel template.
//
// One kernel instantiation per angular class (li,lj|lk,ll) with li>=lj,
// lk>=ll and class(ij) >= class(kl), in FP64 or FP32.  A block of 256
// threads works on QB shell quartets that share the bra pair; each quartet
// is owned by G threads.  Per primitive quartet the block runs three
// stages separated by barriers:
//   S1  one thread per quartet: Rys roots and weights (table Horner or
//       Gauss-Hermite asymptote), prefactor and recurrence scalars -> smem;
//   S2  one thread per (quartet, root, axis): 2D integrals by the vertical
//       recurrence with the bra horizontal transfer done column by column in
//       registers, then the ket horizontal transfer in place -> smem;
//   S3  every thread: its slice of the Cartesian ERI block accumulates
//       sum_r gx*gy*gz in registers.
// After the primitive loop the block stages the contracted ERIs in shared
// memory and forms the six J/K contractions, one output element per thread,
// with one FP64 atomic add per element (instead of one per ERI and
// contraction).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// highest angular momentum of the engine (g); the templated kernels cover
// classes up to f, classes with a g shell run the generic kernel
#define JK_LMAX 4
#define JK_LMAX_TEMPLATED 3
#define JK_THREADS 256
#define JK_SMEM_CAP (100 * 1024)

namespace jk {

struct __align__(32) d4 { double x, y, z, w; };

struct ShellDev {
    double x, y, z;
    int l, nprim;
    int ao;    // first Cartesian AO within the shell's molecule
    int mol;   // molecule of the shell (0 for a single molecule)
};

// one pair class (li, lj) with pairs sorted by Schwarz factor, descending
struct PairList {
    int n;
    const int2 *ij;        // shell indices (i >= j)
    const float *logq;     // log sqrt(max |(ij|ij)|)
    const int *prim_off;   // first primitive pair
    const int *prim_cnt;   // primitive pairs kept for the pair
};

struct EngineDev {
    const ShellDev *shells;
    // primitive-pair data, one entry per primitive pair of every kept shell pair
    const d4 *pp_a;        // {p, Px, Py, Pz}
    const d4 *pp_b;        // {PAx, PAy, PAz, sqrt(2 pi^(5/2)) Kab ci cj / p}   (A = first shell)
    const double *pp_ip;      // 1/p
    const float4 *pp_af;      // float copies for the FP32 quartets
    const float4 *pp_bf;
    const float *pp_ipf;
    const float *dm_cond;     // [nbas*nbas] log absmax of the density blocks
    const double *rys_coef;   // Rys interpolation table
    const float *rys_coef_f;
    const double *dmj;        // [n_dm][nao][nao]  D + D^T
    const double *dmk;        // [n_dmk][nao][nao] densities for K
    const float *dmj_f;       // float copies (FP32 quartets)
    const float *dmk_f;
    double *vj;               // J accumulator, symmetrised later
    double *vk;               // K accumulator
    float *qout;              // Schwarz mode output (per pair)
    unsigned long long *counters;  // per class: [quartets, prim quartets]
    // launch sizing from the optimizer's history: quartets each class launch
    // (index class_id) computed in the previous build (null: none) and the
    // counts of this build
    const unsigned long long *qprev;
    unsigned long long *qnow;
    // deterministic accumulation (non-null when enabled): J and K elements
    // as pairs of 64-bit fixed-point sums [2 * element] (see jk_add)
    unsigned long long *vj_fx, *vk_fx;
    int nbas, nao, n_dm, n_dmk;
    // densities and J/K are stored per molecule as packed square blocks:
    // element (a, b) of molecule m in density idm sits at
    // idm * ntot + mol_base[m] + a * mol_nao[m] + b
    long long ntot;
    const long long *mol_base;
    const int *mol_nao;
    const int *mol_ndm;       // densities each molecule carries (null: all n_dm)
    int with_j, with_k;
    float log_cut;
    float log_split;          // mixed builds: log of the FP64/FP32 split threshold
    int fp32_asym;            // 1: FP32 quartets take the large-T asymptote in FP32 too
    // range separation: omega2 = omega^2 > 0 evaluates erf(omega r)/r instead
    // of 1/r (rys_roots_rs); op_scale multiplies every integral (a negative
    // scale subtracts a long-range pass from a full-range one)
    double omega2, op_scale;
    float omega2_f, op_scale_f;
};

// Work of one quartet class.  The ket list is split into buckets of equal
// primitive-pair count (each bucket sorted by Schwarz factor, descending);
// x = bucket * bra.n + bra indexes the ket range [ket_begin[x], ket_end[x]),
// and each range is cut into work units of JK_KCHUNK kets numbered through
// the class (range x holds units q_off[x] .. q_off[x+1]-1), so consecutive
// units share primitive counts.
struct ClassDev {
    PairList bra, ket;
    int same;                 // bra list == ket list
    int class_id;
    int nbk;                  // ket buckets
    int nx;                   // bra.n * nbk
    const int *q_off;         // [nx + 1] work-unit offsets (units of JK_KCHUNK kets)
    const int *ket_begin;     // [nx]
    const int *ket_end;       // [nx]
    int *work;                // range counter of this launch (zeroed per build)
    // which screened quartets of the ranges this launch computes:
    // SPLIT_ALL every one, SPLIT_HIGH those whose bound reaches the split
    // (FP64 part of a mixed build), SPLIT_LOW those below it (FP32 part)
    int split_mode;
    int li, lj, lk, ll;       // angular momenta of the class (read by the generic kernel)
};

enum { SPLIT_ALL = 0, SPLIT_HIGH = 1, SPLIT_LOW = 2 };

// Screening of (bra, ket) of a class: q_ij q_kl times the largest of the six
// density blocks the quartet touches against the cutoff
// (gpu4pyscf/lib/gvhf-rys/create_tasks.cu:152-162).  A J-only build needs
// only the two Coulomb blocks D_ij and D_kl (the screening of the
// reference's J engine), which drops far more quartets of a sparse density.
// In a mixed build the same bound, the quartet's own, decides its
// precision: FP64 when it reaches the split threshold, FP32 below it.
__device__ __forceinline__ bool pair_passes(const EngineDev &d, const ClassDev &c, int bra, int ket) {
    const int2 pij = c.bra.ij[bra], pkl = c.ket.ij[ket];
    const float *dc = d.dm_cond;
    const int nb = d.nbas;
    float dmax = fmaxf(__ldg(dc + pij.x * nb + pij.y), __ldg(dc + pkl.x * nb + pkl.y));
    if (d.with_k)
        dmax = fmaxf(dmax, fmaxf(fmaxf(__ldg(dc + pij.x * nb + pkl.x), __ldg(dc + pij.x * nb + pkl.y)),
                                 fmaxf(__ldg(dc + pij.y * nb + pkl.x), __ldg(dc + pij.y * nb + pkl.y))));
    const float v = __ldg(c.bra.logq + bra) + __ldg(c.ket.logq + ket) + dmax;
    if (!(v >= d.log_cut)) return false;
    if (c.split_mode == SPLIT_HIGH) return v >= d.log_split;
    if (c.split_mode == SPLIT_LOW) return v < d.log_split;
    return true;
}

// float -> double on the integer pipe: the exponent rebiased, the
// significand shifted into place (normal numbers exactly; zero and FP32
// denormals, below 1.2e-38, become 0).  GB300 runs the F2F conversion
// instruction on its FP64 pipe, the scarce one, which the FP32 quartets
// would otherwise spend on every contribution they add to J and K.
__device__ __forceinline__ double widen_f32(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    const unsigned lo = u << 29;
    return ex == 0u ? 0. : __hiloint2double((int)hi, (int)lo);
}

// Adds v to J (isk false) or K element *addr.  Default: one FP64 atomic.
// Deterministic mode: v = a 2^-24 + b 2^-56 (a = rint(v 2^24), b the
// rounded remainder, |b| <= 2^31) goes into two 64-bit integer sums per
// element; integer addition does not depend on the order of the atomics, so
// the result is bitwise reproducible (rounding error <= 2^-57 per
// contribution).
#define JK_FX_HI 0x1p24
#define JK_FX_LO 0x1p56
__device__ __forceinline__ void jk_add(const EngineDev &d, bool isk, double *addr, double v) {
    unsigned long long *fx = isk ? d.vk_fx : d.vj_fx;
    if (fx == nullptr) {
        atomicAdd(addr, v);
        return;
    }
    const size_t off = addr - (isk ? d.vk : d.vj);
    const double a = rint(v * JK_FX_HI);
    const double r = fma(-a, 1. / JK_FX_HI, v);
    atomicAdd(fx + 2 * off, (unsigned long long)__double2ll_rn(a));
    atomicAdd(fx + 2 * off + 1, (unsigned long long)__double2ll_rn(r * JK_FX_LO));
}

// kets per work unit: a range [ket_begin[x], ket_end[x]) is cut into units
// of JK_KCHUNK kets, numbered through the class by q_off (unit prefix sums)
#define JK_KCHUNK 64

// work unit w -> range x and its ket interval [k0, k1), found by the 32
// lanes of a warp together (all must call it with the same w): each step
// probes 32 evenly spaced unit offsets with one load per lane and keeps the
// interval between the last offset <= w and the next, so a search over nx
// ranges takes log32(nx) dependent loads instead of log2(nx).
__device__ __forceinline__ void unit_at_warp(const ClassDev &c, int w, int lane, int &x, int &k0, int &k1) {
    int lo = 0, hi = c.nx;   // q_off[lo] <= w < q_off[hi]
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) >> 5;
        const int p = lo + lane * step;
        const bool le = p < hi && __ldg(c.q_off + p) <= w;
        const unsigned m = __ballot_sync(0xffffffffu, le);
        const int t = 31 - __clz(m);   // lane 0 probes lo, so m != 0
        lo += t * step;
        hi = min(hi, lo + step);
    }
    x = lo;
    k0 = __ldg(c.ket_begin + lo) + (w - __ldg(c.q_off + lo)) * JK_KCHUNK;
    k1 = min(__ldg(c.ket_end + lo), k0 + JK_KCHUNK);
}

// A launch's warps (lean family) or blocks (cooperative family) beyond one
// per JK_MIN_UNITS work units return at once: in classes with little work
// the remaining ones then run full warps instead of many warps with a few
// quartets each.
#define JK_MIN_UNITS 8

// With the previous build's count of a launch's quartets at hand, a launch
// keeps enough warps (blocks) for about JK_Q_PER_LANE quartets per lane (per
// slot): classes whose kets mostly fail the density screening otherwise
// spread a few quartets over thousands of warps.
#define JK_Q_PER_LANE 4

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Threads per quartet and quartets per block for a class.
template <int LI, int LJ, int LK, int LL, typename Real>
struct ClassShape {
    static constexpr int NFI = ncart(LI), NFJ = ncart(LJ), NFK = ncart(LK), NFL = ncart(LL);
    static constexpr int NF = NFI * NFJ * NFK * NFL;
    static constexpr int NR = (LI + LJ + LK + LL) / 2 + 1;
    static constexpr int IJ = LI + LJ, KL = LK + LL;
    static constexpr int GSKL = (LK + 1) * (LL + 1);
    static constexpr int GS = (LI + 1) * (LJ + 1) * GSKL;   // 2D integrals per (root, axis)
    static constexpr int NSC = 20;                            // per-quartet scalars
    // per (quartet, root): u, w * prefactor and the axis-independent
    // recurrence coefficients b00, b10, b01, u q/(p+q), u p/(p+q)
    static constexpr int NRW = 7;
    __host__ __device__ static constexpr int g_bytes(int qb) { return qb * NR * 3 * GS * (int)sizeof(Real); }
    __host__ __device__ static constexpr int e_bytes(int qb) { return qb * NF * (int)sizeof(Real); }
    __host__ __device__ static constexpr int aux_bytes(int qb) { return qb * (NR * NRW + NSC) * (int)sizeof(Real); }
    __host__ __device__ static constexpr int smem_of(int g) {
        return (g_bytes(JK_THREADS / g) > e_bytes(JK_THREADS / g) ? g_bytes(JK_THREADS / g) : e_bytes(JK_THREADS / g))
               + aux_bytes(JK_THREADS / g);
    }
    __host__ __device__ static constexpr int pick_g() {
        int g = 1;
        while (g * 40 < NF && g < JK_THREADS) g *= 2;
        while (smem_of(g) > JK_SMEM_CAP && g < JK_THREADS) g *= 2;
        return g;
    }
    static constexpr int G = pick_g();
    static constexpr int QB = JK_THREADS / G;
    static constexpr int NPT = (NF + G - 1) / G;
    static constexpr int SMEM = smem_of(G);
};

}  // namespace jk
