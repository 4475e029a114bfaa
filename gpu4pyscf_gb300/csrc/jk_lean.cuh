// Register-resident Rys J/K kernel for the small angular classes.
//
// One thread owns one shell quartet at a time, with no block barriers.  Per
// primitive quartet and root the 2D integrals of the three axes live in
// registers (fully unrolled vertical recurrence and horizontal transfers)
// and the Cartesian ERI block accumulates in registers.  Quartets differ in
// their primitive-pair counts, so lanes are refilled one by one: each warp
// iteration runs one primitive quartet on every busy lane, a lane whose
// quartet is complete stages its ERI block in shared memory and takes the
// next quartet from the warp's queue of screened (bra, ket) pairs, and the
// warp digests staged blocks 32 at a time (every lane one quartet: the six
// contractions with the density blocks, added to J and K with one atomic
// per element).  The FP64 pipe, GB300's scarcest, so sees full warps except
// at the very end of a launch.
#pragma once
#include "jk_device.cuh"
#include "rys_roots.cuh"

#define LEAN_THREADS 128

namespace jk {

__host__ __device__ constexpr int ctri(int c) {
    int t = 0;
    while ((t + 1) * (t + 2) / 2 <= c) ++t;
    return t;
}
// Cartesian component c of a shell of angular momentum l: lx, ly, lz
__host__ __device__ constexpr int cx_of(int l, int c) { return l - ctri(c); }
__host__ __device__ constexpr int cy_of(int l, int c) { return ctri(c) - (c - ctri(c) * (ctri(c) + 1) / 2); }
__host__ __device__ constexpr int cz_of(int l, int c) { return l - cx_of(l, c) - cy_of(l, c); }

template <int LI, int LJ, int LK, int LL>
struct LeanShape {
    static constexpr int NFI = ncart(LI), NFJ = ncart(LJ), NFK = ncart(LK), NFL = ncart(LL);
    static constexpr int NF = NFI * NFJ * NFK * NFL;
    static constexpr int NR = (LI + LJ + LK + LL) / 2 + 1;
    static constexpr int IJ = LI + LJ, KL = LK + LL;
    static constexpr int GSKL = (LK + 1) * (LL + 1);
    static constexpr int GS = (LI + 1) * (LJ + 1) * GSKL;
    static constexpr int COST = NF + 3 * GS;  // doubles held in registers
};

// 2D integrals of one axis for one root: g[((i*(LJ+1)+j)*(LK+1)+k)*(LL+1)+l]
template <int LI, int LJ, int LK, int LL, typename Real>
__device__ __forceinline__ void rys2d(Real i00, Real c00, Real cp00, Real b00, Real b10, Real b01, Real ab, Real cd,
                                      Real *g) {
    constexpr int IJ = LI + LJ, KL = LK + LL, GSKL = (LK + 1) * (LL + 1);
    Real v[KL + 1][IJ + 1];
#pragma unroll
    for (int n = 0; n <= IJ; ++n) {
        if (n == 0) v[0][0] = i00;
        else if (n == 1) v[0][1] = c00 * i00;
        else v[0][n] = c00 * v[0][n - 1] + Real(n - 1) * b10 * v[0][n - 2];
    }
#pragma unroll
    for (int m = 1; m <= KL; ++m)
#pragma unroll
        for (int n = 0; n <= IJ; ++n) {
            Real t = cp00 * v[m - 1][n];
            if (m > 1) t += Real(m - 1) * b01 * v[m - 2][n];
            if (n > 0) t += Real(n) * b00 * v[m - 1][n - 1];
            v[m][n] = t;
        }
    // bra transfer: h[m][j][i]
    Real h[KL + 1][LJ + 1][IJ + 1];
#pragma unroll
    for (int m = 0; m <= KL; ++m) {
#pragma unroll
        for (int n = 0; n <= IJ; ++n) h[m][0][n] = v[m][n];
#pragma unroll
        for (int j = 1; j <= LJ; ++j)
#pragma unroll
            for (int i = 0; i <= IJ - j; ++i) h[m][j][i] = h[m][j - 1][i + 1] + ab * h[m][j - 1][i];
    }
    // ket transfer
#pragma unroll
    for (int i = 0; i <= LI; ++i)
#pragma unroll
        for (int j = 0; j <= LJ; ++j) {
            Real t[LL + 1][KL + 1];
#pragma unroll
            for (int k = 0; k <= KL; ++k) t[0][k] = h[k][j][i];
#pragma unroll
            for (int l = 1; l <= LL; ++l)
#pragma unroll
                for (int k = 0; k <= KL - l; ++k) t[l][k] = t[l - 1][k + 1] + cd * t[l - 1][k];
#pragma unroll
            for (int k = 0; k <= LK; ++k)
#pragma unroll
                for (int l = 0; l <= LL; ++l) g[(i * (LJ + 1) + j) * GSKL + k * (LL + 1) + l] = t[l][k];
        }
}

// Atomic add aggregated over the lanes of a warp that target the same
// address: one atomic per distinct address (lanes with addr == nullptr add
// nothing).  The lanes' values are summed in the kernel's precision (for the
// FP32 quartets a sum of at most 32 FP32 integrals, within their own error)
// and converted once for the FP64 accumulator.  All 32 lanes must call it
// together.
template <typename Real>
__device__ __forceinline__ void warp_agg_add(double *addr, Real v, Real *buf, int lane) {
    const unsigned peers = __match_any_sync(0xffffffffu, (unsigned long long)addr);
    buf[lane] = v;
    __syncwarp();
    if (addr != nullptr && lane == __ffs(peers) - 1) {
        Real s = Real(0);
        unsigned m = peers;
        while (m) {
            s += buf[__ffs(m) - 1];
            m &= m - 1;
        }
        if (s != Real(0)) {
            if constexpr (sizeof(Real) == 4) atomicAdd(addr, widen_f32(s));
            else atomicAdd(addr, (double)s);
        }
    }
    __syncwarp();
}

template <typename Real> struct LeanIO;
template <> struct LeanIO<double> {
    static __device__ __forceinline__ const double *dj(const EngineDev &d) { return d.dmj; }
    static __device__ __forceinline__ const double *dk(const EngineDev &d) { return d.dmk; }
};
template <> struct LeanIO<float> {
    static __device__ __forceinline__ const float *dj(const EngineDev &d) { return d.dmj_f; }
    static __device__ __forceinline__ const float *dk(const EngineDev &d) { return d.dmk_f; }
};

// Finished quartets of a warp wait in shared memory until 32 of them can be
// digested together: their ERI blocks as [NF][LEAN_STAGE] (quartet index
// fastest, so the lanes of a warp hit consecutive banks) and their
// (bra, ket) indices.  LEAN_STAGE = 64 holds the at most 31 waiting plus 32
// newly finished quartets of one step.
#define LEAN_STAGE 64

template <int LI, int LJ, int LK, int LL, typename Real>
struct LeanSmem {
    static constexpr int NF = LeanShape<LI, LJ, LK, LL>::NF;
    static constexpr int WARPS = LEAN_THREADS / 32;
    static constexpr int BYTES = WARPS * LEAN_STAGE * (NF * (int)sizeof(Real) + (int)sizeof(int2));
};

// Adds v to *addr for every lane with a non-null addr.  FP64 quartets add
// lane by lane: the atomics resolve in L2 and cost the FP64 pipe nothing,
// where summing lanes first would.  FP32 quartets sum lanes that hit the same
// element in FP32 (warp aggregation) and convert once.  All 32 lanes call it.
// (In deterministic mode the FP32 quartets add lane by lane as well: a sum
// over the lanes would depend on which quartets share a warp.)
template <typename Real>
__device__ __forceinline__ void lean_add(const EngineDev &d, bool isk, double *addr, Real v, Real *buf, int lane) {
    if (sizeof(Real) == 8 || d.vj_fx != nullptr) {
        if (addr != nullptr) {
            if constexpr (sizeof(Real) == 4) jk_add(d, isk, addr, widen_f32(v));
            else jk_add(d, isk, addr, (double)v);
        }
    } else {
        warp_agg_add(addr, v, buf, lane);
    }
}

// Digestion of n staged quartets (lane l takes slot l < n; n >= 1): the six
// contractions of each quartet's ERI block with the density blocks it
// touches, added to J and K.
template <int LI, int LJ, int LK, int LL, typename Real>
__device__ __forceinline__ void lean_digest(const EngineDev &d, const ClassDev &c, const Real *st, const int2 *sq,
                                            int n, Real *aggbuf, int lane) {
    using S = LeanShape<LI, LJ, LK, LL>;
    constexpr int NFI = S::NFI, NFJ = S::NFJ, NFK = S::NFK, NFL = S::NFL;
    const bool valid = lane < n;
    const int2 q = sq[valid ? lane : 0];
    const int2 pij = c.bra.ij[q.x], pkl = c.ket.ij[q.y];
    const ShellDev &A = d.shells[pij.x];
    const int mol = A.mol;
    const int nao = __ldg(d.mol_nao + mol);
    const size_t nn = (size_t)d.ntot;
    const size_t mbase = (size_t)__ldg(d.mol_base + mol);
    const int ndm_m = d.mol_ndm ? __ldg(d.mol_ndm + mol) : d.n_dm;
    const Real fac = (sizeof(Real) == 8 ? Real(d.op_scale) : Real(d.op_scale_f)) *
                     Real((pij.x == pij.y ? .5f : 1.f) * (pkl.x == pkl.y ? .5f : 1.f) * (c.same && q.x == q.y ? .5f : 1.f));
    const int ai = A.ao, aj = d.shells[pij.y].ao;
    const int ak = d.shells[pkl.x].ao, al = d.shells[pkl.y].ao;
    const Real *E = st + lane;   // element e of this lane's quartet: E[e * LEAN_STAGE]
#define LEAN_E(a, b, cc, dd) E[((((a) * NFJ + (b)) * NFK + (cc)) * NFL + (dd)) * LEAN_STAGE]
    if (d.with_j) {
        for (int idm = 0; idm < d.n_dm; ++idm) {
            // densities the molecule does not carry are skipped
            const bool vd = valid && idm < ndm_m;
            if (!__any_sync(0xffffffffu, vd)) continue;
            const Real *Dm = LeanIO<Real>::dj(d) + idm * nn + mbase;
            double *V = d.vj + idm * nn + mbase;
            Real dkl[NFK * NFL], dij[NFI * NFJ];
#pragma unroll
            for (int cc = 0; cc < NFK; ++cc)
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) dkl[cc * NFL + dd] = Dm[(size_t)(ak + cc) * nao + al + dd];
#pragma unroll
            for (int a = 0; a < NFI; ++a)
#pragma unroll
                for (int b = 0; b < NFJ; ++b) dij[a * NFJ + b] = Dm[(size_t)(ai + a) * nao + aj + b];
#pragma unroll
            for (int a = 0; a < NFI; ++a)
#pragma unroll
                for (int b = 0; b < NFJ; ++b) {   // J[ij] += E D[kl]
                    Real s = Real(0);
#pragma unroll
                    for (int cc = 0; cc < NFK; ++cc)
#pragma unroll
                        for (int dd = 0; dd < NFL; ++dd) s += LEAN_E(a, b, cc, dd) * dkl[cc * NFL + dd];
                    lean_add(d, false, vd ? V + (size_t)(ai + a) * nao + aj + b : nullptr, fac * s, aggbuf, lane);
                }
#pragma unroll
            for (int cc = 0; cc < NFK; ++cc)
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) {   // J[kl] += E D[ij]
                    Real s = Real(0);
#pragma unroll
                    for (int a = 0; a < NFI; ++a)
#pragma unroll
                        for (int b = 0; b < NFJ; ++b) s += LEAN_E(a, b, cc, dd) * dij[a * NFJ + b];
                    lean_add(d, false, vd ? V + (size_t)(ak + cc) * nao + al + dd : nullptr, fac * s, aggbuf, lane);
                }
        }
    }
    if (d.with_k) {
        for (int idm = 0; idm < d.n_dmk; ++idm) {
            const bool vd = valid && (idm % d.n_dm) < ndm_m;
            if (!__any_sync(0xffffffffu, vd)) continue;
            const Real *Dm = LeanIO<Real>::dk(d) + idm * nn + mbase;
            double *V = d.vk + idm * nn + mbase;
            Real djl[NFJ * NFL], djk[NFJ * NFK], dil[NFI * NFL], dik[NFI * NFK];
#pragma unroll
            for (int b = 0; b < NFJ; ++b) {
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) djl[b * NFL + dd] = Dm[(size_t)(aj + b) * nao + al + dd];
#pragma unroll
                for (int cc = 0; cc < NFK; ++cc) djk[b * NFK + cc] = Dm[(size_t)(aj + b) * nao + ak + cc];
            }
#pragma unroll
            for (int a = 0; a < NFI; ++a) {
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) dil[a * NFL + dd] = Dm[(size_t)(ai + a) * nao + al + dd];
#pragma unroll
                for (int cc = 0; cc < NFK; ++cc) dik[a * NFK + cc] = Dm[(size_t)(ai + a) * nao + ak + cc];
            }
#pragma unroll
            for (int a = 0; a < NFI; ++a)
#pragma unroll
                for (int cc = 0; cc < NFK; ++cc) {   // K[i a, k c] += E D[j b, l d]
                    Real s = Real(0);
#pragma unroll
                    for (int b = 0; b < NFJ; ++b)
#pragma unroll
                        for (int dd = 0; dd < NFL; ++dd) s += LEAN_E(a, b, cc, dd) * djl[b * NFL + dd];
                    lean_add(d, true, vd ? V + (size_t)(ai + a) * nao + ak + cc : nullptr, fac * s, aggbuf, lane);
                }
#pragma unroll
            for (int a = 0; a < NFI; ++a)
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) {   // K[i a, l d] += E D[j b, k c]
                    Real s = Real(0);
#pragma unroll
                    for (int b = 0; b < NFJ; ++b)
#pragma unroll
                        for (int cc = 0; cc < NFK; ++cc) s += LEAN_E(a, b, cc, dd) * djk[b * NFK + cc];
                    lean_add(d, true, vd ? V + (size_t)(ai + a) * nao + al + dd : nullptr, fac * s, aggbuf, lane);
                }
#pragma unroll
            for (int b = 0; b < NFJ; ++b)
#pragma unroll
                for (int cc = 0; cc < NFK; ++cc) {   // K[j b, k c] += E D[i a, l d]
                    Real s = Real(0);
#pragma unroll
                    for (int a = 0; a < NFI; ++a)
#pragma unroll
                        for (int dd = 0; dd < NFL; ++dd) s += LEAN_E(a, b, cc, dd) * dil[a * NFL + dd];
                    lean_add(d, true, vd ? V + (size_t)(aj + b) * nao + ak + cc : nullptr, fac * s, aggbuf, lane);
                }
#pragma unroll
            for (int b = 0; b < NFJ; ++b)
#pragma unroll
                for (int dd = 0; dd < NFL; ++dd) {   // K[j b, l d] += E D[i a, k c]
                    Real s = Real(0);
#pragma unroll
                    for (int a = 0; a < NFI; ++a)
#pragma unroll
                        for (int cc = 0; cc < NFK; ++cc) s += LEAN_E(a, b, cc, dd) * dik[a * NFK + cc];
                    lean_add(d, true, vd ? V + (size_t)(aj + b) * nao + al + dd : nullptr, fac * s, aggbuf, lane);
                }
        }
    }
#undef LEAN_E
}

template <int LI, int LJ, int LK, int LL, typename Real>
__global__ void __launch_bounds__(LEAN_THREADS)
rys_lean_kernel(EngineDev d, ClassDev c, int unused)
{
    using S = LeanShape<LI, LJ, LK, LL>;
    constexpr int NR = S::NR, NF = S::NF, GS = S::GS;
    constexpr int NFI = S::NFI, NFJ = S::NFJ, NFK = S::NFK, NFL = S::NFL;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int WARPS = LEAN_THREADS / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    // Per warp: a queue of screened quartets (bra, ket) waiting for a lane,
    // the staging area of finished ERI blocks, and the buffer of the FP32
    // warp aggregation.
    __shared__ int2 queue[WARPS][64];
    __shared__ Real aggbuf[WARPS][32];
    extern __shared__ __align__(16) unsigned char lean_smem[];
    Real *stage = reinterpret_cast<Real *>(lean_smem) + (size_t)wid * NF * LEAN_STAGE;
    int2 *stage_q = reinterpret_cast<int2 *>(reinterpret_cast<Real *>(lean_smem) + (size_t)WARPS * NF * LEAN_STAGE) +
                    wid * LEAN_STAGE;
    // FP32: the Rys table block of this class in shared memory (the lanes'
    // T values fall in different intervals; global loads of the table would
    // cost one L1 wavefront per interval, shared loads one per instruction)
    constexpr bool F32 = sizeof(Real) == 4;
    __shared__ float s_rys[F32 ? rys_f_smem(NR) : 1];
    if constexpr (F32) {
        rys_stage_f<NR>(d.rys_coef_f, s_rys, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    int2 *wq = queue[wid];
    Real *ab_buf = aggbuf[wid];
    const int nunits = __ldg(c.q_off + c.nx);
    const int gwarp = (blockIdx.x * LEAN_THREADS + threadIdx.x) >> 5;
    if (gwarp > 0 && (long long)gwarp * JK_MIN_UNITS >= nunits) return;
    // (an eighth of the grid always stays, in case this build has far more
    // quartets than the last)
    // (FP32 launches keep their grid: their quartets are cheap and their
    // time is latency, which more warps hide)
    if (sizeof(Real) == 8 && gwarp >= (int)(gridDim.x * (LEAN_THREADS / 32)) / 8 && d.qprev != nullptr) {
        const unsigned long long prev = d.qprev[c.class_id];
        if (prev > 0 && (unsigned long long)gwarp * 32 * JK_Q_PER_LANE >= prev) return;
    }
    int kcur = 0, kend = 0, bcur = 0;
    bool exhausted = false;
    int nq = 0, nst = 0;
    // the lane's quartet: indices, primitive-pair offsets and counters,
    // centre differences and the ERI block accumulated so far
    bool has = false;
    int qb = 0, qk = 0, pb0 = 0, pk0 = 0, npk = 1, pbi = 0, pki = 0, left = 0;
    Real abx = 0, aby = 0, abz = 0, cdx = 0, cdy = 0, cdz = 0;
    Real acc[NF];
#pragma unroll
    for (int e = 0; e < NF; ++e) acc[e] = Real(0);
    while (true) {
        // ---- lanes without a quartet take the next ones from the queue,
        // which is refilled from work units (JK_KCHUNK kets of one
        // (bucket, bra) range, screened 32 at a time) as needed
        const unsigned empty = __ballot_sync(FULL, !has);
        if (empty) {
            const int need = __popc(empty);
            while (nq < need && !exhausted) {
                if (kcur >= kend) {
                    int w = 0;
                    if (lane == 0) w = atomicAdd(c.work, 1);
                    w = __shfl_sync(FULL, w, 0);
                    if (w >= nunits) { exhausted = true; break; }
                    int xw;
                    unit_at_warp(c, w, lane, xw, kcur, kend);
                    bcur = xw % c.bra.n;
                    continue;
                }
                const int kk = kcur + lane;
                const bool ok = kk < kend && pair_passes(d, c, bcur, kk);
                const unsigned m = __ballot_sync(FULL, ok);
                if (ok) wq[nq + __popc(m & lt)] = make_int2(bcur, kk);
                nq += __popc(m);
                kcur += 32;
                __syncwarp();
            }
            const int take = min(nq, need);
            const int rank = __popc(empty & lt);
            if (d.qnow != nullptr && lane == 0 && take > 0) atomicAdd(d.qnow + c.class_id, (unsigned long long)take);
            if (!has && rank < take) {
                const int2 e = wq[rank];
                qb = e.x;
                qk = e.y;
                const int2 pij = c.bra.ij[qb], pkl = c.ket.ij[qk];
                const ShellDev &A = d.shells[pij.x], &B = d.shells[pij.y];
                const ShellDev &C = d.shells[pkl.x], &D = d.shells[pkl.y];
                abx = Real(A.x - B.x); aby = Real(A.y - B.y); abz = Real(A.z - B.z);
                cdx = Real(C.x - D.x); cdy = Real(C.y - D.y); cdz = Real(C.z - D.z);
                pb0 = c.bra.prim_off[qb];
                pk0 = c.ket.prim_off[qk];
                const int npb = __ldg(c.bra.prim_cnt + qb);
                npk = __ldg(c.ket.prim_cnt + qk);
                left = npb * npk;
                pbi = 0;
                pki = 0;
#pragma unroll
                for (int k = 0; k < NF; ++k) acc[k] = Real(0);
                has = true;
                if (d.counters) {
                    atomicAdd(d.counters + 2 * c.class_id, 1ull);
                    atomicAdd(d.counters + 2 * c.class_id + 1, (unsigned long long)left);
                }
            }
            __syncwarp();
            if (nq > take) {   // drop the taken entries (at most 63 remain)
                const int rem = nq - take;
                const int2 t0 = lane < rem ? wq[take + lane] : make_int2(0, 0);
                const int2 t1 = lane + 32 < rem ? wq[take + 32 + lane] : make_int2(0, 0);
                __syncwarp();
                if (lane < rem) wq[lane] = t0;
                if (lane + 32 < rem) wq[lane + 32] = t1;
            }
            nq -= take;
            __syncwarp();
        }
        // an empty queue after the refill means the launch's units are
        // exhausted; the warp ends when its lanes have finished too
        if (!__any_sync(FULL, has)) break;

        // ---- one primitive quartet of every busy lane
        if (has) {
            const int pb = pb0 + pbi, pk = pk0 + pki;
            Real p, Px, Py, Pz, PAx, PAy, PAz, Kb, ipb;
            Real q, Qx, Qy, Qz, QCx, QCy, QCz, Kk, ipk;
            if constexpr (sizeof(Real) == 8) {
                const d4 a = d.pp_a[pb], b = d.pp_b[pb];
                p = a.x; Px = a.y; Py = a.z; Pz = a.w; PAx = b.x; PAy = b.y; PAz = b.z; Kb = b.w;
                ipb = d.pp_ip[pb];
                const d4 a2 = d.pp_a[pk], b2 = d.pp_b[pk];
                q = a2.x; Qx = a2.y; Qy = a2.z; Qz = a2.w; QCx = b2.x; QCy = b2.y; QCz = b2.z; Kk = b2.w;
                ipk = d.pp_ip[pk];
            } else {
                const float4 a = d.pp_af[pb], b = d.pp_bf[pb];
                p = a.x; Px = a.y; Py = a.z; Pz = a.w; PAx = b.x; PAy = b.y; PAz = b.z; Kb = b.w;
                ipb = d.pp_ipf[pb];
                const float4 a2 = d.pp_af[pk], b2 = d.pp_bf[pk];
                q = a2.x; Qx = a2.y; Qy = a2.z; Qz = a2.w; QCx = b2.x; QCy = b2.y; QCz = b2.z; Kk = b2.w;
                ipk = d.pp_ipf[pk];
            }
            Real rs, u[NR], w[NR];
            const Real PQx = Px - Qx, PQy = Py - Qy, PQz = Pz - Qz;
            if constexpr (sizeof(Real) == 8) {
                rs = rsqrt(p + q);
                const double rho = p * q * rs * rs;
                const double T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
                rys_roots_rs<NR>(T, rho, d.omega2, d.rys_coef, u, w);
            } else {
                rs = rsqrtf(p + q);
                const float rho = p * q * rs * rs;
                const float T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
                rys_roots_rs_f<NR, true>(T, rho, d.omega2_f, s_rys, u, w, d.fp32_asym);
            }
            const Real ipq = rs * rs;
            // the operator scale is applied once per quartet, at digestion
            const Real pref = Kb * Kk * rs;
            const Real qpq = q * ipq, ppq = p * ipq;
            const Real h2p = Real(0.5) * ipb, h2q = Real(0.5) * ipk, h2pq = Real(0.5) * ipq;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const Real ur = u[r];
                const Real b00 = ur * h2pq;
                const Real b10 = h2p - ur * h2p * qpq;
                const Real b01 = h2q - ur * h2q * ppq;
                const Real uq = qpq * ur, up = ppq * ur;
                Real gx[GS], gy[GS], gz[GS];
                rys2d<LI, LJ, LK, LL, Real>(Real(1), PAx - uq * PQx, QCx + up * PQx, b00, b10, b01, abx, cdx, gx);
                rys2d<LI, LJ, LK, LL, Real>(Real(1), PAy - uq * PQy, QCy + up * PQy, b00, b10, b01, aby, cdy, gy);
                rys2d<LI, LJ, LK, LL, Real>(w[r] * pref, PAz - uq * PQz, QCz + up * PQz, b00, b10, b01, abz, cdz, gz);
#pragma unroll
                for (int a = 0; a < NFI; ++a)
#pragma unroll
                    for (int b = 0; b < NFJ; ++b)
#pragma unroll
                        for (int cc = 0; cc < NFK; ++cc)
#pragma unroll
                            for (int dd = 0; dd < NFL; ++dd) {
                                const int ix = ((cx_of(LI, a) * (LJ + 1) + cx_of(LJ, b)) * (LK + 1) + cx_of(LK, cc)) * (LL + 1) + cx_of(LL, dd);
                                const int iy = ((cy_of(LI, a) * (LJ + 1) + cy_of(LJ, b)) * (LK + 1) + cy_of(LK, cc)) * (LL + 1) + cy_of(LL, dd);
                                const int iz = ((cz_of(LI, a) * (LJ + 1) + cz_of(LJ, b)) * (LK + 1) + cz_of(LK, cc)) * (LL + 1) + cz_of(LL, dd);
                                acc[((a * NFJ + b) * NFK + cc) * NFL + dd] += gx[ix] * gy[iy] * gz[iz];
                            }
            }
            if (++pki == npk) {
                pki = 0;
                ++pbi;
            }
            --left;
        }

        // ---- finished quartets: stage their ERI blocks; digest 32 at a time
        const bool done = has && left == 0;
        const unsigned fin = __ballot_sync(FULL, done);
        if (fin) {
            if (done) {
                const int slot = nst + __popc(fin & lt);
#pragma unroll
                for (int e = 0; e < NF; ++e) stage[e * LEAN_STAGE + slot] = acc[e];
                stage_q[slot] = make_int2(qb, qk);
                has = false;
            }
            nst += __popc(fin);
            __syncwarp();
            if (nst >= 32) {
                lean_digest<LI, LJ, LK, LL, Real>(d, c, stage, stage_q, 32, ab_buf, lane);
                __syncwarp();
                const int rem = nst - 32;   // at most 31: move them to the front
                if (lane < rem) {
#pragma unroll
                    for (int e = 0; e < NF; ++e) stage[e * LEAN_STAGE + lane] = stage[e * LEAN_STAGE + 32 + lane];
                    stage_q[lane] = stage_q[32 + lane];
                }
                nst = rem;
                __syncwarp();
            }
        }
    }
    if (nst > 0) lean_digest<LI, LJ, LK, LL, Real>(d, c, stage, stage_q, nst, ab_buf, lane);
}

}  // namespace jk
