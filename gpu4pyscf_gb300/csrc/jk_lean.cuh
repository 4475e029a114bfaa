// Register-resident Rys J/K kernel for the small angular classes.
//
// One thread owns one shell quartet from start to end, with no block
// barriers.  Each warp takes (ket bucket, bra) ranges from a work counter,
// screens their kets and queues the survivors, so its 32 lanes run 32
// quartets with the same ket primitive count at a time.  Per primitive quartet and root the
// 2D integrals of the three axes live in registers (fully unrolled vertical
// recurrence and horizontal transfers), the Cartesian ERI block accumulates
// in registers, and after the primitive loops the thread contracts its block
// with the six density blocks.  The J block of the bra pair, common to the
// warp when all its lanes share the bra pair, is summed across the warp with
// shuffles before one atomic add per element; the four K blocks go out with
// one atomic add per distinct address of the warp, J_kl directly.
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
        if (s != Real(0)) atomicAdd(addr, (double)s);
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

template <int LI, int LJ, int LK, int LL, typename Real>
__global__ void __launch_bounds__(LEAN_THREADS)
rys_lean_kernel(EngineDev d, ClassDev c, int unused)
{
    using S = LeanShape<LI, LJ, LK, LL>;
    constexpr int NR = S::NR, NF = S::NF, GS = S::GS, GSKL = S::GSKL;
    constexpr int NFI = S::NFI, NFJ = S::NFJ, NFK = S::NFK, NFL = S::NFL;
    const int lane = threadIdx.x & 31;
    // Per-warp work: the warp takes work units (JK_KCHUNK kets of one
    // (bucket, bra) range) from the launch's counter, screens their kets 32 at
    // a time and queues the quartets that pass; each iteration runs 32 queued
    // quartets.
    __shared__ int2 queue[LEAN_THREADS / 32][64];
    __shared__ Real aggbuf[LEAN_THREADS / 32][32];
    // FP32: the Rys table block of this class in shared memory (the lanes'
    // T values fall in different intervals; global loads of the table would
    // cost one L1 wavefront per interval, shared loads one per instruction)
    constexpr bool F32 = sizeof(Real) == 4;
    __shared__ float s_rys[F32 ? rys_f_smem(NR) : 1];
    if constexpr (F32) {
        rys_stage_f<NR>(d.rys_coef_f, s_rys, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    int2 *wq = queue[threadIdx.x >> 5];
    Real *ab_buf = aggbuf[threadIdx.x >> 5];
    const int nunits = __ldg(c.q_off + c.nx);
    int kcur = 0, kend = 0, bcur = 0;
    bool exhausted = false;
    int nq = 0;
    while (true) {
        while (nq < 32 && !exhausted) {
            if (kcur >= kend) {
                int w = 0;
                if (lane == 0) w = atomicAdd(c.work, 1);
                w = __shfl_sync(0xffffffffu, w, 0);
                if (w >= nunits) { exhausted = true; break; }
                int xw;
                unit_at(c, w, xw, kcur, kend);
                bcur = xw % c.bra.n;
                continue;
            }
            const int kk = kcur + lane;
            const bool ok = kk < kend && pair_passes(d, c, bcur, kk);
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) wq[nq + __popc(m & ((1u << lane) - 1u))] = make_int2(bcur, kk);
            nq += __popc(m);
            kcur += 32;
            __syncwarp();
        }
        if (nq == 0) break;
        const int take = min(nq, 32);
        const int2 mine = lane < take ? wq[lane] : make_int2(-1, -1);
        __syncwarp();
        if (nq > 32) {
            int2 t = lane < nq - 32 ? wq[32 + lane] : make_int2(0, 0);
            __syncwarp();
            if (lane < nq - 32) wq[lane] = t;
        }
        nq -= take;
        __syncwarp();
        const bool valid = mine.x >= 0;
        // lane 0 always holds a quartet; idle lanes borrow its indices
        const int lead_b = __shfl_sync(0xffffffffu, mine.x, 0);
        const int lead_k = __shfl_sync(0xffffffffu, mine.y, 0);
        const int ib = valid ? mine.x : lead_b;
        const int ket = valid ? mine.y : lead_k;
        const int2 pij = c.bra.ij[ib];
        int2 pkl = make_int2(0, 0);
        if (valid) pkl = c.ket.ij[ket];
        // the J block of the bra pair can be summed across the warp when all
        // its lanes share the bra
        const bool same_bra = __all_sync(0xffffffffu, ib == __shfl_sync(0xffffffffu, ib, 0));
        Real acc[NF];
#pragma unroll
        for (int e = 0; e < NF; ++e) acc[e] = Real(0);
        const ShellDev &A = d.shells[pij.x], &B = d.shells[pij.y];
        const int npb = __ldg(c.bra.prim_cnt + ib);
        const int pb0 = c.bra.prim_off[ib];
        int npk = 0, pk0 = 0;
        Real abx = Real(A.x - B.x), aby = Real(A.y - B.y), abz = Real(A.z - B.z);
        Real cdx = 0, cdy = 0, cdz = 0;
        if (valid) {
            const ShellDev &C = d.shells[pkl.x], &D = d.shells[pkl.y];
            npk = __ldg(c.ket.prim_cnt + ket);
            pk0 = c.ket.prim_off[ket];
            cdx = Real(C.x - D.x); cdy = Real(C.y - D.y); cdz = Real(C.z - D.z);
            if (d.counters) {
                atomicAdd(d.counters + 2 * c.class_id, 1ull);
                atomicAdd(d.counters + 2 * c.class_id + 1, (unsigned long long)(npb * npk));
            }
        }
        for (int pb = 0; pb < npb; ++pb) {
            Real p, Px, Py, Pz, PAx, PAy, PAz, Kb, ipb;
            if constexpr (sizeof(Real) == 8) {
                d4 a = d.pp_a[pb0 + pb], b = d.pp_b[pb0 + pb];
                p = a.x; Px = a.y; Py = a.z; Pz = a.w; PAx = b.x; PAy = b.y; PAz = b.z; Kb = b.w;
                ipb = d.pp_ip[pb0 + pb];
            } else {
                float4 a = d.pp_af[pb0 + pb], b = d.pp_bf[pb0 + pb];
                p = a.x; Px = a.y; Py = a.z; Pz = a.w; PAx = b.x; PAy = b.y; PAz = b.z; Kb = b.w;
                ipb = d.pp_ipf[pb0 + pb];
            }
            for (int pk = 0; pk < npk; ++pk) {
                Real q, Qx, Qy, Qz, QCx, QCy, QCz, Kk, ipk;
                if constexpr (sizeof(Real) == 8) {
                    d4 a = d.pp_a[pk0 + pk], b = d.pp_b[pk0 + pk];
                    q = a.x; Qx = a.y; Qy = a.z; Qz = a.w; QCx = b.x; QCy = b.y; QCz = b.z; Kk = b.w;
                    ipk = d.pp_ip[pk0 + pk];
                } else {
                    float4 a = d.pp_af[pk0 + pk], b = d.pp_bf[pk0 + pk];
                    q = a.x; Qx = a.y; Qy = a.z; Qz = a.w; QCx = b.x; QCy = b.y; QCz = b.z; Kk = b.w;
                    ipk = d.pp_ipf[pk0 + pk];
                }
                Real rs, u[NR], w[NR];
                const Real PQx = Px - Qx, PQy = Py - Qy, PQz = Pz - Qz;
                if constexpr (sizeof(Real) == 8) {
                    rs = rsqrt(p + q);
                    const double rho = p * q * rs * rs;
                    double T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
                    rys_roots_rs<NR>(T, rho, d.omega2, d.rys_coef, u, w);
                } else {
                    rs = rsqrtf(p + q);
                    const float rho = p * q * rs * rs;
                    float T = rho * (PQx * PQx + PQy * PQy + PQz * PQz);
                    rys_roots_rs_f<NR, true>(T, rho, d.omega2_f, s_rys, u, w, d.fp32_asym);
                }
                const Real ipq = rs * rs;
                const Real pref = Real(34.98683665524972497) * Kb * Kk * ipb * ipk * rs *
                                  (sizeof(Real) == 8 ? Real(d.op_scale) : Real(d.op_scale_f));
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
                                    constexpr int dummy = 0;
                                    (void)dummy;
                                    const int ix = ((cx_of(LI, a) * (LJ + 1) + cx_of(LJ, b)) * (LK + 1) + cx_of(LK, cc)) * (LL + 1) + cx_of(LL, dd);
                                    const int iy = ((cy_of(LI, a) * (LJ + 1) + cy_of(LJ, b)) * (LK + 1) + cy_of(LK, cc)) * (LL + 1) + cy_of(LL, dd);
                                    const int iz = ((cz_of(LI, a) * (LJ + 1) + cz_of(LJ, b)) * (LK + 1) + cz_of(LK, cc)) * (LL + 1) + cz_of(LL, dd);
                                    acc[((a * NFJ + b) * NFK + cc) * NFL + dd] += gx[ix] * gy[iy] * gz[iz];
                                }
                }
            }
        }
        // ---- digestion ----
        const int mol = A.mol;
        const int nao = __ldg(d.mol_nao + mol);
        const size_t nn = (size_t)d.ntot;
        const size_t mbase = (size_t)__ldg(d.mol_base + mol);
        const int ndm_m = d.mol_ndm ? __ldg(d.mol_ndm + mol) : d.n_dm;
        const Real fac = Real((pij.x == pij.y ? .5 : 1.) * (pkl.x == pkl.y ? .5 : 1.) *
                              (c.same && ib == ket ? .5 : 1.));
        const int ai = A.ao, aj = B.ao;
        const int ak = valid ? d.shells[pkl.x].ao : 0, al = valid ? d.shells[pkl.y].ao : 0;
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
                    for (int dd = 0; dd < NFL; ++dd)
                        dkl[cc * NFL + dd] = vd ? Dm[(size_t)(ak + cc) * nao + al + dd] : Real(0);
#pragma unroll
                for (int a = 0; a < NFI; ++a)
#pragma unroll
                    for (int b = 0; b < NFJ; ++b) dij[a * NFJ + b] = Dm[(size_t)(ai + a) * nao + aj + b];
                // J[ij] += sum_kl E D[kl]: same bra for the warp -> shuffle reduction
#pragma unroll
                for (int ab = 0; ab < NFI * NFJ; ++ab) {
                    Real s = Real(0);
#pragma unroll
                    for (int cd = 0; cd < NFK * NFL; ++cd) s += acc[ab * NFK * NFL + cd] * dkl[cd];
                    // (summed across the warp in the kernel's precision,
                    // converted once for the FP64 accumulator)
                    Real sd = vd ? fac * s : Real(0);
                    double *dst = V + (size_t)(ai + ab / NFJ) * nao + aj + ab % NFJ;
                    if (same_bra) {
#pragma unroll
                        for (int off = 16; off > 0; off >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, off);
                        if (lane == 0 && sd != Real(0)) atomicAdd(dst, (double)sd);
                    } else if (vd) {
                        atomicAdd(dst, (double)sd);
                    }
                }
                if (vd) {
#pragma unroll
                    for (int cd = 0; cd < NFK * NFL; ++cd) {
                        Real s = Real(0);
#pragma unroll
                        for (int ab = 0; ab < NFI * NFJ; ++ab) s += acc[ab * NFK * NFL + cd] * dij[ab];
                        atomicAdd(V + (size_t)(ak + cd / NFL) * nao + al + cd % NFL, (double)(fac * s));
                    }
                }
            }
        }
        if (d.with_k) {
            // lanes whose kets share a shell hit the same K elements: add
            // through warp aggregation (idle lanes contribute nothing)
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
                            for (int dd = 0; dd < NFL; ++dd) s += acc[((a * NFJ + b) * NFK + cc) * NFL + dd] * djl[b * NFL + dd];
                        warp_agg_add(vd ? V + (size_t)(ai + a) * nao + ak + cc : nullptr, fac * s, ab_buf, lane);
                    }
#pragma unroll
                for (int a = 0; a < NFI; ++a)
#pragma unroll
                    for (int dd = 0; dd < NFL; ++dd) {   // K[i a, l d] += E D[j b, k c]
                        Real s = Real(0);
#pragma unroll
                        for (int b = 0; b < NFJ; ++b)
#pragma unroll
                            for (int cc = 0; cc < NFK; ++cc) s += acc[((a * NFJ + b) * NFK + cc) * NFL + dd] * djk[b * NFK + cc];
                        warp_agg_add(vd ? V + (size_t)(ai + a) * nao + al + dd : nullptr, fac * s, ab_buf, lane);
                    }
#pragma unroll
                for (int b = 0; b < NFJ; ++b)
#pragma unroll
                    for (int cc = 0; cc < NFK; ++cc) {   // K[j b, k c] += E D[i a, l d]
                        Real s = Real(0);
#pragma unroll
                        for (int a = 0; a < NFI; ++a)
#pragma unroll
                            for (int dd = 0; dd < NFL; ++dd) s += acc[((a * NFJ + b) * NFK + cc) * NFL + dd] * dil[a * NFL + dd];
                        warp_agg_add(vd ? V + (size_t)(aj + b) * nao + ak + cc : nullptr, fac * s, ab_buf, lane);
                    }
#pragma unroll
                for (int b = 0; b < NFJ; ++b)
#pragma unroll
                    for (int dd = 0; dd < NFL; ++dd) {   // K[j b, l d] += E D[i a, k c]
                        Real s = Real(0);
#pragma unroll
                        for (int a = 0; a < NFI; ++a)
#pragma unroll
                            for (int cc = 0; cc < NFK; ++cc) s += acc[((a * NFJ + b) * NFK + cc) * NFL + dd] * dik[a * NFK + cc];
                        warp_agg_add(vd ? V + (size_t)(aj + b) * nao + al + dd : nullptr, fac * s, ab_buf, lane);
                    }
            }
        }
    }
}

}  // namespace jk
