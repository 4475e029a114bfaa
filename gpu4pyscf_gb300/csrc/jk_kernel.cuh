// Per-class Rys J/K kernel template (see jk_device.cuh for the scheme).
#pragma once
#include "jk_device.cuh"
#include "rys_roots.cuh"

namespace jk {

enum { MODE_JK = 0, MODE_DIAG = 1 };

__device__ __forceinline__ void cart_xyz(int l, int c, int &x, int &y, int &z) {
    int idx = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            if (idx == c) { x = lx; y = ly; z = l - lx - ly; return; }
            ++idx;
        }
    x = y = z = 0;
}

struct SlotInfo {
    int valid, ish, jsh, ksh, lsh;
    int pb_off, npb, pk_off, npk, nsteps, step;
    float fac;
    int pair;  // bra pair index (Schwarz mode)
};

template <typename Real>
__device__ __forceinline__ const Real *dm_ptr(const EngineDev &d, bool jpart, int idm);
template <>
__device__ __forceinline__ const double *dm_ptr<double>(const EngineDev &d, bool jpart, int idm) {
    size_t nn = (size_t)d.ntot;
    return jpart ? d.dmj + idm * nn : d.dmk + idm * nn;
}
template <>
__device__ __forceinline__ const float *dm_ptr<float>(const EngineDev &d, bool jpart, int idm) {
    size_t nn = (size_t)d.ntot;
    return jpart ? d.dmj_f + idm * nn : d.dmk_f + idm * nn;
}

// Two blocks per SM (at most 128 registers a thread): while one block's few
// root-evaluating threads run stage S1, the other block keeps the FP64
// pipes busy with its S2/S3 work.
// Exclusive rank of `flag` among the block's threads below tid, and the
// number of threads with the flag set (all threads call it; two barriers).
__device__ __forceinline__ int block_rank(bool flag, int tid, int *wcnt, int &total) {
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if ((tid & 31) == 0) wcnt[tid >> 5] = __popc(m);
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < JK_THREADS / 32; ++w) {
        if (w < (tid >> 5)) off += wcnt[w];
        tot += wcnt[w];
    }
    __syncthreads();
    total = tot;
    return off + __popc(m & ((1u << (tid & 31)) - 1u));
}

template <int LI, int LJ, int LK, int LL, typename Real, int MODE>
__global__ void __launch_bounds__(JK_THREADS, 2)
rys_class_kernel(EngineDev d, ClassDev c, int ntiles_static)
{
    using S = ClassShape<LI, LJ, LK, LL, Real>;
    constexpr int NR = S::NR, G = S::G, QB = S::QB, NPT = S::NPT, NF = S::NF, GS = S::GS;
    constexpr int NFI = S::NFI, NFJ = S::NFJ, NFK = S::NFK, NFL = S::NFL;
    constexpr int IJ = S::IJ, KL = S::KL, GSKL = S::GSKL, NSC = S::NSC;
    constexpr int GREG = (S::g_bytes(QB) > S::e_bytes(QB) ? S::g_bytes(QB) : S::e_bytes(QB)) / (int)sizeof(Real);

    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *gbuf = reinterpret_cast<Real *>(smem_raw);          // [QB][NR][3][GS]  or E[QB][NF]
    Real *rw = gbuf + GREG;                                     // [QB][NR][NRW]
    Real *sc = rw + QB * NR * S::NRW;                           // [QB][NSC]
    __shared__ SlotInfo slots[QB];
    __shared__ unsigned int smax[MODE == MODE_DIAG ? QB : 1];

    const int tid = threadIdx.x;
    const int s_own = tid / G;      // quartet slot owned in S3
    const int gl = tid % G;

    // element -> packed (ix, iy, iz) indices into the 2D integral arrays
    int eidx[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        int e = gl + k * G;
        if (e < NF) {
            int dd = e % NFL, t = e / NFL;
            int cc = t % NFK; t /= NFK;
            int bb = t % NFJ;
            int aa = t / NFJ;
            int ax, ay, az, bx, by, bz, cx, cy, cz, dx, dy, dz;
            cart_xyz(LI, aa, ax, ay, az);
            cart_xyz(LJ, bb, bx, by, bz);
            cart_xyz(LK, cc, cx, cy, cz);
            cart_xyz(LL, dd, dx, dy, dz);
            int ix = ((ax * (LJ + 1) + bx) * (LK + 1) + cx) * (LL + 1) + dx;
            int iy = ((ay * (LJ + 1) + by) * (LK + 1) + cy) * (LL + 1) + dy;
            int iz = ((az * (LJ + 1) + bz) * (LK + 1) + cz) * (LL + 1) + dz;
            eidx[k] = ix | (iy << 10) | (iz << 20);
        } else {
            eidx[k] = -1;
        }
    }

    const int ntiles = ntiles_static;

    // Work acquisition.  J/K mode: the block takes work units (JK_KCHUNK kets
    // of one (ket bucket, bra) range) from the launch's counter, screens them
    // and keeps the quartets that pass in a shared queue.  Schwarz mode:
    // tiles of QB diagonal pairs.  Slots are refilled one by one: every step
    // runs one primitive quartet of every busy slot, and a slot whose quartet
    // is complete is digested right away and takes the next queued quartet,
    // so no slot idles while its neighbours run longer primitive loops.
    __shared__ int2 bq[QB + JK_THREADS];
    __shared__ int wcnt[JK_THREADS / 32];
    __shared__ int s_unit[4];
    __shared__ int fin_list[QB];
    int chunk = blockIdx.x;
    const int nunits = MODE == MODE_JK ? __ldg(c.q_off + c.nx) : 0;
    if (MODE == MODE_JK && blockIdx.x > 0 && (long long)blockIdx.x * JK_MIN_UNITS >= nunits) return;
    if (MODE == MODE_JK && sizeof(Real) == 8 && blockIdx.x >= gridDim.x / 2 && d.qprev != nullptr) {
        const unsigned long long prev = d.qprev[c.class_id];
        if (prev > 0 && (unsigned long long)blockIdx.x * QB * JK_Q_PER_LANE >= prev) return;
    }
    int kcur = 0, kend = 0, bcur = 0;
    bool exhausted = false;
    int nq = 0;
    if (tid < QB) {
        slots[tid].valid = 0;
        slots[tid].step = slots[tid].nsteps = 0;
    }
    Real acc[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) acc[k] = Real(0);
    const SlotInfo &mine = slots[s_own];

    for (;;) {
        // ---- refill the empty slots from the queue
        const int nempty = __syncthreads_count(tid < QB && !slots[tid].valid);
        if (nempty > 0) {
            if (MODE == MODE_JK) {
                while (nq < nempty && !exhausted) {
                    if (kcur >= kend) {
                        // warp 0 takes the next unit and finds its range
                        if (tid < 32) {
                            int w = 0;
                            if (tid == 0) w = atomicAdd(c.work, 1);
                            w = __shfl_sync(0xffffffffu, w, 0);
                            int xw = 0, k0 = 0, k1 = 0;
                            if (w < nunits) unit_at_warp(c, w, tid, xw, k0, k1);
                            if (tid == 0) {
                                s_unit[0] = w;
                                s_unit[1] = xw % c.bra.n;
                                s_unit[2] = k0;
                                s_unit[3] = k1;
                            }
                        }
                        __syncthreads();
                        const int w = s_unit[0];
                        bcur = s_unit[1];
                        kcur = s_unit[2];
                        kend = s_unit[3];
                        __syncthreads();
                        if (w >= nunits) { exhausted = true; break; }
                        continue;
                    }
                    const int kk = kcur + tid;
                    const bool okc = kk < kend && pair_passes(d, c, bcur, kk);
                    int tot;
                    const int r = block_rank(okc, tid, wcnt, tot);
                    if (okc) bq[nq + r] = make_int2(bcur, kk);
                    nq += tot;
                    kcur += JK_THREADS;
                    __syncthreads();
                }
            } else if (nq < nempty && !exhausted) {
                if (chunk >= ntiles) {
                    exhausted = true;
                } else {
                    const int p = chunk * QB + tid;
                    if (tid < QB && p < c.bra.n) bq[nq + tid] = make_int2(p, p);
                    nq += min(QB, c.bra.n - chunk * QB);
                    chunk += gridDim.x;
                    __syncthreads();
                }
            }
            const int take = min(nq, nempty);
            if (MODE == MODE_JK && d.qnow != nullptr && tid == 0 && take > 0)
                atomicAdd(d.qnow + c.class_id, (unsigned long long)take);
            const bool emp = tid < QB && !slots[tid].valid;
            int tot;
            const int r = block_rank(emp, tid, wcnt, tot);
            if (emp && r < take) {
                const int bra = bq[r].x, ket = bq[r].y;
                const int2 pij = c.bra.ij[bra];
                const int2 pkl = c.ket.ij[ket];
                SlotInfo si;
                si.valid = 1;
                si.ish = pij.x; si.jsh = pij.y; si.ksh = pkl.x; si.lsh = pkl.y;
                si.pb_off = c.bra.prim_off[bra];
                si.npb = c.bra.prim_cnt[bra];
                si.pk_off = c.ket.prim_off[ket];
                si.npk = c.ket.prim_cnt[ket];
                si.nsteps = si.npb * si.npk;
                si.step = 0;
                float fac = 1.f;
                if (pij.x == pij.y) fac *= .5f;
                if (pkl.x == pkl.y) fac *= .5f;
                if (c.same && bra == ket) fac *= .5f;
                si.fac = fac;
                si.pair = bra;
                const ShellDev &A = d.shells[pij.x], &B = d.shells[pij.y];
                const ShellDev &C = d.shells[pkl.x], &D = d.shells[pkl.y];
                Real *m = sc + tid * NSC;
                m[14] = (Real)(A.x - B.x); m[15] = (Real)(A.y - B.y); m[16] = (Real)(A.z - B.z);
                m[17] = (Real)(C.x - D.x); m[18] = (Real)(C.y - D.y); m[19] = (Real)(C.z - D.z);
                slots[tid] = si;
                if (MODE == MODE_DIAG) smax[tid] = 0u;
                if (d.counters != nullptr && MODE == MODE_JK) {
                    atomicAdd(d.counters + 2 * c.class_id, 1ull);
                    atomicAdd(d.counters + 2 * c.class_id + 1, (unsigned long long)si.nsteps);
                }
            }
            // drop the taken entries (at most QB + JK_THREADS - 1 remain)
            const int rem = nq - take;
            const int2 t0 = tid < rem ? bq[take + tid] : make_int2(0, 0);
            const int2 t1 = tid + JK_THREADS < rem ? bq[take + JK_THREADS + tid] : make_int2(0, 0);
            __syncthreads();
            if (tid < rem) bq[tid] = t0;
            if (tid + JK_THREADS < rem) bq[JK_THREADS + tid] = t1;
            nq = rem;
        }
        // no busy slot after the refill: the work is exhausted
        if (__syncthreads_count(tid < QB && slots[tid].valid) == 0) break;

        // ---- S1: roots, weights, scalars.  FP64: one thread per (slot,
        // root), so the root evaluation of a step spreads over NR times as
        // many warps (and SM sub-partitions) instead of leaving most of them
        // waiting at the barrier; FP32: one thread per slot ----
        if constexpr (sizeof(Real) == 8) {
            for (int t = tid; t < QB * NR; t += JK_THREADS) {
                const int s = t / NR, r = t % NR;
                const SlotInfo &si = slots[s];
                if (!si.valid) continue;
                const int pb = si.pb_off + si.step / si.npk;
                const int pk = si.pk_off + si.step % si.npk;
                const d4 a1 = d.pp_a[pb], a2 = d.pp_a[pk];
                const d4 b1 = d.pp_b[pb], b2 = d.pp_b[pk];
                const double ip1 = d.pp_ip[pb], ip2 = d.pp_ip[pk];
                const double p = a1.x, q = a2.x;
                const double rs = rsqrt(p + q);
                const double ipq = rs * rs;
                const double PQx = a1.y - a2.y, PQy = a1.z - a2.z, PQz = a1.w - a2.w;
                const double T = p * q * ipq * (PQx * PQx + PQy * PQy + PQz * PQz);
                double ur, wr;
                rys_root_one_rs<NR>(T, p * q * ipq, d.omega2, d.rys_coef, r, ur, wr);
                // the coefficients the three axes share (computed here once
                // instead of in each of the axis tasks of S2)
                const double qpq = q * ipq, ppq = p * ipq;
                Real *x = rw + (s * NR + r) * S::NRW;
                x[0] = ur;
                x[1] = wr * (b1.w * b2.w * rs * d.op_scale);
                x[2] = ur * (0.5 * ipq);
                x[3] = 0.5 * ip1 - ur * qpq * (0.5 * ip1);
                x[4] = 0.5 * ip2 - ur * ppq * (0.5 * ip2);
                x[5] = ur * qpq;
                x[6] = ur * ppq;
                if (r == 0) {
                    Real *m = sc + s * NSC;
                    m[5] = b1.x; m[6] = b1.y; m[7] = b1.z;
                    m[8] = b2.x; m[9] = b2.y; m[10] = b2.z;
                    m[11] = PQx; m[12] = PQy; m[13] = PQz;
                }
            }
        } else for (int s = tid; s < QB; s += JK_THREADS) {
            const SlotInfo &si = slots[s];
            if (!si.valid) continue;
            int pb = si.pb_off + si.step / si.npk;
            int pk = si.pk_off + si.step % si.npk;
            Real *myrw = rw + s * NR * S::NRW;
            Real *m = sc + s * NSC;
            {
                float4 a1 = d.pp_af[pb], a2 = d.pp_af[pk];
                float4 b1 = d.pp_bf[pb], b2 = d.pp_bf[pk];
                float ip1 = d.pp_ipf[pb], ip2 = d.pp_ipf[pk];
                float p = a1.x, q = a2.x;
                float rs = rsqrtf(p + q);
                float ipq = rs * rs;
                float PQx = a1.y - a2.y, PQy = a1.z - a2.z, PQz = a1.w - a2.w;
                float T = p * q * ipq * (PQx * PQx + PQy * PQy + PQz * PQz);
                float pref = b1.w * b2.w * rs * d.op_scale_f;
                float u[NR], w[NR];
                rys_roots_rs_f<NR>(T, p * q * ipq, d.omega2_f, d.rys_coef_f, u, w, d.fp32_asym);
                const float h2p = 0.5f * ip1, h2q = 0.5f * ip2, qpq = q * ipq, ppq = p * ipq, h2pq = 0.5f * ipq;
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    Real *x = myrw + r * S::NRW;
                    x[0] = (Real)u[r];
                    x[1] = (Real)(w[r] * pref);
                    x[2] = (Real)(u[r] * h2pq);
                    x[3] = (Real)(h2p - u[r] * qpq * h2p);
                    x[4] = (Real)(h2q - u[r] * ppq * h2q);
                    x[5] = (Real)(u[r] * qpq);
                    x[6] = (Real)(u[r] * ppq);
                }
                m[5] = (Real)b1.x; m[6] = (Real)b1.y; m[7] = (Real)b1.z;
                m[8] = (Real)b2.x; m[9] = (Real)b2.y; m[10] = (Real)b2.z;
                m[11] = (Real)PQx; m[12] = (Real)PQy; m[13] = (Real)PQz;
            }
        }
        __syncthreads();
        // ---- S2: 2D integrals per (slot, root, axis) ----
        for (int task = tid; task < QB * NR * 3; task += JK_THREADS) {
            int s = task / (NR * 3);
            int rem = task % (NR * 3);
            int r = rem / 3, ax = rem % 3;
            if (!slots[s].valid) continue;
            const Real *m = sc + s * NSC;
            const Real *x = rw + (s * NR + r) * S::NRW;
            Real i00 = (ax == 2) ? x[1] : Real(1);
            Real *g = gbuf + ((s * NR + r) * 3 + ax) * GS;
            if (IJ == 0 && KL == 0) { g[0] = i00; continue; }
            Real b00 = x[2], b10 = x[3], b01 = x[4];
            Real pq = m[11 + ax];
            Real c00 = m[5 + ax] - x[5] * pq;
            Real cp00 = m[8 + ax] + x[6] * pq;
            Real ab = m[14 + ax], cd = m[17 + ax];
            Real prev[IJ + 1], cur[IJ + 1];
            // column 0 of the vertical recurrence
            cur[0] = i00;
            if (IJ > 0) cur[1] = c00 * i00;
#pragma unroll
            for (int n = 1; n < IJ; ++n) cur[n + 1] = c00 * cur[n] + Real(n) * b10 * cur[n - 1];
#pragma unroll
            for (int mcol = 0; mcol <= KL; ++mcol) {
                if (mcol > 0) {
                    Real nxt[IJ + 1];
#pragma unroll
                    for (int n = 0; n <= IJ; ++n) {
                        Real v = cp00 * cur[n];
                        if (mcol > 1) v += Real(mcol - 1) * b01 * prev[n];
                        if (n > 0) v += Real(n) * b00 * cur[n - 1];
                        nxt[n] = v;
                    }
#pragma unroll
                    for (int n = 0; n <= IJ; ++n) { prev[n] = cur[n]; cur[n] = nxt[n]; }
                }
                // bra horizontal transfer on this column
                Real h[LJ + 1][IJ + 1];
#pragma unroll
                for (int n = 0; n <= IJ; ++n) h[0][n] = cur[n];
#pragma unroll
                for (int j = 1; j <= LJ; ++j)
#pragma unroll
                    for (int i = 0; i <= IJ - j; ++i) h[j][i] = h[j - 1][i + 1] + ab * h[j - 1][i];
#pragma unroll
                for (int i = 0; i <= LI; ++i)
#pragma unroll
                    for (int j = 0; j <= LJ; ++j) g[(i * (LJ + 1) + j) * (KL + 1) + mcol] = h[j][i];
            }
            if (KL > 0) {
                // ket horizontal transfer in place, highest (i,j) first
#pragma unroll
                for (int ij = (LI + 1) * (LJ + 1) - 1; ij >= 0; --ij) {
                    Real t[LL + 1][KL + 1];
#pragma unroll
                    for (int k = 0; k <= KL; ++k) t[0][k] = g[ij * (KL + 1) + k];
#pragma unroll
                    for (int l = 1; l <= LL; ++l)
#pragma unroll
                        for (int k = 0; k <= KL - l; ++k) t[l][k] = t[l - 1][k + 1] + cd * t[l - 1][k];
#pragma unroll
                    for (int k = 0; k <= LK; ++k)
#pragma unroll
                        for (int l = 0; l <= LL; ++l) g[ij * GSKL + k * (LL + 1) + l] = t[l][k];
                }
            }
        }
        __syncthreads();
        // ---- S3: accumulate the Cartesian ERIs owned by this thread ----
        if (mine.valid) {
            const Real *gq = gbuf + s_own * NR * 3 * GS;
#pragma unroll
            for (int k = 0; k < NPT; ++k) {
                int pk = eidx[k];
                if (pk < 0) continue;
                int ix = pk & 1023, iy = (pk >> 10) & 1023, iz = pk >> 20;
                Real sum = Real(0);
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const Real *gr = gq + r * 3 * GS;
                    sum += gr[ix] * gr[GS + iy] * gr[2 * GS + iz];
                }
                acc[k] += sum;
            }
        }
        // ---- slots whose quartet is complete (S3 reads no step counter) ----
        bool fin = false;
        if (tid < QB && slots[tid].valid) {
            const int st = slots[tid].step + 1;
            slots[tid].step = st;
            fin = st == slots[tid].nsteps;
        }
        int nfin;
        const int fr = block_rank(fin, tid, wcnt, nfin);
        if (nfin == 0) continue;
        if (fin) fin_list[fr] = tid;
        const bool my_fin = mine.valid && mine.step == mine.nsteps;

        if (MODE == MODE_DIAG) {
            // Schwarz factor: max over the diagonal elements (ab|ab)
            if (my_fin) {
                float mx = 0.f;
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    int e = gl + k * G;
                    if (e >= NF) continue;
                    int ab = e / (NFK * NFL), cd = e % (NFK * NFL);
                    if (ab == cd) mx = fmaxf(mx, fabsf((float)acc[k]));
                }
                atomicMax(&smax[s_own], __float_as_uint(mx));
            }
            __syncthreads();
            if (fin) d.qout[slots[tid].pair] = sqrtf(__uint_as_float(smax[tid]));
        } else {
            // ---- digestion of the complete slots: stage their ERIs (the 2D
            // integrals of this step are consumed), contract with the densities
            Real *E = gbuf;
            if (my_fin) {
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    int e = gl + k * G;
                    if (e < NF) E[s_own * NF + e] = acc[k];
                }
            }
            __syncthreads();
            constexpr int NJ = NFI * NFJ + NFK * NFL;
            constexpr int NK = NFI * NFK + NFI * NFL + NFJ * NFK + NFJ * NFL;
            const int nj = d.with_j ? d.n_dm * NJ : 0;
            const int nk = d.with_k ? d.n_dmk * NK : 0;
            const int per = nj + nk;
            // consecutive threads take the same output element of different
            // slots, so a warp runs one contraction type (one loop length)
            for (int task = tid; task < nfin * per; task += JK_THREADS) {
                const int s = fin_list[task % nfin];
                int t = task / nfin;
                const SlotInfo &si = slots[s];
                const int mol = d.shells[si.ish].mol;
                const int nao = __ldg(d.mol_nao + mol);
                const size_t mbase = (size_t)__ldg(d.mol_base + mol);
                const int ndm_m = d.mol_ndm ? __ldg(d.mol_ndm + mol) : d.n_dm;
                const Real *Es = E + s * NF;
                const int ai = d.shells[si.ish].ao, aj = d.shells[si.jsh].ao;
                const int ak = d.shells[si.ksh].ao, al = d.shells[si.lsh].ao;
                Real sum = Real(0);
                double *out;
                const bool isk = t >= nj;
                if (t < nj) {
                    int idm = t / NJ, o = t % NJ;
                    if (idm >= ndm_m) continue;  // density the molecule does not carry
                    const Real *D = dm_ptr<Real>(d, true, idm) + mbase;
                    if (o < NFI * NFJ) {
                        int a = o / NFJ, b = o % NFJ;
                        const Real *Er = Es + (a * NFJ + b) * NFK * NFL;
#pragma unroll 4
                        for (int cc = 0; cc < NFK; ++cc)
                            for (int dd = 0; dd < NFL; ++dd)
                                sum += Er[cc * NFL + dd] * D[(size_t)(ak + cc) * nao + al + dd];
                        out = d.vj + (size_t)idm * d.ntot + mbase + (size_t)(ai + a) * nao + aj + b;
                    } else {
                        o -= NFI * NFJ;
                        int cc = o / NFL, dd = o % NFL;
                        for (int a = 0; a < NFI; ++a)
                            for (int b = 0; b < NFJ; ++b)
                                sum += Es[(a * NFJ + b) * NFK * NFL + cc * NFL + dd] * D[(size_t)(ai + a) * nao + aj + b];
                        out = d.vj + (size_t)idm * d.ntot + mbase + (size_t)(ak + cc) * nao + al + dd;
                    }
                } else {
                    t -= nj;
                    int idm = t / NK, o = t % NK;
                    if (idm % d.n_dm >= ndm_m) continue;
                    const Real *D = dm_ptr<Real>(d, false, idm) + mbase;
                    double *V = d.vk + (size_t)idm * d.ntot + mbase;
                    if (o < NFI * NFK) {            // K[i a, k c] += E[abcd] D[j b, l d]
                        int a = o / NFK, cc = o % NFK;
                        for (int b = 0; b < NFJ; ++b)
                            for (int dd = 0; dd < NFL; ++dd)
                                sum += Es[((a * NFJ + b) * NFK + cc) * NFL + dd] * D[(size_t)(aj + b) * nao + al + dd];
                        out = V + (size_t)(ai + a) * nao + ak + cc;
                    } else if ((o -= NFI * NFK) < NFI * NFL) {   // K[i a, l d] += E D[j b, k c]
                        int a = o / NFL, dd = o % NFL;
                        for (int b = 0; b < NFJ; ++b)
                            for (int cc = 0; cc < NFK; ++cc)
                                sum += Es[((a * NFJ + b) * NFK + cc) * NFL + dd] * D[(size_t)(aj + b) * nao + ak + cc];
                        out = V + (size_t)(ai + a) * nao + al + dd;
                    } else if ((o -= NFI * NFL) < NFJ * NFK) {   // K[j b, k c] += E D[i a, l d]
                        int b = o / NFK, cc = o % NFK;
                        for (int a = 0; a < NFI; ++a)
                            for (int dd = 0; dd < NFL; ++dd)
                                sum += Es[((a * NFJ + b) * NFK + cc) * NFL + dd] * D[(size_t)(ai + a) * nao + al + dd];
                        out = V + (size_t)(aj + b) * nao + ak + cc;
                    } else {                                     // K[j b, l d] += E D[i a, k c]
                        o -= NFJ * NFK;
                        int b = o / NFL, dd = o % NFL;
                        for (int a = 0; a < NFI; ++a)
                            for (int cc = 0; cc < NFK; ++cc)
                                sum += Es[((a * NFJ + b) * NFK + cc) * NFL + dd] * D[(size_t)(ai + a) * nao + ak + cc];
                        out = V + (size_t)(aj + b) * nao + al + dd;
                    }
                }
                if constexpr (sizeof(Real) == 4) jk_add(d, isk, out, widen_f32(si.fac * sum));
                else jk_add(d, isk, out, (double)si.fac * (double)sum);
            }
        }
        if (my_fin) {
#pragma unroll
            for (int k = 0; k < NPT; ++k) acc[k] = Real(0);
        }
        __syncthreads();
        if (fin) slots[tid].valid = 0;
    }
}

}  // namespace jk
