// Nuclear gradient of the J/K energy (counterpart of the reference's
// RYS_per_atom_jk_ip1, gpu4pyscf/lib/gvhf-rys/rys_contract_jk_ip1.cu:1747,
// driven by gpu4pyscf/grad/rhf.py:60-171).  For every screened shell
// quartet (ij|kl) of the optimizer's pair lists the kernel evaluates the
// derivative integrals with respect to the centres A, B, C of its first
// three shells, contracts them on the fly with the quartet's density
// weights and adds the nine sums to per-atom accumulators; the fourth centre
// follows from translational invariance, dD = -(dA + dB + dC).  No J or K
// matrix is formed.
//
// Derivative of a primitive Cartesian Gaussian x_A^a exp(-alpha x_A^2) with
// respect to its centre: 2 alpha (a+1) - a (a-1) in the index notation, so
// the 2D integrals of a primitive quartet are built with i, j and k raised
// by one ("raised box": i <= li+1, j <= lj+1, k <= lk+1, l <= ll, with at
// most one index raised at a time, which the bra and ket horizontal
// transfers give from the vertical recurrence up to li+lj+1 and lk+ll+1).
// One more root than the energy's is needed: NR = (L + 1)/2 + 1.
//
// Work layout.  A block of 256 threads takes a work unit (one bra pair and
// up to 64 kets of one primitive-count bucket), screens its kets and works
// on the passing quartets qb at a time ("slots", qb per class so that the
// slots' shared-memory arrays fit).  Quartets of a unit share the bra pair
// and the primitive counts, so the slots walk their primitive quartets in
// lockstep: per step one thread per (slot, root) evaluates a root and
// weight (S1), one thread per (slot, root, axis) the raised box (S2), every
// thread a share of the derivative arrays (S2b, see rys_ip1_kernel), and
// the 256/qb threads of a slot their share of the slot's Cartesian
// elements (S3), each holding the density weights of its elements in
// registers.
#include "jk_device.cuh"
#include "jk_registry.h"
#include "rys_roots.cuh"

namespace jk {

namespace {

// elements per thread and chunk, and blocks per SM the register budget is
// sized for (two: 128 registers, a few hundred bytes spilled, 19% faster
// on the dense 30-atom gradient than one block of 255 registers)
#ifndef GRAD_EPT
#define GRAD_EPT 8
#endif
#ifndef GRAD_MIN_BLOCKS
#define GRAD_MIN_BLOCKS 2
#endif
constexpr int GR_EPT = GRAD_EPT;  // elements per thread and chunk
constexpr int GR_NSC = 24;       // per-slot scalars of a primitive step
constexpr int GR_QBMAX = 64;     // slots per block (JK_KCHUNK kets per unit)
constexpr int GR_SMEM_BUDGET = 100 * 1024;   // dynamic shared memory per block: two blocks per SM
constexpr int GR_NRMAX = (4 * GRAD_LMAX + 1) / 2 + 1;

__host__ __device__ __forceinline__ int gr_ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponents of component c of a shell of angular momentum l (the
// order x^l, x^(l-1) y, x^(l-1) z, ...)
__device__ __forceinline__ void gr_cart(int l, int c, int &x, int &y, int &z) {
    int t = 0;
    while ((t + 1) * (t + 2) / 2 <= c) ++t;
    x = l - t;
    y = t - (c - t * (t + 1) / 2);
    z = l - x - y;
}

__host__ __device__ __forceinline__ int gr_box(int li, int lj, int lk, int ll) {
    return (li + 2) * (lj + 2) * (lk + 2) * (ll + 1);
}
__host__ __device__ __forceinline__ int gr_nroots(int li, int lj, int lk, int ll) {
    return (li + lj + lk + ll + 1) / 2 + 1;
}
__host__ __device__ __forceinline__ int gr_obox(int li, int lj, int lk, int ll) {
    return (li + 1) * (lj + 1) * (lk + 1) * (ll + 1);
}
// doubles per slot: the raised boxes, with der the derivative arrays
// (integral and its A, B, C derivatives over the class's own index box),
// roots and weights, scalars
__host__ __device__ __forceinline__ int gr_slot_doubles(int li, int lj, int lk, int ll, bool der) {
    const int nr = gr_nroots(li, lj, lk, ll);
    return nr * 3 * gr_box(li, lj, lk, ll) + (der ? nr * 12 * gr_obox(li, lj, lk, ll) : 0) + 2 * nr + GR_NSC;
}

// Screening of a quartet for the gradient: q_ij q_kl times the largest
// density product its weight holds (D_ij D_kl for J, D_jk D_li and
// D_jl D_ki for K) against the cutoff.
__device__ __forceinline__ bool grad_passes(const EngineDev &d, const GradDev &g, const ClassDev &c, int bra,
                                            int ket) {
    const int2 pij = c.bra.ij[bra], pkl = c.ket.ij[ket];
    const float *dc = d.dm_cond;
    const int nb = d.nbas;
    const int i = pij.x, j = pij.y, k = pkl.x, l = pkl.y;
    const float vj = __ldg(dc + i * nb + j) + __ldg(dc + k * nb + l) + g.log_j;
    const float vk = fmaxf(__ldg(dc + j * nb + k) + __ldg(dc + l * nb + i),
                           __ldg(dc + j * nb + l) + __ldg(dc + k * nb + i)) + g.log_k;
    const float v = __ldg(c.bra.logq + bra) + __ldg(c.ket.logq + ket) + fmaxf(vj, vk);
    return v >= d.log_cut;
}

}  // namespace

// DER: after the raised boxes one more stage (S2b, every thread) forms the
// derivative arrays G, dA, dB, dC of each (slot, root, axis) over the
// class's own index box, so that the element stage needs 15 FP64
// instructions per element and root instead of 33; classes whose arrays
// do not fit the shared-memory budget (pairs of f shells) take the
// derivatives from the raised box inside the element stage.
template <int NR, bool DER>
__global__ void __launch_bounds__(JK_THREADS, GRAD_MIN_BLOCKS)
rys_ip1_kernel(EngineDev d, ClassDev c, GradDev gd)
{
    const int li = c.li, lj = c.lj, lk = c.lk, ll = c.ll;
    const int nfi = gr_ncart(li), nfj = gr_ncart(lj), nfk = gr_ncart(lk), nfl = gr_ncart(ll);
    const int nf = nfi * nfj * nfk * nfl;
    const int ijm = li + lj + 1, klm = lk + ll + 1;
    // raised box of one (root, axis): index a sA + b sB + c sC + d
    const int sC = ll + 1, sB = (lk + 2) * sC, sA = (lj + 2) * sB, box = (li + 2) * sA;
    // the class's own index box: index ((a (lj+1) + b) (lk+1) + c) (ll+1) + d
    const int oC = ll + 1, oB = (lk + 1) * oC, oA = (lj + 1) * oB, obox = (li + 1) * oA;
    const int qoff = NR * 3 * box;                              // derivative arrays
    const int rwoff = qoff + (DER ? NR * 12 * obox : 0);        // roots, weights, scalars
    const int slot_d = rwoff + 2 * NR + GR_NSC;
    const int qb = gd.qb, tps = JK_THREADS / qb;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);   // [qb][slot_d]
    __shared__ int bq[JK_KCHUNK];
    __shared__ int wcnt[JK_THREADS / 32];
    __shared__ int s_unit[4];
    __shared__ int s_k[GR_QBMAX], s_l[GR_QBMAX], s_pk[GR_QBMAX];
    __shared__ double s_fac[GR_QBMAX];
    __shared__ double s_acc[GR_QBMAX * 9];
    const int tid = threadIdx.x, lane = tid & 31;
    const int slot = tid / tps, sub = tid - slot * tps;
    const int nunits = __ldg(c.q_off + c.nx);
    const size_t nn = (size_t)gd.nao * gd.nao;
    for (;;) {
        // ---- next work unit and its passing kets
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
        const int w = s_unit[0], bra = s_unit[1], k0 = s_unit[2], k1 = s_unit[3];
        if (w >= nunits) break;
        const int kk = k0 + tid;
        const bool ok = tid < JK_KCHUNK && kk < k1 && grad_passes(d, gd, c, bra, kk);
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (lane == 0) wcnt[tid >> 5] = __popc(m);
        __syncthreads();
        int off = 0, nq = 0;
        for (int x = 0; x < JK_THREADS / 32; ++x) {
            if (x < (tid >> 5)) off += wcnt[x];
            nq += wcnt[x];
        }
        if (ok) bq[off + __popc(m & ((1u << lane) - 1u))] = kk;
        __syncthreads();
        const int2 pij = c.bra.ij[bra];
        const int pb_off = c.bra.prim_off[bra], npb = c.bra.prim_cnt[bra];
        const ShellDev &A = d.shells[pij.x], &B = d.shells[pij.y];
        for (int b0 = 0; b0 < nq; b0 += qb) {
            const int nb = min(qb, nq - b0);
            if (tid < nb) {
                const int ket = bq[b0 + tid];
                const int2 pkl = c.ket.ij[ket];
                s_k[tid] = pkl.x;
                s_l[tid] = pkl.y;
                s_pk[tid] = c.ket.prim_off[ket];
                s_fac[tid] = d.op_scale * (pij.x == pij.y ? .5 : 1.) * (pkl.x == pkl.y ? .5 : 1.) *
                             (c.same && bra == ket ? .5 : 1.);
            }
            for (int t = tid; t < qb * 9; t += JK_THREADS) s_acc[t] = 0.;
            __syncthreads();
            const int npk = c.ket.prim_cnt[bq[b0]];   // one primitive count per unit
            const int nsteps = npb * npk;
            if (tid == 0 && d.counters != nullptr) {
                atomicAdd(d.counters + 2 * c.class_id, (unsigned long long)nb);
                atomicAdd(d.counters + 2 * c.class_id + 1, (unsigned long long)nb * nsteps);
            }
            const bool active = slot < nb;
            double acc[9];
#pragma unroll
            for (int x = 0; x < 9; ++x) acc[x] = 0.;
            for (int e0 = 0; e0 < nf; e0 += GR_EPT * tps) {
                // ---- this thread's elements of the chunk: raised-box
                // offsets, Cartesian exponents and density weights
                double W[GR_EPT];
                int ix3[GR_EPT], ex9[GR_EPT];
#pragma unroll
                for (int mm = 0; mm < GR_EPT; ++mm) {
                    W[mm] = 0.;
                    ix3[mm] = 0;
                    ex9[mm] = 0;
                    const int e = e0 + sub + mm * tps;
                    if (active && e < nf) {
                        const int dd = e % nfl, t1 = e / nfl;
                        const int cc = t1 % nfk, t2 = t1 / nfk;
                        const int bb = t2 % nfj, aa = t2 / nfj;
                        int ax, ay, az, bx, by, bz, cx, cy, cz, dx, dy, dz;
                        gr_cart(li, aa, ax, ay, az);
                        gr_cart(lj, bb, bx, by, bz);
                        gr_cart(lk, cc, cx, cy, cz);
                        gr_cart(ll, dd, dx, dy, dz);
                        if (DER) {
                            const int ox = ax * oA + bx * oB + cx * oC + dx;
                            const int oy = ay * oA + by * oB + cy * oC + dy;
                            const int oz = az * oA + bz * oB + cz * oC + dz;
                            ix3[mm] = ox | (oy << 10) | (oz << 20);
                        } else {
                            const int ix = ax * sA + bx * sB + cx * sC + dx;
                            const int iy = ay * sA + by * sB + cy * sC + dy;
                            const int iz = az * sA + bz * sB + cz * sC + dz;
                            ix3[mm] = ix | (iy << 10) | (iz << 20);
                            ex9[mm] = ax | (ay << 3) | (az << 6) | (bx << 9) | (by << 12) | (bz << 15) |
                                      (cx << 18) | (cy << 21) | (cz << 24);
                        }
                        const size_t i = A.ao + aa, j = B.ao + bb;
                        const size_t k = d.shells[s_k[slot]].ao + cc, l = d.shells[s_l[slot]].ao + dd;
                        double js_ij = 0., js_kl = 0., kx = 0.;
                        for (int s = 0; s < gd.n_dm; ++s) {
                            const double *D = gd.dm + s * nn;
                            if (gd.jfac != 0.) {
                                js_ij += __ldg(D + j * gd.nao + i);
                                js_kl += __ldg(D + l * gd.nao + k);
                            }
                            if (gd.kfac != 0.)
                                kx += __ldg(D + j * gd.nao + k) * __ldg(D + l * gd.nao + i) +
                                      __ldg(D + j * gd.nao + l) * __ldg(D + k * gd.nao + i);
                        }
                        W[mm] = s_fac[slot] * (gd.jfac * js_ij * js_kl + gd.kfac * kx);
                    }
                }
                for (int step = 0; step < nsteps; ++step) {
                    // ---- S1: roots and weights, one thread per (slot, root);
                    // the root-0 thread of a slot also stores its scalars
                    for (int t = tid; t < nb * NR; t += JK_THREADS) {
                        const int s = t / NR, r = t - s * NR;
                        double *sl = sm + s * slot_d;
                        double *rw = sl + rwoff;
                        double *sc = rw + 2 * NR;
                        const int pb = pb_off + step / npk, pk = s_pk[s] + step % npk;
                        const d4 a1 = d.pp_a[pb], a2 = d.pp_a[pk];
                        const double p = a1.x, qq = a2.x;
                        const double rs = rsqrt(p + qq);
                        const double ipq = rs * rs;
                        const double PQx = a1.y - a2.y, PQy = a1.z - a2.z, PQz = a1.w - a2.w;
                        const double T = p * qq * ipq * (PQx * PQx + PQy * PQy + PQz * PQz);
                        const d4 b1 = d.pp_b[pb], b2 = d.pp_b[pk];
                        double u, wt;
                        rys_root_one_rs<NR>(T, p * qq * ipq, d.omega2, d.rys_coef, r, u, wt);
                        rw[r] = u;
                        rw[NR + r] = wt * (b1.w * b2.w * rs);
                        if (r == 0) {
                            const double ip1 = d.pp_ip[pb], ip2 = d.pp_ip[pk];
                            sc[0] = 0.5 * ip1; sc[1] = 0.5 * ip2;
                            sc[2] = qq * ipq; sc[3] = p * ipq; sc[4] = 0.5 * ipq;
                            sc[5] = b1.x; sc[6] = b1.y; sc[7] = b1.z;
                            sc[8] = b2.x; sc[9] = b2.y; sc[10] = b2.z;
                            sc[11] = PQx; sc[12] = PQy; sc[13] = PQz;
                            const ShellDev &C = d.shells[s_k[s]], &Dsh = d.shells[s_l[s]];
                            sc[14] = A.x - B.x; sc[15] = A.y - B.y; sc[16] = A.z - B.z;
                            sc[17] = C.x - Dsh.x; sc[18] = C.y - Dsh.y; sc[19] = C.z - Dsh.z;
                            const double2 ea = gd.pp_e[pb], ec = gd.pp_e[pk];
                            sc[20] = 2. * ea.x; sc[21] = 2. * ea.y; sc[22] = 2. * ec.x;
                        }
                    }
                    __syncthreads();
                    // ---- S2: raised box of every (slot, root, axis)
                    for (int t = tid; t < nb * NR * 3; t += JK_THREADS) {
                        const int s = t / (NR * 3), r = (t / 3) % NR, ax = t % 3;
                        double *sl = sm + s * slot_d;
                        const double *rw = sl + rwoff;
                        const double *sc = rw + 2 * NR;
                        double *gq = sl + (r * 3 + ax) * box;
                        const double u = rw[r];
                        const double i00 = ax == 2 ? rw[NR + r] : 1.;
                        const double b00 = u * sc[4];
                        const double b10 = sc[0] * (1. - u * sc[2]);
                        const double b01 = sc[1] * (1. - u * sc[3]);
                        const double pq = sc[11 + ax];
                        const double c00 = sc[5 + ax] - sc[2] * u * pq;
                        const double cp00 = sc[8 + ax] + sc[3] * u * pq;
                        const double ab = sc[14 + ax], cd = sc[17 + ax];
                        double prev[2 * GRAD_LMAX + 2], cv[2 * GRAD_LMAX + 2];
                        cv[0] = i00;
                        cv[1] = c00 * i00;
                        for (int n = 1; n < ijm; ++n) cv[n + 1] = c00 * cv[n] + n * b10 * cv[n - 1];
                        for (int mc = 0; mc <= klm; ++mc) {
                            if (mc > 0) {
                                double nxt[2 * GRAD_LMAX + 2];
                                for (int n = 0; n <= ijm; ++n) {
                                    double v = cp00 * cv[n];
                                    if (mc > 1) v += (mc - 1) * b01 * prev[n];
                                    if (n > 0) v += n * b00 * cv[n - 1];
                                    nxt[n] = v;
                                }
                                for (int n = 0; n <= ijm; ++n) { prev[n] = cv[n]; cv[n] = nxt[n]; }
                            }
                            // bra transfer of this column: h[j][i] for
                            // j <= lj+1, i <= ijm - j
                            double h[GRAD_LMAX + 2][2 * GRAD_LMAX + 2];
                            for (int n = 0; n <= ijm; ++n) h[0][n] = cv[n];
                            for (int j = 1; j <= lj + 1; ++j)
                                for (int i = 0; i <= ijm - j; ++i) h[j][i] = h[j - 1][i + 1] + ab * h[j - 1][i];
                            for (int i = 0; i <= li + 1; ++i)
                                for (int j = 0; j <= lj + 1 && i + j <= ijm; ++j) gq[i * sA + j * sB + mc] = h[j][i];
                        }
                        // ket transfer of every (i, j) in place: its column
                        // occupies the first klm + 1 <= sB entries
                        for (int i = 0; i <= li + 1; ++i)
                            for (int j = 0; j <= lj + 1 && i + j <= ijm; ++j) {
                                double *col = gq + i * sA + j * sB;
                                double tt[GRAD_LMAX + 1][2 * GRAD_LMAX + 2];
                                for (int k = 0; k <= klm; ++k) tt[0][k] = col[k];
                                for (int l = 1; l <= ll; ++l)
                                    for (int k = 0; k <= klm - l; ++k) tt[l][k] = tt[l - 1][k + 1] + cd * tt[l - 1][k];
                                for (int k = 0; k <= lk + 1; ++k)
                                    for (int l = 0; l <= ll; ++l) col[k * sC + l] = tt[l][k];
                            }
                    }
                    __syncthreads();
                    if (DER) {
                        // ---- S2b: derivative arrays of every (slot, root,
                        // axis): G, 2 a_i G(a+1) - a G(a-1), and the same
                        // for b and c
                        const int per = NR * 3 * obox;
                        for (int t = tid; t < nb * per; t += JK_THREADS) {
                            const int s = t / per, rem = t - s * per;
                            const int ra = rem / obox, o = rem - ra * obox;
                            const int dd = o % oC, t1 = o / oC;
                            const int cc = t1 % (lk + 1), t2 = t1 / (lk + 1);
                            const int bb = t2 % (lj + 1), aa = t2 / (lj + 1);
                            double *sl = sm + s * slot_d;
                            const double *sc = sl + rwoff + 2 * NR;
                            const double *R = sl + ra * box;
                            double *Q = sl + qoff + ra * 4 * obox;
                            const int ri = aa * sA + bb * sB + cc * sC + dd;
                            Q[o] = R[ri];
                            Q[obox + o] = fma(sc[20], R[ri + sA], -aa * R[ri - (aa ? sA : 0)]);
                            Q[2 * obox + o] = fma(sc[21], R[ri + sB], -bb * R[ri - (bb ? sB : 0)]);
                            Q[3 * obox + o] = fma(sc[22], R[ri + sC], -cc * R[ri - (cc ? sC : 0)]);
                        }
                        __syncthreads();
                    }
                    // ---- S3: this thread's elements, nine derivative sums
                    if (active && DER) {
                        const double *Qs = sm + slot * slot_d + qoff;
#pragma unroll
                        for (int mm = 0; mm < GR_EPT; ++mm) {
                            if (W[mm] == 0.) continue;
                            const int ox = ix3[mm] & 1023, oy = (ix3[mm] >> 10) & 1023, oz = ix3[mm] >> 20;
                            const double wgt = W[mm];
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                const double *qx = Qs + r * 12 * obox, *qy = qx + 4 * obox, *qz = qy + 4 * obox;
                                const double X = qx[ox], Y = qy[oy], Z = qz[oz];
                                const double wyz = wgt * Y * Z, wxz = wgt * X * Z, wxy = wgt * X * Y;
                                acc[0] = fma(qx[obox + ox], wyz, acc[0]);
                                acc[1] = fma(qy[obox + oy], wxz, acc[1]);
                                acc[2] = fma(qz[obox + oz], wxy, acc[2]);
                                acc[3] = fma(qx[2 * obox + ox], wyz, acc[3]);
                                acc[4] = fma(qy[2 * obox + oy], wxz, acc[4]);
                                acc[5] = fma(qz[2 * obox + oz], wxy, acc[5]);
                                acc[6] = fma(qx[3 * obox + ox], wyz, acc[6]);
                                acc[7] = fma(qy[3 * obox + oy], wxz, acc[7]);
                                acc[8] = fma(qz[3 * obox + oz], wxy, acc[8]);
                            }
                        }
                    }
                    if (active && !DER) {
                        const double *sl = sm + slot * slot_d;
                        const double *sc = sl + rwoff + 2 * NR;
                        const double ai2 = sc[20], aj2 = sc[21], ak2 = sc[22];
#pragma unroll
                        for (int mm = 0; mm < GR_EPT; ++mm) {
                            if (W[mm] == 0.) continue;
                            const int ix = ix3[mm] & 1023, iy = (ix3[mm] >> 10) & 1023, iz = ix3[mm] >> 20;
                            const int ex = ex9[mm];
                            const int ax = ex & 7, ay = (ex >> 3) & 7, az = (ex >> 6) & 7;
                            const int bx = (ex >> 9) & 7, by = (ex >> 12) & 7, bz = (ex >> 15) & 7;
                            const int cx = (ex >> 18) & 7, cy = (ex >> 21) & 7, cz = (ex >> 24) & 7;
                            // lowered neighbours; a zero exponent multiplies
                            // an in-box entry by 0
                            const int xam = ix - (ax ? sA : 0), xbm = ix - (bx ? sB : 0), xcm = ix - (cx ? sC : 0);
                            const int yam = iy - (ay ? sA : 0), ybm = iy - (by ? sB : 0), ycm = iy - (cy ? sC : 0);
                            const int zam = iz - (az ? sA : 0), zbm = iz - (bz ? sB : 0), zcm = iz - (cz ? sC : 0);
                            const double wgt = W[mm];
                            for (int r = 0; r < NR; ++r) {
                                const double *gx = sl + r * 3 * box, *gy = gx + box, *gz = gy + box;
                                const double X = gx[ix], Y = gy[iy], Z = gz[iz];
                                const double wyz = wgt * Y * Z, wxz = wgt * X * Z, wxy = wgt * X * Y;
                                acc[0] = fma(fma(ai2, gx[ix + sA], -ax * gx[xam]), wyz, acc[0]);
                                acc[1] = fma(fma(ai2, gy[iy + sA], -ay * gy[yam]), wxz, acc[1]);
                                acc[2] = fma(fma(ai2, gz[iz + sA], -az * gz[zam]), wxy, acc[2]);
                                acc[3] = fma(fma(aj2, gx[ix + sB], -bx * gx[xbm]), wyz, acc[3]);
                                acc[4] = fma(fma(aj2, gy[iy + sB], -by * gy[ybm]), wxz, acc[4]);
                                acc[5] = fma(fma(aj2, gz[iz + sB], -bz * gz[zbm]), wxy, acc[5]);
                                acc[6] = fma(fma(ak2, gx[ix + sC], -cx * gx[xcm]), wyz, acc[6]);
                                acc[7] = fma(fma(ak2, gy[iy + sC], -cy * gy[ycm]), wxz, acc[7]);
                                acc[8] = fma(fma(ak2, gz[iz + sC], -cz * gz[zcm]), wxy, acc[8]);
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            // ---- the slot's nine sums, then per atom: A, B, C and
            // D = -(A + B + C)
            const int span = tps < 32 ? tps : 32;
#pragma unroll
            for (int x = 0; x < 9; ++x) {
                double v = acc[x];
                for (int o = span >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (active && (lane & (span - 1)) == 0) atomicAdd(s_acc + slot * 9 + x, v);
            }
            __syncthreads();
            for (int t = tid; t < nb * 12; t += JK_THREADS) {
                const int s = t / 12, comp = t % 12, ctr = comp / 3, x = comp % 3;
                const double *a9 = s_acc + s * 9;
                const double v = ctr < 3 ? a9[ctr * 3 + x] : -(a9[x] + a9[3 + x] + a9[6 + x]);
                const int sh = ctr == 0 ? pij.x : ctr == 1 ? pij.y : ctr == 2 ? s_k[s] : s_l[s];
                atomicAdd(gd.grad + 3 * __ldg(gd.shell_atom + sh) + x, v);
            }
            __syncthreads();
        }
    }
}

namespace {

template <bool DER>
const void *grad_kernel_of(int nr) {
    switch (nr) {
        case 1: return (const void *)rys_ip1_kernel<1, DER>;
        case 2: return (const void *)rys_ip1_kernel<2, DER>;
        case 3: return (const void *)rys_ip1_kernel<3, DER>;
        case 4: return (const void *)rys_ip1_kernel<4, DER>;
        case 5: return (const void *)rys_ip1_kernel<5, DER>;
        case 6: return (const void *)rys_ip1_kernel<6, DER>;
        case 7: return (const void *)rys_ip1_kernel<7, DER>;
        default: return nullptr;
    }
}

}  // namespace

int grad_class(int li, int lj, int lk, int ll, GradClass *out) {
    if (li > GRAD_LMAX || lj > GRAD_LMAX || lk > GRAD_LMAX || ll > GRAD_LMAX) return 1;
    const int nr = gr_nroots(li, lj, lk, ll);
    static_assert(GR_NRMAX <= 7, "gradient kernels are instantiated up to 7 roots");
    const bool der = gr_slot_doubles(li, lj, lk, ll, true) * (int)sizeof(double) <= GR_SMEM_BUDGET;
    const int slot = gr_slot_doubles(li, lj, lk, ll, der) * (int)sizeof(double);
    int qb = GR_QBMAX;
    while (qb > 1 && qb * slot > GR_SMEM_BUDGET) qb >>= 1;
    out->kernel = der ? grad_kernel_of<true>(nr) : grad_kernel_of<false>(nr);
    out->qb = qb;
    out->smem = qb * slot;
    return out->kernel ? 0 : 1;
}

int grad_set_smem_attrs() {
    for (int li = 0; li <= GRAD_LMAX; ++li)
        for (int lj = 0; lj <= GRAD_LMAX; ++lj)
            for (int lk = 0; lk <= GRAD_LMAX; ++lk)
                for (int ll = 0; ll <= GRAD_LMAX; ++ll) {
                    GradClass g;
                    if (grad_class(li, lj, lk, ll, &g)) continue;
                    cudaFuncAttributes fa;
                    cudaError_t e = cudaFuncGetAttributes(&fa, g.kernel);
                    if (e != cudaSuccess) return (int)e;
                    if (fa.maxDynamicSharedSizeBytes >= g.smem) continue;
                    e = cudaFuncSetAttribute(g.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.smem);
                    if (e != cudaSuccess) return (int)e;
                }
    return 0;
}

}  // namespace jk
