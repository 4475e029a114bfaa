// Rys J/K kernel for the angular classes with a g shell (l = 4), whose ERI
// blocks (up to 50,625 Cartesian integrals for (gg|gg)) fit neither in
// registers nor in shared memory.  The angular momenta are runtime values;
// one template instance per root count.  A block of 256 threads works on one
// shell quartet at a time and walks its ERI block in chunks of
// GEN_EPT * 256 elements: per chunk it runs the primitive loop (roots and
// weights by one thread, the 2D integrals of every (root, axis) by one
// thread each into shared memory, the chunk's integrals by every thread),
// then adds the chunk's contributions to J and K with one atomic per
// element and output.  Correct for every class up to (gg|gg); the
// templated kernels of jk_classes.cu serve all classes up to f.
#include "jk_device.cuh"
#include "jk_registry.h"
#include "rys_roots.cuh"

namespace jk {

namespace {

constexpr int GEN_EPT = 16;      // integrals per thread and chunk
constexpr int GEN_LMAX = 4;
constexpr int GEN_NSC = 20;      // per-quartet scalars (as the cooperative kernel)

__device__ __forceinline__ int gen_ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponents of component c of a shell of angular momentum l (the
// order x^l, x^(l-1) y, x^(l-1) z, ...)
__device__ __forceinline__ void gen_cart(int l, int c, int &x, int &y, int &z) {
    int t = 0;
    while ((t + 1) * (t + 2) / 2 <= c) ++t;
    x = l - t;
    y = t - (c - t * (t + 1) / 2);
    z = l - x - y;
}

struct GenQuartet {
    int valid, ish, jsh, ksh, lsh, pb_off, npk, pk_off, nsteps, pair;
    double fac;
};

}  // namespace

// Shared memory of a class: the 2D integrals [NR][3][GS] plus roots,
// weights and scalars.
int generic_smem_bytes(int li, int lj, int lk, int ll) {
    const int nr = (li + lj + lk + ll) / 2 + 1;
    const int gs = (li + 1) * (lj + 1) * (lk + 1) * (ll + 1);
    return (nr * 3 * gs + 2 * nr + GEN_NSC) * (int)sizeof(double);
}

template <int NR, int MODE>
__global__ void __launch_bounds__(JK_THREADS)
rys_generic_kernel(EngineDev d, ClassDev c, int ntiles)
{
    const int li = c.li, lj = c.lj, lk = c.lk, ll = c.ll;
    const int nfi = gen_ncart(li), nfj = gen_ncart(lj), nfk = gen_ncart(lk), nfl = gen_ncart(ll);
    const int nf = nfi * nfj * nfk * nfl;
    const int ij = li + lj, kl = lk + ll;
    const int gskl = (lk + 1) * (ll + 1);
    const int gs = (li + 1) * (lj + 1) * gskl;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *g = reinterpret_cast<double *>(smem_raw);   // [NR][3][gs]
    double *rw = g + NR * 3 * gs;                        // u[NR], w[NR]
    double *sc = rw + 2 * NR;                            // scalars
    __shared__ GenQuartet cur;
    __shared__ int2 bq[JK_THREADS + 1];
    __shared__ int wcnt[JK_THREADS / 32];
    __shared__ int s_unit[4];
    __shared__ unsigned int s_max;
    const int tid = threadIdx.x;
    const int nunits = MODE == 0 ? __ldg(c.q_off + c.nx) : 0;
    int kcur = 0, kend = 0, bcur = 0, chunk = blockIdx.x, nq = 0, head = 0;
    bool exhausted = false;
    for (;;) {
        // ---- next quartet: from the block's queue, refilled by screening
        // work units (J/K) or one diagonal pair per tile (Schwarz)
        if (head >= nq) {
            nq = head = 0;
            if (MODE == 0) {
                while (nq == 0 && !exhausted) {
                    if (kcur >= kend) {
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
                        if (w >= nunits) exhausted = true;
                        continue;
                    }
                    const int kk = kcur + tid;
                    const bool ok = kk < kend && pair_passes(d, c, bcur, kk);
                    const unsigned m = __ballot_sync(0xffffffffu, ok);
                    if ((tid & 31) == 0) wcnt[tid >> 5] = __popc(m);
                    __syncthreads();
                    int off = 0, tot = 0;
                    for (int w = 0; w < JK_THREADS / 32; ++w) {
                        if (w < (tid >> 5)) off += wcnt[w];
                        tot += wcnt[w];
                    }
                    if (ok) bq[off + __popc(m & ((1u << (tid & 31)) - 1u))] = make_int2(bcur, kk);
                    nq = tot;
                    kcur += JK_THREADS;
                    __syncthreads();
                }
            } else if (chunk < ntiles) {
                if (tid == 0) bq[0] = make_int2(chunk, chunk);
                nq = 1;
                chunk += gridDim.x;
            }
            if (nq == 0) break;
        }
        if (tid == 0) {
            const int bra = bq[head].x, ket = bq[head].y;
            const int2 pij = c.bra.ij[bra], pkl = c.ket.ij[ket];
            cur.valid = 1;
            cur.ish = pij.x; cur.jsh = pij.y; cur.ksh = pkl.x; cur.lsh = pkl.y;
            cur.pb_off = c.bra.prim_off[bra];
            cur.pk_off = c.ket.prim_off[ket];
            cur.npk = c.ket.prim_cnt[ket];
            cur.nsteps = c.bra.prim_cnt[bra] * cur.npk;
            cur.pair = bra;
            cur.fac = d.op_scale * (pij.x == pij.y ? .5 : 1.) * (pkl.x == pkl.y ? .5 : 1.) *
                      (c.same && bra == ket ? .5 : 1.);
            const ShellDev &A = d.shells[pij.x], &B = d.shells[pij.y];
            const ShellDev &C = d.shells[pkl.x], &D = d.shells[pkl.y];
            sc[14] = A.x - B.x; sc[15] = A.y - B.y; sc[16] = A.z - B.z;
            sc[17] = C.x - D.x; sc[18] = C.y - D.y; sc[19] = C.z - D.z;
            s_max = 0u;
            if (d.counters != nullptr && MODE == 0) {
                atomicAdd(d.counters + 2 * c.class_id, 1ull);
                atomicAdd(d.counters + 2 * c.class_id + 1, (unsigned long long)cur.nsteps);
            }
        }
        ++head;
        __syncthreads();
        const GenQuartet q = cur;
        for (int e0 = 0; e0 < nf; e0 += GEN_EPT * JK_THREADS) {
            double acc[GEN_EPT];
            int idx[GEN_EPT];
#pragma unroll
            for (int k = 0; k < GEN_EPT; ++k) {
                acc[k] = 0.;
                const int e = e0 + tid + k * JK_THREADS;
                idx[k] = -1;
                if (e < nf) {
                    const int dd = e % nfl, t1 = e / nfl;
                    const int cc = t1 % nfk, t2 = t1 / nfk;
                    const int bb = t2 % nfj, aa = t2 / nfj;
                    int ax, ay, az, bx, by, bz, cx, cy, cz, dx, dy, dz;
                    gen_cart(li, aa, ax, ay, az);
                    gen_cart(lj, bb, bx, by, bz);
                    gen_cart(lk, cc, cx, cy, cz);
                    gen_cart(ll, dd, dx, dy, dz);
                    const int ix = ((ax * (lj + 1) + bx) * (lk + 1) + cx) * (ll + 1) + dx;
                    const int iy = ((ay * (lj + 1) + by) * (lk + 1) + cy) * (ll + 1) + dy;
                    const int iz = ((az * (lj + 1) + bz) * (lk + 1) + cz) * (ll + 1) + dz;
                    idx[k] = ix | (iy << 10) | (iz << 20);
                }
            }
            for (int step = 0; step < q.nsteps; ++step) {
                // ---- roots, weights and scalars of this primitive quartet
                if (tid == 0) {
                    const int pb = q.pb_off + step / q.npk, pk = q.pk_off + step % q.npk;
                    const d4 a1 = d.pp_a[pb], a2 = d.pp_a[pk];
                    const d4 b1 = d.pp_b[pb], b2 = d.pp_b[pk];
                    const double ip1 = d.pp_ip[pb], ip2 = d.pp_ip[pk];
                    const double p = a1.x, qq = a2.x;
                    const double rs = rsqrt(p + qq);
                    const double ipq = rs * rs;
                    const double PQx = a1.y - a2.y, PQy = a1.z - a2.z, PQz = a1.w - a2.w;
                    const double T = p * qq * ipq * (PQx * PQx + PQy * PQy + PQz * PQz);
                    const double pref = b1.w * b2.w * rs;
                    double u[NR], w[NR];
                    rys_roots_rs<NR>(T, p * qq * ipq, d.omega2, d.rys_coef, u, w);
                    for (int r = 0; r < NR; ++r) { rw[r] = u[r]; rw[NR + r] = w[r] * pref; }
                    sc[0] = 0.5 * ip1; sc[1] = 0.5 * ip2;
                    sc[2] = qq * ipq; sc[3] = p * ipq; sc[4] = 0.5 * ipq;
                    sc[5] = b1.x; sc[6] = b1.y; sc[7] = b1.z;
                    sc[8] = b2.x; sc[9] = b2.y; sc[10] = b2.z;
                    sc[11] = PQx; sc[12] = PQy; sc[13] = PQz;
                }
                __syncthreads();
                // ---- 2D integrals, one thread per (root, axis)
                if (tid < NR * 3) {
                    const int r = tid / 3, ax = tid % 3;
                    const double u = rw[r];
                    const double i00 = ax == 2 ? rw[NR + r] : 1.;
                    double *gq = g + (r * 3 + ax) * gs;
                    const double b00 = u * sc[4];
                    const double b10 = sc[0] * (1. - u * sc[2]);
                    const double b01 = sc[1] * (1. - u * sc[3]);
                    const double pq = sc[11 + ax];
                    const double c00 = sc[5 + ax] - sc[2] * u * pq;
                    const double cp00 = sc[8 + ax] + sc[3] * u * pq;
                    const double ab = sc[14 + ax], cd = sc[17 + ax];
                    double prev[2 * GEN_LMAX + 1], cv[2 * GEN_LMAX + 1];
                    cv[0] = i00;
                    if (ij > 0) cv[1] = c00 * i00;
                    for (int n = 1; n < ij; ++n) cv[n + 1] = c00 * cv[n] + n * b10 * cv[n - 1];
                    for (int mcol = 0; mcol <= kl; ++mcol) {
                        if (mcol > 0) {
                            double nxt[2 * GEN_LMAX + 1];
                            for (int n = 0; n <= ij; ++n) {
                                double v = cp00 * cv[n];
                                if (mcol > 1) v += (mcol - 1) * b01 * prev[n];
                                if (n > 0) v += n * b00 * cv[n - 1];
                                nxt[n] = v;
                            }
                            for (int n = 0; n <= ij; ++n) { prev[n] = cv[n]; cv[n] = nxt[n]; }
                        }
                        // bra horizontal transfer of this column: h[j][i]
                        double h[GEN_LMAX + 1][2 * GEN_LMAX + 1];
                        for (int n = 0; n <= ij; ++n) h[0][n] = cv[n];
                        for (int j = 1; j <= lj; ++j)
                            for (int i = 0; i <= ij - j; ++i) h[j][i] = h[j - 1][i + 1] + ab * h[j - 1][i];
                        for (int i = 0; i <= li; ++i)
                            for (int j = 0; j <= lj; ++j) gq[(i * (lj + 1) + j) * gskl + mcol] = h[j][i];
                    }
                    // ket horizontal transfer of every (i, j) in place (its
                    // column sits in the first kl + 1 <= gskl entries)
                    for (int t = 0; t < (li + 1) * (lj + 1); ++t) {
                        double tt[GEN_LMAX + 1][2 * GEN_LMAX + 1];
                        for (int k = 0; k <= kl; ++k) tt[0][k] = gq[t * gskl + k];
                        for (int l = 1; l <= ll; ++l)
                            for (int k = 0; k <= kl - l; ++k) tt[l][k] = tt[l - 1][k + 1] + cd * tt[l - 1][k];
                        for (int k = 0; k <= lk; ++k)
                            for (int l = 0; l <= ll; ++l) gq[t * gskl + k * (ll + 1) + l] = tt[l][k];
                    }
                }
                __syncthreads();
                // ---- this thread's integrals of the chunk
#pragma unroll
                for (int k = 0; k < GEN_EPT; ++k) {
                    if (idx[k] < 0) continue;
                    const int ix = idx[k] & 1023, iy = (idx[k] >> 10) & 1023, iz = idx[k] >> 20;
                    double s = 0.;
                    for (int r = 0; r < NR; ++r) {
                        const double *gr = g + r * 3 * gs;
                        s += gr[ix] * gr[gs + iy] * gr[2 * gs + iz];
                    }
                    acc[k] += s;
                }
                __syncthreads();
            }
            if (MODE == 1) {
                // Schwarz factor: max over the diagonal elements (ab|ab)
                float mx = 0.f;
#pragma unroll
                for (int k = 0; k < GEN_EPT; ++k) {
                    const int e = e0 + tid + k * JK_THREADS;
                    if (idx[k] < 0) continue;
                    if (e / (nfk * nfl) == e % (nfk * nfl)) mx = fmaxf(mx, fabsf((float)acc[k]));
                }
                atomicMax(&s_max, __float_as_uint(mx));
                continue;
            }
            // ---- digestion of the chunk: every integral into its six J/K
            // elements (per density)
            const ShellDev &A = d.shells[q.ish];
            const int mol = A.mol;
            const int nao = __ldg(d.mol_nao + mol);
            const size_t nn = (size_t)d.ntot;
            const size_t mbase = (size_t)__ldg(d.mol_base + mol);
            const int ndm_m = d.mol_ndm ? __ldg(d.mol_ndm + mol) : d.n_dm;
            const int ai = A.ao, aj = d.shells[q.jsh].ao, ak = d.shells[q.ksh].ao, al = d.shells[q.lsh].ao;
#pragma unroll
            for (int k = 0; k < GEN_EPT; ++k) {
                if (idx[k] < 0) continue;
                const int e = e0 + tid + k * JK_THREADS;
                const int dd = e % nfl, t1 = e / nfl;
                const int cc = t1 % nfk, t2 = t1 / nfk;
                const int bb = t2 % nfj, aa = t2 / nfj;
                const size_t ri = ai + aa, rj = aj + bb, rk = ak + cc, rl = al + dd;
                const double v = q.fac * acc[k];
                if (d.with_j) {
                    for (int idm = 0; idm < d.n_dm && idm < ndm_m; ++idm) {
                        const double *D = d.dmj + idm * nn + mbase;
                        double *V = d.vj + idm * nn + mbase;
                        jk_add(d, false, V + ri * nao + rj, v * D[rk * nao + rl]);
                        jk_add(d, false, V + rk * nao + rl, v * D[ri * nao + rj]);
                    }
                }
                if (d.with_k) {
                    for (int idm = 0; idm < d.n_dmk; ++idm) {
                        if (idm % d.n_dm >= ndm_m) continue;
                        const double *D = d.dmk + idm * nn + mbase;
                        double *V = d.vk + idm * nn + mbase;
                        jk_add(d, true, V + ri * nao + rk, v * D[rj * nao + rl]);
                        jk_add(d, true, V + ri * nao + rl, v * D[rj * nao + rk]);
                        jk_add(d, true, V + rj * nao + rk, v * D[ri * nao + rl]);
                        jk_add(d, true, V + rj * nao + rl, v * D[ri * nao + rk]);
                    }
                }
            }
        }
        if (MODE == 1) {
            __syncthreads();
            if (tid == 0) d.qout[q.pair] = sqrtf(__uint_as_float(s_max));
        }
        __syncthreads();
    }
}

template <int NR>
static void reg_nr(ClassEntry &e) {
    e.k64 = e.k32 = (const void *)rys_generic_kernel<NR, 0>;
    if (e.li == e.lk && e.lj == e.ll) e.kdiag = (const void *)rys_generic_kernel<NR, 1>;
}

// Classes whose bra pair class holds a g shell (pair classes 10..14): the
// generic kernel, FP64 for both precisions (mixed builds evaluate these
// quartets in FP64 too).
void register_generic(ClassEntry *tab) {
    for (int a = pair_class(4, 0); a < NPAIRCLASS; ++a)
        for (int b = 0; b <= a; ++b) {
            ClassEntry &e = tab[quartet_class(a, b)];
            e.li = pc_li(a); e.lj = pc_lj(a); e.lk = pc_li(b); e.ll = pc_lj(b);
            const int nr = (e.li + e.lj + e.lk + e.ll) / 2 + 1;
            const int smem = generic_smem_bytes(e.li, e.lj, e.lk, e.ll);
            e.lean64 = e.lean32 = 0;
            e.generic = 1;
            e.qb64 = e.qb32 = 1;
            e.smem64 = e.smem32 = smem;
            e.threads64 = e.threads32 = JK_THREADS;
            e.k64_alt = e.k32_alt = nullptr;
            e.qbdiag = 1;
            e.smemdiag = smem;
            e.kdiag = nullptr;
            switch (nr) {
                case 3: reg_nr<3>(e); break;
                case 4: reg_nr<4>(e); break;
                case 5: reg_nr<5>(e); break;
                case 6: reg_nr<6>(e); break;
                case 7: reg_nr<7>(e); break;
                case 8: reg_nr<8>(e); break;
                case 9: reg_nr<9>(e); break;
                default: break;
            }
        }
}

}  // namespace jk
