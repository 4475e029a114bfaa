// Rys roots and weights on the device from the tables of gen_rys_tables.py.
//
// T < 40 + 6n: Horner evaluation of the interval polynomial (degree 13 in
// x = T - centre, intervals of width 2; degree 8 for the FP32 table), for the
// roots u_r = t_r^2 and the weights w_r (sum_r w_r = F_0(T)).
// T >= 40 + 6n: u_r = h_r^2 / T, w_r = W_r / sqrt(T) from 2n-point
// Gauss-Hermite quadrature, always evaluated in FP64.
#pragma once
#include "rys_tables.inc"

namespace jk {

__constant__ double c_rys_asym_x2[RYS_ASYM_SIZE] = {RYS_ASYM_X2_LIST};
__constant__ double c_rys_asym_w[RYS_ASYM_SIZE] = {RYS_ASYM_W_LIST};

__host__ __device__ constexpr int rys_nint(int n) { return (40 + 6 * n) / RYS_WIDTH; }
__host__ __device__ constexpr int rys_off(int n) {
    return n <= 1 ? 0 : rys_off(n - 1) + rys_nint(n - 1) * (RYS_DEG + 1) * 2 * (n - 1);
}
// the FP32 table: same intervals, degree RYS_DEG_F
__host__ __device__ constexpr int rys_off_f(int n) {
    return n <= 1 ? 0 : rys_off_f(n - 1) + rys_nint(n - 1) * (RYS_DEG_F + 1) * 2 * (n - 1);
}

template <int NR>
__device__ __forceinline__ void rys_asym(double T, double *u, double *w) {
    double rs = rsqrt(T);
    double it = rs * rs;
    constexpr int o = NR * (NR - 1) / 2;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        u[r] = c_rys_asym_x2[o + r] * it;
        w[r] = c_rys_asym_w[o + r] * rs;
    }
}

// FP64 roots: table in double
template <int NR>
__device__ __forceinline__ void rys_roots(double T, const double *__restrict__ coef, double *u, double *w) {
    static_assert(NR <= RYS_NMAX, "too many roots");
    if (!(T < 2.0 * rys_nint(NR))) {  // NaN also takes this branch (no table access)
        rys_asym<NR>(T, u, w);
        return;
    }
    int k = (int)(T * 0.5);
    double x = T - (2 * k + 1);
    const double *c = coef + rys_off(NR) + k * (RYS_DEG + 1) * 2 * NR;
    double a[2 * NR];
#pragma unroll
    for (int f = 0; f < 2 * NR; ++f) a[f] = __ldg(c + RYS_DEG * 2 * NR + f);
#pragma unroll
    for (int i = RYS_DEG - 1; i >= 0; --i)
#pragma unroll
        for (int f = 0; f < 2 * NR; ++f) a[f] = fma(a[f], x, __ldg(c + i * 2 * NR + f));
#pragma unroll
    for (int r = 0; r < NR; ++r) { u[r] = a[r]; w[r] = a[NR + r]; }
}

// FP32 table staged in shared memory by a kernel: the block of NR roots,
// one interval every rys_f_stride(NR) floats.  The stride is odd, so lanes
// evaluating different intervals read different banks (every class has
// fewer than 32 intervals per root count).
__host__ __device__ constexpr int rys_f_stride(int n) { return ((RYS_DEG_F + 1) * 2 * n) | 1; }
__host__ __device__ constexpr int rys_f_smem(int n) { return rys_nint(n) * rys_f_stride(n); }

template <int NR>
__device__ __forceinline__ void rys_stage_f(const float *__restrict__ coef, float *s, int tid, int nthreads) {
    constexpr int per = (RYS_DEG_F + 1) * 2 * NR;
    const float *src = coef + rys_off_f(NR);
    for (int e = tid; e < rys_nint(NR) * per; e += nthreads) s[(e / per) * rys_f_stride(NR) + e % per] = __ldg(src + e);
}

// FP32 roots: table in float; the asymptote in FP64 (or in FP32 when
// asym32 is set: u = h^2/T, w = W/sqrt(T) have no cancellation, so FP32
// keeps its relative 1e-7 there).  SMEM: coef is the block staged by
// rys_stage_f, else the whole global table.
template <int NR, bool SMEM = false>
__device__ __forceinline__ void rys_roots_f(float T, const float *__restrict__ coef, float *u, float *w,
                                            int asym32 = 0) {
    if (!(T < 2.f * rys_nint(NR))) {
        if (asym32) {
            const float rs = rsqrtf(T);
            const float it = rs * rs;
            constexpr int o = NR * (NR - 1) / 2;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                u[r] = (float)c_rys_asym_x2[o + r] * it;
                w[r] = (float)c_rys_asym_w[o + r] * rs;
            }
            return;
        }
        double ud[NR], wd[NR];
        rys_asym<NR>((double)T, ud, wd);
#pragma unroll
        for (int r = 0; r < NR; ++r) { u[r] = (float)ud[r]; w[r] = (float)wd[r]; }
        return;
    }
    int k = (int)(T * 0.5f);
    float x = T - (float)(2 * k + 1);
    float a[2 * NR];
    if constexpr (SMEM) {
        const float *c = coef + k * rys_f_stride(NR);
#pragma unroll
        for (int f = 0; f < 2 * NR; ++f) a[f] = c[RYS_DEG_F * 2 * NR + f];
#pragma unroll
        for (int i = RYS_DEG_F - 1; i >= 0; --i)
#pragma unroll
            for (int f = 0; f < 2 * NR; ++f) a[f] = fmaf(a[f], x, c[i * 2 * NR + f]);
    } else {
        const float *c = coef + rys_off_f(NR) + k * (RYS_DEG_F + 1) * 2 * NR;
#pragma unroll
        for (int f = 0; f < 2 * NR; ++f) a[f] = __ldg(c + RYS_DEG_F * 2 * NR + f);
#pragma unroll
        for (int i = RYS_DEG_F - 1; i >= 0; --i)
#pragma unroll
            for (int f = 0; f < 2 * NR; ++f) a[f] = fmaf(a[f], x, __ldg(c + i * 2 * NR + f));
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) { u[r] = a[r]; w[r] = a[NR + r]; }
}

// Range-separated roots.  The long-range operator erf(omega r)/r stops the
// Gaussian transform of 1/r at omega, which cuts the Rys integral over t at
// t^2 = theta = omega^2 / (omega^2 + rho) (rho = pq/(p+q)).  Substituting
// t^2 = theta s^2 gives sqrt(theta) times the standard quadrature at theta*T,
// with roots s_r^2 mapped back to u_r = theta s_r^2.  omega2 = omega^2 <= 0
// selects the plain Coulomb operator (theta = 1, the same roots exactly).
template <int NR>
__device__ __forceinline__ void rys_roots_rs(double T, double rho, double omega2,
                                             const double *__restrict__ coef, double *u, double *w) {
    const double theta = omega2 > 0. ? omega2 / (omega2 + rho) : 1.;
    rys_roots<NR>(T * theta, coef, u, w);
    if (omega2 > 0.) {
        const double st = sqrt(theta);
#pragma unroll
        for (int r = 0; r < NR; ++r) { u[r] *= theta; w[r] *= st; }
    }
}

template <int NR, bool SMEM = false>
__device__ __forceinline__ void rys_roots_rs_f(float T, float rho, float omega2, const float *__restrict__ coef,
                                               float *u, float *w, int asym32) {
    const float theta = omega2 > 0.f ? omega2 / (omega2 + rho) : 1.f;
    rys_roots_f<NR, SMEM>(T * theta, coef, u, w, asym32);
    if (omega2 > 0.f) {
        const float st = sqrtf(theta);
#pragma unroll
        for (int r = 0; r < NR; ++r) { u[r] *= theta; w[r] *= st; }
    }
}

}  // namespace jk
