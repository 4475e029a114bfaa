// Rys roots and weights on the device from the tables of gen_rys_tables.py.
//
// T < 40 + 6n: Horner evaluation of the interval polynomial, for the roots
// u_r = t_r^2 and the weights w_r (sum_r w_r = F_0(T)): degree 9 in
// x = T - centre on intervals of width 1/2 for the FP64 table, degree 8 on
// intervals of width 2 for the FP32 table.
// T >= 40 + 6n: u_r = h_r^2 / T, w_r = W_r / sqrt(T) from 2n-point
// Gauss-Hermite quadrature, evaluated in FP64 (or FP32 on request for the
// FP32 quartets).
#pragma once
#include "rys_tables.inc"

namespace jk {

__constant__ double c_rys_asym_x2[RYS_ASYM_SIZE] = {RYS_ASYM_X2_LIST};
__constant__ double c_rys_asym_w[RYS_ASYM_SIZE] = {RYS_ASYM_W_LIST};
__constant__ float c_rys_asym_x2_f[RYS_ASYM_SIZE] = {RYS_ASYM_X2_LIST_F};
__constant__ float c_rys_asym_w_f[RYS_ASYM_SIZE] = {RYS_ASYM_W_LIST_F};

static_assert(RYS_INV_WIDTH == 2, "the FP64 interval index below assumes intervals of width 1/2");

__host__ __device__ constexpr int rys_tmax(int n) { return 40 + 6 * n; }
__host__ __device__ constexpr int rys_nint(int n) { return rys_tmax(n) * RYS_INV_WIDTH; }
__host__ __device__ constexpr int rys_off(int n) {
    return n <= 1 ? 0 : rys_off(n - 1) + rys_nint(n - 1) * (RYS_DEG + 1) * 2 * (n - 1);
}
// the FP32 table: its own intervals and degree
__host__ __device__ constexpr int rys_nint_f(int n) { return rys_tmax(n) / RYS_WIDTH_F; }
__host__ __device__ constexpr int rys_off_f(int n) {
    return n <= 1 ? 0 : rys_off_f(n - 1) + rys_nint_f(n - 1) * (RYS_DEG_F + 1) * 2 * (n - 1);
}

// High 32 bits of the double of a small positive integer v (its low word is
// zero): sign 0, biased exponent, the top 20 bits of the fraction.
__host__ __device__ constexpr int dbl_hi_of_int(int v) {
    int e = 0;
    while ((2 << e) <= v) ++e;
    return ((1023 + e) << 20) | ((v - (1 << e)) << (20 - e));
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

// FP64 roots: table in double.  The branch on T, the interval index
// k = floor(2T) and the interval centre (2k+1)/4 come from the bits of T with
// integer operations, leaving one FP64 subtraction before the Horner steps:
// on GB300 FP64 instructions are the scarce resource and the integer pipes
// idle.  T >= 0 (a -0 lands in interval 0); NaN takes the asymptote branch
// (no table access).
template <int NR>
__device__ __forceinline__ void rys_roots(double T, const double *__restrict__ coef, double *u, double *w) {
    static_assert(NR <= RYS_NMAX, "too many roots");
    const int hi = __double2hiint(T);
    if (hi >= dbl_hi_of_int(rys_tmax(NR))) {   // T >= T_asym(n), or NaN
        rys_asym<NR>(T, u, w);
        return;
    }
    // T = m 2^(e-20) with m the 21-bit significand of the high word; the low
    // word cannot change floor(2T) = m >> (19 - e) (zero for T < 1/2)
    const int e = ((hi >> 20) & 0x7ff) - 1023;
    const int m = (hi & 0xfffff) | 0x100000;
    const int sh = 19 - e;
    const int k = sh > 20 ? 0 : (m >> sh);
    // centre (2k+1)/4 as a double built from its bits (an odd integer n
    // below 2^9 times 2^-2: exponent b-2 for its top bit b, fraction bits in
    // the high word)
    const int n = 2 * k + 1;
    const int b = 31 - __clz(n);
    const double centre = __hiloint2double(((1023 + b - 2) << 20) | ((n - (1 << b)) << (20 - b)), 0);
    const double x = T - centre;
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

// One root r (u_r, w_r) of the FP64 quadrature: the same branch, interval
// and Horner steps as rys_roots, for the two columns of root r only (a
// block spreads the roots of a quartet over NR threads).
template <int NR>
__device__ __forceinline__ void rys_root_one(double T, int r, const double *__restrict__ coef, double &u, double &w) {
    const int hi = __double2hiint(T);
    if (hi >= dbl_hi_of_int(rys_tmax(NR))) {
        const double rs = rsqrt(T);
        constexpr int o = NR * (NR - 1) / 2;
        u = c_rys_asym_x2[o + r] * rs * rs;
        w = c_rys_asym_w[o + r] * rs;
        return;
    }
    const int e = ((hi >> 20) & 0x7ff) - 1023;
    const int m = (hi & 0xfffff) | 0x100000;
    const int sh = 19 - e;
    const int k = sh > 20 ? 0 : (m >> sh);
    const int n = 2 * k + 1;
    const int b = 31 - __clz(n);
    const double centre = __hiloint2double(((1023 + b - 2) << 20) | ((n - (1 << b)) << (20 - b)), 0);
    const double x = T - centre;
    const double *c = coef + rys_off(NR) + k * (RYS_DEG + 1) * 2 * NR;
    double a0 = __ldg(c + RYS_DEG * 2 * NR + r), a1 = __ldg(c + RYS_DEG * 2 * NR + NR + r);
#pragma unroll
    for (int i = RYS_DEG - 1; i >= 0; --i) {
        a0 = fma(a0, x, __ldg(c + i * 2 * NR + r));
        a1 = fma(a1, x, __ldg(c + i * 2 * NR + NR + r));
    }
    u = a0;
    w = a1;
}

template <int NR>
__device__ __forceinline__ void rys_root_one_rs(double T, double rho, double omega2, const double *__restrict__ coef,
                                                int r, double &u, double &w) {
    if (__double2hiint(omega2) <= 0) {
        rys_root_one<NR>(T, r, coef, u, w);
        return;
    }
    const double theta = omega2 / (omega2 + rho);
    rys_root_one<NR>(T * theta, r, coef, u, w);
    u *= theta;
    w *= sqrt(theta);
}

// FP32 table staged in shared memory by a kernel: the block of NR roots,
// one interval every rys_f_stride(NR) floats.  The stride is odd, so lanes
// evaluating different intervals read different banks (every class has
// fewer than 32 intervals per root count).
__host__ __device__ constexpr int rys_f_stride(int n) { return ((RYS_DEG_F + 1) * 2 * n) | 1; }
__host__ __device__ constexpr int rys_f_smem(int n) { return rys_nint_f(n) * rys_f_stride(n); }

template <int NR>
__device__ __forceinline__ void rys_stage_f(const float *__restrict__ coef, float *s, int tid, int nthreads) {
    constexpr int per = (RYS_DEG_F + 1) * 2 * NR;
    const float *src = coef + rys_off_f(NR);
    for (int e = tid; e < rys_nint_f(NR) * per; e += nthreads) s[(e / per) * rys_f_stride(NR) + e % per] = __ldg(src + e);
}

// FP32 roots: table in float; the asymptote in FP64 (or in FP32 when
// asym32 is set: u = h^2/T, w = W/sqrt(T) have no cancellation, so FP32
// keeps its relative 1e-7 there).  SMEM: coef is the block staged by
// rys_stage_f, else the whole global table.
template <int NR, bool SMEM = false>
__device__ __forceinline__ void rys_roots_f(float T, const float *__restrict__ coef, float *u, float *w,
                                            int asym32 = 0) {
    if (!(T < (float)rys_tmax(NR))) {
        if (asym32) {
            const float rs = rsqrtf(T);
            const float it = rs * rs;
            constexpr int o = NR * (NR - 1) / 2;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                u[r] = c_rys_asym_x2_f[o + r] * it;
                w[r] = c_rys_asym_w_f[o + r] * rs;
            }
            return;
        }
        double ud[NR], wd[NR];
        rys_asym<NR>((double)T, ud, wd);
#pragma unroll
        for (int r = 0; r < NR; ++r) { u[r] = (float)ud[r]; w[r] = (float)wd[r]; }
        return;
    }
    static_assert(RYS_WIDTH_F == 2, "FP32 intervals of width 2");
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
    // omega2 >= 0; its high word tells 0 from positive without an FP64 compare
    if (__double2hiint(omega2) <= 0) {
        rys_roots<NR>(T, coef, u, w);
        return;
    }
    const double theta = omega2 / (omega2 + rho);
    rys_roots<NR>(T * theta, coef, u, w);
    const double st = sqrt(theta);
#pragma unroll
    for (int r = 0; r < NR; ++r) { u[r] *= theta; w[r] *= st; }
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
