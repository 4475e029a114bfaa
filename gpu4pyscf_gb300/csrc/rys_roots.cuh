// Rys roots and weights on the device from the tables of gen_rys_tables.py.
//
// T < 40 + 6n: Horner evaluation of the interval polynomial (degree 13 in
// x = T - centre, intervals of width 2), for the roots u_r = t_r^2 and the
// weights w_r (sum_r w_r = F_0(T)).
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

// FP32 roots: table in float; the asymptote in FP64 (or in FP32 when
// asym32 is set: u = h^2/T, w = W/sqrt(T) have no cancellation, so FP32
// keeps its relative 1e-7 there)
template <int NR>
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
    const float *c = coef + rys_off(NR) + k * (RYS_DEG + 1) * 2 * NR;
    float a[2 * NR];
#pragma unroll
    for (int f = 0; f < 2 * NR; ++f) a[f] = __ldg(c + RYS_DEG * 2 * NR + f);
#pragma unroll
    for (int i = RYS_DEG - 1; i >= 0; --i)
#pragma unroll
        for (int f = 0; f < 2 * NR; ++f) a[f] = fmaf(a[f], x, __ldg(c + i * 2 * NR + f));
#pragma unroll
    for (int r = 0; r < NR; ++r) { u[r] = a[r]; w[r] = a[NR + r]; }
}

}  // namespace jk
