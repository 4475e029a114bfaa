// Exact widening of an FP32 value to FP64 on the integer pipe.
//
// GB300 runs FP64 instructions, conversions included, at 1/64 of the FP32
// rate, so in the FP32 quartet kernels the float -> double conversion of
// every contribution before its FP64 atomic costs more issue time than the
// integrals themselves.  The IEEE-754 fields map directly: same sign, the
// exponent re-biased from 127 to 1023, the 23-bit fraction shifted into the
// top of the 52-bit one.  Zeros and FP32 subnormals (below 1.2e-38, far
// beneath anything a J/K contribution can carry) give a signed zero;
// infinities and NaNs keep their class.  Usable in host code as well, where
// the tests compare it with the compiler's conversion.
#pragma once
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define F2D_HD inline
#else
#define F2D_HD __host__ __device__ __forceinline__
#endif

F2D_HD double f32_to_f64_exact(float f) {
    uint32_t u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(f);
#else
    memcpy(&u, &f, 4);
#endif
    const uint32_t e = (u >> 23) & 0xffu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    const uint64_t ee = e == 255u ? 0x7ffull : (uint64_t)(e + 896u);  // 1023 - 127 = 896
    uint64_t bits = sign | (ee << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
    bits = e == 0u ? sign : bits;
    double d;
#ifdef __CUDA_ARCH__
    d = __longlong_as_double((long long)bits);
#else
    memcpy(&d, &bits, 8);
#endif
    return d;
}
