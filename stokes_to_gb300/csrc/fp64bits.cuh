// FP32 <-> FP64 conversions by integer arithmetic on the bit patterns.
//
// GB300 runs FP64 arithmetic, and conversions to and from FP64, on a narrow pipe (about two
// operations per SM and clock against 128 FP32 operations), so a conversion per vector
// element costs more than the element's memory traffic. The conversions below use the
// integer pipe for the values the solver meets (zero and normal magnitudes) and give the
// same results as the FP64 pipe; the rest (float subnormals, very small or very large
// doubles, infinities, NaN) take the FP64 pipe.
#pragma once
#include <cuda_runtime.h>

namespace stg {

// (double)f
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));  // +-0
    if (e == 0u || e == 0xffu) return (double)f;
    const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) | ((unsigned long long)(e + 896u) << 52) |
                                 ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)b);
}

// hi = (float)d and lo = (float)(d - (double)hi), both rounded to nearest even. With d =
// (-1)^s 1.m 2^e, hi keeps the top 24 of the 53 significand bits, rounded with the low 29
// (ties to even, a carry moving to exponent e + 1); the remainder d - hi is r 2^(e-52)
// exactly, r a signed integer of at most 29 bits, so lo = fl32(r) 2^(e-52), an integer to
// float conversion and an exact power-of-two scaling. Taken for -74 <= e <= 126, where hi
// and lo are normal floats; zero gives zeros.
__device__ __forceinline__ void split_bits(double d, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    if ((b << 1) == 0ull) {
        hi = __uint_as_float((unsigned)(b >> 32));
        lo = 0.f;
        return;
    }
    const int e = (int)((b >> 52) & 0x7ffu) - 1023;
    if (e < -74 || e > 126) {
        hi = (float)d;
        lo = (float)(d - (double)hi);
        return;
    }
    const unsigned long long m53 = (b & 0xfffffffffffffull) | (1ull << 52);
    unsigned top = (unsigned)(m53 >> 29);
    const int rem = (int)(m53 & 0x1fffffffull);
    int r = rem;
    if (rem > (1 << 28) || (rem == (1 << 28) && (top & 1u))) {
        top += 1u;
        r = rem - (1 << 29);
    }
    int eh = e;
    if (top == (1u << 24)) {
        top = 1u << 23;
        eh = e + 1;
    }
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    hi = __uint_as_float(sign | ((unsigned)(eh + 127) << 23) | (top & 0x7fffffu));
    if (r == 0) {
        lo = 0.f;
    } else {
        const float scale = __uint_as_float((unsigned)(e - 52 + 127) << 23);  // 2^(e-52), normal for e >= -74
        const float l = __int2float_rn(r) * scale;
        lo = sign ? -l : l;
    }
}

}  // namespace stg
