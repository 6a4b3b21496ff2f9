// knc_bits.cuh — FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the FP64 pipe retires about 1/64 of the FP32 rate, and the
// hardware conversions between double and float issue on that pipe too. The
// mixed-precision stage converts every zone's five FP64 conserved values to
// FP32 and every FP32 increment back to FP64, so these conversions are done
// here with 32-bit integer operations, which issue at the full ALU rate.
//
// d2f_rn: round to nearest even, like __double2float_rn, for values in
// float's normal range; smaller magnitudes flush to a signed zero, larger ones
// (and inf / NaN) become a signed infinity. The stage only converts conserved
// volume integrals and increments, which stay well inside that range.
// f2d: exact (every float is a double), with float subnormals flushed to zero.
#pragma once

#include <stdint.h>

namespace knc {

__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u;
    const int e32 = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    const uint32_t m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu;     // the 29 dropped mantissa bits
    uint32_t r = ((uint32_t)e32 << 23) + m23;   // exponent and mantissa; a carry from rounding
    r += (rest > 0x10000000u) || (rest == 0x10000000u && (m23 & 1u));   // propagates into the exponent
    r = e32 <= 0 ? 0u : r;
    r = e32 >= 255 ? 0x7f800000u : r;
    r = r > 0x7f800000u ? 0x7f800000u : r;      // rounding up from the largest float
    return __uint_as_float(sign | r);
}

__device__ __forceinline__ double f2d(float x) {
    const uint32_t f = __float_as_uint(x);
    const uint32_t sign = f & 0x80000000u;
    const uint32_t e = (f >> 23) & 0xffu;
    const uint32_t m = f & 0x7fffffu;
    uint32_t hi, lo;
    if (e == 0u) {                 // zero or subnormal -> signed zero
        hi = sign;
        lo = 0u;
    } else if (e == 0xffu) {       // inf / NaN
        hi = sign | 0x7ff00000u | (m >> 3);
        lo = m << 29;
    } else {
        hi = sign | ((e - 127u + 1023u) << 20) | (m >> 3);
        lo = m << 29;
    }
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// d2f_rn(x * 2^de) and x * 2^de exactly as a double (de small; the mixed
// stage's length scale): the power of two enters the exponent field, so the
// scaled value is formed without an FP64 multiply.
__device__ __forceinline__ float d2f_rn_exp(double x, int de) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t ex = (hi >> 20) & 0x7ffu;
    const int e32 = (int)ex - 1023 + 127 + (ex ? de : 0);
    const uint32_t m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu;
    uint32_t r = ((uint32_t)e32 << 23) + m23;
    r += (rest > 0x10000000u) || (rest == 0x10000000u && (m23 & 1u));
    r = e32 <= 0 ? 0u : r;
    r = (e32 >= 255 || ex == 0x7ffu) ? 0x7f800000u : r;
    r = r > 0x7f800000u ? 0x7f800000u : r;
    return __uint_as_float(sign | r);
}

__device__ __forceinline__ double f2d_exp(float x, int de) {
    const uint32_t f = __float_as_uint(x);
    const uint32_t sign = f & 0x80000000u;
    const uint32_t e = (f >> 23) & 0xffu;
    const uint32_t m = f & 0x7fffffu;
    uint32_t hi, lo;
    if (e == 0u) {
        hi = sign;
        lo = 0u;
    } else if (e == 0xffu) {
        hi = sign | 0x7ff00000u | (m >> 3);
        lo = m << 29;
    } else {
        hi = sign | ((uint32_t)((int)e - 127 + 1023 + de) << 20) | (m >> 3);
        lo = m << 29;
    }
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// True when x < 0 (a negative number, not -0), from the high word alone.
__device__ __forceinline__ bool is_negative(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) && (b << 1) != 0ull;
}

// x / 2, exact: decrement the exponent of normal numbers on the integer pipe;
// zeros, subnormals and the smallest normals take the FP64 multiply.
__device__ __forceinline__ double half_exact(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
    if (e > 1u && e < 0x7ffu) return __longlong_as_double((long long)(b - (1ull << 52)));
    return x * 0.5;
}

}  // namespace knc
