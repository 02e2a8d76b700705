// fp_convert.cuh -- FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the conversion instruction (F2F.F32.F64) issues on the FP64 unit
// at the FP64 rate (~2 per clock per SM); kernels that convert every value
// they gather from an FP64 array become FP64-bound on it.  These do the
// same with a funnel shift, an exponent rebias and integer compares.
#pragma once

namespace mgpu {

// Round to nearest even.  Magnitudes below FP32's smallest normal (before
// rounding) become a signed zero, those above its range become infinity,
// NaN stays NaN.
__device__ __forceinline__ float f32_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned e = hi & 0x7ff00000u, sign = hi & 0x80000000u;
    // exponent (E - 1023 + 127 when E is in FP32's normal range) and the top 23 mantissa bits
    unsigned r = ((__funnelshift_l(lo, hi, 3) & 0x7fffffffu) - 0x40000000u) & 0x7fffffffu;
    // the 29 dropped bits: round bit 28, sticky bits 0..27; ties go to even
    const unsigned up = (lo >> 28) & ((lo & 0x0fffffffu) != 0u || (r & 1u) ? 1u : 0u);
    r = (r + up) | sign;
    if (e <= (896u << 20)) r = sign;
    if (e > (1150u << 20)) r = sign | 0x7f800000u | (e == 0x7ff00000u && (lo | (hi & 0xfffffu)) ? 0x400000u : 0u);
    return __uint_as_float(r);
}

// FP32 -> FP64, exact (every float is a double): sign, rebiased exponent and
// the mantissa shifted up; subnormal floats are normalised, infinity and NaN
// keep their class (and payload).
__device__ __forceinline__ double f64_of(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    unsigned long long r;
    if (e == 0xffu) {
        r = sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29);
    } else if (e != 0u) {
        r = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (m != 0u) {
        const unsigned top = 31u - (unsigned)__clz(m);  // m = 2^top (1 + f), value m 2^-149
        r = sign | ((unsigned long long)(top + 874u) << 52) |
            (((unsigned long long)m << (52u - top)) & 0x000fffffffffffffull);
    } else {
        r = sign;
    }
    return __longlong_as_double((long long)r);
}

}  // namespace mgpu
