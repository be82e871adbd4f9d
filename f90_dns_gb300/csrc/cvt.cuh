// FP64 <-> FP32 conversions with integer operations.
//
// On this GPU the hardware conversions (F2F) issue on the FP64 pipe, which
// runs at 1/64 of the FP32 rate and is what the mixed-precision kernels are
// bound by; these run on the integer pipes instead, from the IEEE 754 binary64
// and binary32 encodings.  d2f rounds to nearest even (IEEE 754 default
// rounding) for results in the normal float range -- checked bit for bit
// against the hardware conversion by dns3d_check_conversions;
// results below it flush to signed zero (the spectra here never come within
// many decades of 1e-38), overflow gives infinity, NaN stays NaN.  f2d is
// exact (it is a widening).
#pragma once

namespace dns3d {

__device__ __forceinline__ float d2f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int fe = (int)((hi >> 20) & 0x7FFu) - 896;  // biased float exponent
    if (fe <= 0) return __uint_as_float(sign);
    if (fe >= 255) {
        const bool nan = ((hi >> 20) & 0x7FFu) == 0x7FFu && (((hi & 0xFFFFFu) | lo) != 0u);
        return __uint_as_float(sign | (nan ? 0x7FC00000u : 0x7F800000u));
    }
    unsigned f = sign | ((unsigned)fe << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1FFFFFFFu;  // the 29 dropped bits
    f += (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) ? 1u : 0u;  // carries into the exponent
    return __uint_as_float(f);
}

__device__ __forceinline__ double f2d(float v) {
    const unsigned f = __float_as_uint(v);
    const unsigned e = (f >> 23) & 0xFFu;
    if (e == 0u || e == 0xFFu) return (double)v;  // zero, subnormal, inf, NaN: rare, the hardware path
    const unsigned hi = (f & 0x80000000u) | ((e + 896u) << 20) | ((f & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(f << 29));
}

__device__ __forceinline__ float2 d2f(double2 a) { return make_float2(d2f(a.x), d2f(a.y)); }

// X 2^e2 for a 64-bit integer X, rounded to the nearest FP64 value (ties to
// even), from the integer's bits: the same value as the hardware int64 -> FP64
// conversion followed by an exact power-of-two scaling, which both issue on
// the FP64 pipe.  Results below the normal range take that hardware path.
__device__ __forceinline__ double i2d_scaled(long long X, int e2) {
    if (X == 0) return 0.0;
    const unsigned long long sg = X < 0 ? 0x8000000000000000ULL : 0ULL;
    const unsigned long long a = X < 0 ? 0ULL - (unsigned long long)X : (unsigned long long)X;
    const int p = 63 - __clzll((long long)a);  // a in [2^p, 2^(p+1))
    const int be = p + e2 + 1023;
    if (be <= 0) return ldexp(__ll2double_rn(X), e2);
    unsigned long long m;
    if (p > 52) {
        const int sh = p - 52;
        m = a >> sh;
        const unsigned long long rest = a & ((1ULL << sh) - 1ULL), half = 1ULL << (sh - 1);
        m += (rest > half || (rest == half && (m & 1ULL))) ? 1ULL : 0ULL;
    } else {
        m = a << (52 - p);
    }
    if (be >= 2047) return __longlong_as_double((long long)(sg | 0x7FF0000000000000ULL));
    // m in [2^52, 2^53]: the implicit bit (or a rounding carry) adds into the exponent field
    return __longlong_as_double((long long)(sg | (((unsigned long long)(be - 1) << 52) + m)));
}

}  // namespace dns3d
