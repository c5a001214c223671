// Exact FP64 helpers that run on the integer pipes.
//
// GB300 executes FP64 arithmetic, FP64 compares (DSETP) and float<->double
// conversions (F2F) on one narrow FP64 pipe: about 2 lanes per clock per SM,
// against 128 for 32-bit integer and FP32 work.  The step kernels are bound by
// that pipe, so every FP64-pipe instruction whose result can be formed exactly
// from the bit pattern moves here.  Each function returns bit-for-bit what the
// FP64 instruction it replaces returns, for every input (zeros, subnormals,
// infinities and NaNs included: the rare cases fall back to that
// instruction).  The functions compile for the host as well, where
// tests/fp64_int_check.cpp compares them with the host's IEEE arithmetic.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GVX_FP64I __host__ __device__ __forceinline__
#else
#define GVX_FP64I static inline
#endif

namespace gvx {
namespace fp64i {

GVX_FP64I uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u; std::memcpy(&u, &x, 8); return u;
#endif
}
GVX_FP64I double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x; std::memcpy(&x, &u, 8); return x;
#endif
}
GVX_FP64I uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u; std::memcpy(&u, &x, 4); return u;
#endif
}
GVX_FP64I float from_fbits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x; std::memcpy(&x, &u, 4); return x;
#endif
}

constexpr uint64_t kSign = 0x8000000000000000ull, kAbs = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFull, kInf = 0x7FF0000000000000ull;

// x * 2 (exponent + 1 for normal x that stays finite; subnormals shift left)
GVX_FP64I double mul2(double x) {
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e - 1u < 0x7FDu) return from_bits(b + (1ull << 52));
    if (e == 0u) return from_bits((b & kSign) | ((b & kAbs) << 1));
    return x * 2.0;
}
// x * 0.5 (exponent - 1 while the result stays normal; +-0 unchanged)
GVX_FP64I double half(double x) {
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e - 2u < 0x7FDu) return from_bits(b - (1ull << 52));
    if ((b & kAbs) == 0) return x;
    return x * 0.5;
}

// (double)f: exact; normal floats and zeros on the integer pipes
GVX_FP64I double f2d(float f) {
    const uint32_t u = fbits(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u >= 254u) {
        if ((u & 0x7FFFFFFFu) == 0) return from_bits((uint64_t)u << 32);
        return (double)f;
    }
    const uint32_t hi = (u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + (896u << 20));
    return from_bits(((uint64_t)hi << 32) | (((uint64_t)u << 29) & 0xFFFFFFFFull));
}
// (float)x, round to nearest even; results that are normal floats, and zeros, on the integer pipes
GVX_FP64I float d2f(double x) {
    const uint64_t u = bits(x);
    const uint32_t e = (uint32_t)(u >> 52) & 0x7FFu;
    if (e - 897u >= 254u) {
        if ((u & kAbs) == 0) return from_fbits((uint32_t)(u >> 32));
        return (float)x;
    }
    uint32_t m = (uint32_t)((u & kFrac) >> 29);
    const uint32_t rest = (uint32_t)u & 0x1FFFFFFFu;
    m += (uint32_t)((rest > 0x10000000u) | ((rest == 0x10000000u) & (m & 1u)));
    return from_fbits(((uint32_t)(u >> 32) & 0x80000000u) + ((e - 896u) << 23) + m);
}

// Ordered comparisons with IEEE semantics: false when either operand is NaN, -0 == +0.
GVX_FP64I int64_t order_key(uint64_t u) { return (int64_t)u >= 0 ? (int64_t)u : (int64_t)(kSign - u); }
GVX_FP64I bool is_nan_bits(uint64_t u) { return (u & kAbs) > kInf; }
GVX_FP64I bool lt(double a, double b) {
    const uint64_t ua = bits(a), ub = bits(b);
    return !(is_nan_bits(ua) | is_nan_bits(ub)) & (order_key(ua) < order_key(ub));
}
GVX_FP64I bool gt(double a, double b) { return lt(b, a); }
GVX_FP64I bool le(double a, double b) {
    const uint64_t ua = bits(a), ub = bits(b);
    return !(is_nan_bits(ua) | is_nan_bits(ub)) & (order_key(ua) <= order_key(ub));
}
GVX_FP64I bool ge(double a, double b) { return le(b, a); }
// x > 0 and x >= 0 (false for NaN and for -0 in the strict form)
GVX_FP64I bool gt0(double x) { const int64_t b = (int64_t)bits(x); return b > 0 && (uint64_t)b <= kInf; }
GVX_FP64I bool ge0(double x) { const uint64_t b = bits(x); return (b == kSign) | ((int64_t)b >= 0 && b <= kInf); }
// x == 0 (either sign)
GVX_FP64I bool eq0(double x) { return (bits(x) & kAbs) == 0; }

// x + 0.0 with x possibly -0: IEEE gives +0 for -0 and x otherwise (NaN stays NaN)
GVX_FP64I double plus_zero(double x) { const uint64_t b = bits(x); return from_bits(b == kSign ? 0ull : b); }

}  // namespace fp64i
}  // namespace gvx
