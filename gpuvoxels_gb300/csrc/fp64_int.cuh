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

// On the device the bit pattern moves through an opaque register move, so that the
// compiler cannot fold the integer tests below back into FP64 compares.
GVX_FP64I uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
    uint64_t u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
#else
    uint64_t u; std::memcpy(&u, &x, 8); return u;
#endif
}
GVX_FP64I double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
    return x;
#else
    double x; std::memcpy(&x, &u, 8); return x;
#endif
}
// The FP64 instructions of the rare cases, in a form the compiler does not move out
// of their branch (a speculated copy would run on the FP64 pipe for every call).
GVX_FP64I double rare_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
#else
    return a * b;
#endif
}
GVX_FP64I double rare_f2d(float f) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(f));
    return r;
#else
    return (double)f;
#endif
}
GVX_FP64I float rare_d2f(double x) {
#ifdef __CUDA_ARCH__
    float r;
    asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(x));
    return r;
#else
    return (float)x;
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
    return rare_mul(x, 2.0);
}
// x * 0.5 (exponent - 1 while the result stays normal; +-0 unchanged)
GVX_FP64I double half(double x) {
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e - 2u < 0x7FDu) return from_bits(b - (1ull << 52));
    if ((b & kAbs) == 0) return x;
    return rare_mul(x, 0.5);
}

// (double)f: exact; normal floats and zeros on the integer pipes
GVX_FP64I double f2d(float f) {
    const uint32_t u = fbits(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u >= 254u) {
        if ((u & 0x7FFFFFFFu) == 0) return from_bits((uint64_t)u << 32);
        return rare_f2d(f);
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
        return rare_d2f(x);
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

// Sums, differences and products with an operand z that the algorithm makes an
// exact zero (either sign), for any non-NaN y and finite k: IEEE gives the other
// operand, except that a sum of two zeros is -0 only when both are -0 (a difference
// a - b is a + (-b)), and a finite k times a zero is a zero with the XOR of the signs.
GVX_FP64I double zero_plus(double z, double y) {    // z + y, equally y + z
    const uint64_t uz = bits(z), uy = bits(y);
    return from_bits((uy & kAbs) == 0 ? (uz & uy) : uy);
}
GVX_FP64I double zero_minus(double z, double y) {   // z - y
    const uint64_t uz = bits(z), uy = bits(y);
    return from_bits((uy & kAbs) == 0 ? (uz & ~uy & kSign) : (uy ^ kSign));
}
GVX_FP64I double minus_zero(double y, double z) {   // y - z
    const uint64_t uz = bits(z), uy = bits(y);
    return from_bits((uy & kAbs) == 0 ? (uy & ~uz & kSign) : uy);
}
GVX_FP64I double times_zero(double k, double z) {   // k * z
    return from_bits((bits(k) ^ bits(z)) & kSign);
}

}  // namespace fp64i
}  // namespace gvx
