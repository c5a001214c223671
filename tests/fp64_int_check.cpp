// Host check of gpuvoxels_gb300/csrc/fp64_int.cuh: every helper against the host's IEEE-754 arithmetic
// on random bit patterns, exponent-boundary cases, rounding ties and the special values.
// Usage: fp64_int_check [cases]; exit status 0 when no result differs.
#include "../gpuvoxels_gb300/csrc/fp64_int.cuh"

#include <cstdio>
#include <cstdlib>
#include <random>

using namespace gvx::fp64i;

static long bad = 0;
static bool same(double a, double b) { return bits(a) == bits(b) || (a != a && b != b); }
static bool samef(float a, float b) { return fbits(a) == fbits(b) || (a != a && b != b); }
static void report(const char* what, double a, double b) {
    if (bad++ < 8) std::printf("mismatch %s a=%a b=%a\n", what, a, b);
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 10000000;
    std::mt19937_64 rng(20240611);
    const uint64_t specials[] = {0ull, kSign, kInf, kInf | kSign, 0x7FF8000000000000ull, 1ull, kFrac, 0x0010000000000000ull,
                                 0x7FEFFFFFFFFFFFFFull, 0x3FF0000000000000ull, 0xBFF0000000000000ull};
    for (long i = 0; i < n; i++) {
        uint64_t x = rng(), y = rng();
        uint32_t fx = (uint32_t)rng();
        switch (i % 6) {
            case 1: y = x ^ (rng() & 0xFF); break;                                           // near-equal pairs
            case 2: x = specials[rng() % 11]; if (rng() & 1) y = specials[rng() % 11]; break;
            case 3: x = (x & ~(0x7FFull << 52)) | ((uint64_t)(860 + rng() % 330) << 52);      // around the float range
                    if (rng() % 3 == 0) x = (x & ~((1ull << 29) - 1)) | (1ull << 28); break;    // float rounding ties
            case 4: fx &= (rng() & 1) ? 0x807FFFFFu : 0xFFFFFFFFu; break;                      // float zeros/subnormals
            case 5: x = (x & ~(0x7FFull << 52)) | ((uint64_t)(rng() % 4 ? rng() % 4 : 2043 + rng() % 4) << 52); break;
        }
        const double a = from_bits(x), b = from_bits(y);
        const float f = from_fbits(fx);
        if (!same(f2d(f), (double)f)) report("f2d", (double)f, 0);
        if (!samef(d2f(a), (float)a)) report("d2f", a, 0);
        if (lt(a, b) != (a < b)) report("lt", a, b);
        if (gt(a, b) != (a > b)) report("gt", a, b);
        if (le(a, b) != (a <= b)) report("le", a, b);
        if (ge(a, b) != (a >= b)) report("ge", a, b);
        if (gt0(a) != (a > 0)) report("gt0", a, 0);
        if (ge0(a) != (a >= 0)) report("ge0", a, 0);
        if (eq0(a) != (a == 0)) report("eq0", a, 0);
        if (!same(mul2(a), a * 2.0)) report("mul2", a, 0);
        if (!same(half(a), a * 0.5)) report("half", a, 0);
        if (!same(plus_zero(a), a + 0.0)) report("plus_zero", a, 0);
        // known-zero forms: z a zero of either sign, y any non-NaN value, k finite
        const double z = (y & 1) ? -0.0 : 0.0;
        if (a == a) {
            if (!same(zero_plus(z, a), z + a)) report("zero_plus", z, a);
            if (!same(zero_minus(z, a), z - a)) report("zero_minus", z, a);
            if (!same(minus_zero(a, z), a - z)) report("minus_zero", a, z);
            if (a - a == 0 && !same(times_zero(a, z), a * z)) report("times_zero", a, z);
        }
    }
    std::printf("%ld cases, %ld mismatches\n", n, bad);
    return bad ? 1 : 0;
}
