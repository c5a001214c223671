// Host check of gvx::field_atof (the VXA reader's number-field parser) against atof:
// the same double, bit for bit, for random bit patterns printed at 17 digits, random
// values at 1..20 digits, and the forms that take the atof path (blanks, '+', hex,
// out of range, trailing text, inf/nan).  Usage: field_atof_check <cases>
#include "world.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

int main(int argc, char** argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> unit(0, 1);
    long bad = 0, n = 0;
    auto check = [&](const std::string& s) {
        const std::string t = s + ",9";   // the field followed by another one
        const double a = atof(s.c_str());
        const double b = gvx::field_atof(t.c_str(), t.c_str() + t.size());
        const double c = gvx::field_atof(s.c_str(), s.c_str() + s.size());
        n++;
        if (memcmp(&a, &b, 8) != 0 || memcmp(&a, &c, 8) != 0) {
            if (bad++ < 10) printf("mismatch '%s': atof %.17g, field %.17g / %.17g\n", s.c_str(), a, b, c);
        }
    };
    char buf[64];
    for (long i = 0; i < cases; i++) {
        const uint64_t u = g();
        double d;
        memcpy(&d, &u, 8);
        if (d == d) { snprintf(buf, sizeof buf, "%.17g", d); check(buf); }
        snprintf(buf, sizeof buf, "%.*g", 1 + (int)(g() % 20), unit(g));
        check(buf);
    }
    for (const char* s : {"", " 1.5", "+2", "1e400", "-1e400", "1e-400", "4.9e-324", "2.4e-324", "0x1p3", "nan", "inf", "-inf",
                          "-0", "1.5abc", ".5", "5.", "1e", "-.5e-3", "1e+5", "00012", "1.7976931348623157e308",
                          "1.7976931348623159e308", "2.2250738585072011e-308", "  ", "\n3.25"})
        check(s);
    printf("checked %ld, mismatches %ld\n", n, bad);
    return bad != 0;
}
