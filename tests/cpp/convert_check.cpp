// Checks the integer float <-> double conversions of the FP64 replacement
// (fast_gb300/csrc/fp_convert.h) against the native conversions on random
// bit patterns and on edge cases.  Expected differences only: float
// subnormals widen to a signed zero, doubles that narrow to a float
// subnormal become a signed zero, and a NaN narrows to an infinity.
// Prints "widen <n> <bad>" and "narrow <n> <bad>"; exits 1 on any other
// difference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "fp_convert.h"

static uint32_t fb(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static uint64_t db(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static float bf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static double bd(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }

static bool widen_ok(float f)
{
    const double a = ft::widen_f(f);
    if (std::isnan(f)) return std::isnan(a) && std::signbit(a) == std::signbit(f);
    if (std::fpclassify(f) == FP_SUBNORMAL) return a == 0.0 && std::signbit(a) == std::signbit(f);
    return db(a) == db((double)f);
}

static bool narrow_ok(double d)
{
    const float a = ft::narrow_d(d), b = (float)d;
    if (std::isnan(d)) return std::isinf(a) && std::signbit(a) == std::signbit(d);
    if (std::fabs(d) < 0x1p-126 && std::fpclassify(b) != FP_NORMAL)  // narrows to a subnormal or zero
        return a == 0.0f && std::signbit(a) == std::signbit(d);
    return fb(a) == fb(b);
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 20000000L;
    std::mt19937_64 g(7);
    long wbad = 0, nbad = 0;
    for (long i = 0; i < n; ++i) {
        const float f = bf((uint32_t)g());
        if (!widen_ok(f)) {
            if (wbad < 5) printf("widen mismatch %08x\n", fb(f));
            ++wbad;
        }
    }
    for (long i = 0; i < n; ++i) {
        uint64_t u = g();
        if (i & 1)  // exponents around the float range
            u = (u & 0x800fffffffffffffull) | ((uint64_t)(880 + g() % 290) << 52);
        if (i % 5 == 0)  // rounding ties and their neighbours
            u = (u & ~0x1fffffffull) | (g() % 3 == 0 ? 0x10000000ull : (g() & 0x1fffffffull));
        if (!narrow_ok(bd(u))) {
            if (nbad < 5) printf("narrow mismatch %016llx\n", (unsigned long long)u);
            ++nbad;
        }
    }
    const double edge_d[] = {0.0, -0.0, 1.0, -1.0, 0.1, 1e-8, -2.5e-7, 3.4028234663852886e38,
                             3.4028235677973366e38, -3.402823567797337e38, 0x1p-126, 0x1.fffffcp-127,
                             0x1p-149, 5e-324, 1e300, -1e300, INFINITY, -INFINITY, NAN};
    for (double d : edge_d)
        if (!narrow_ok(d)) {
            printf("narrow edge mismatch %a\n", d);
            ++nbad;
        }
    const float edge_f[] = {0.f, -0.f, 1.f, -1.f, 0x1p-149f, 0x1p-126f, 3.4028235e38f, INFINITY, -INFINITY, NAN, 1e-8f};
    for (float f : edge_f)
        if (!widen_ok(f)) {
            printf("widen edge mismatch %a\n", f);
            ++wbad;
        }
    printf("widen %ld %ld\nnarrow %ld %ld\n", n, wbad, n, nbad);
    return (wbad || nbad) ? 1 : 0;
}
