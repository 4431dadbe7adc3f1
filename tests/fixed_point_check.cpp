// The FP32 fixed-point conversion of the dJ/dtheta contributions
// (sph_fixed.cuh, integer instructions only) against the double-precision
// form it replaces, on random float patterns and scales, on the halfway
// cases of its rounding, and on subnormals. Prints the counts; exits 1 on
// any difference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "sph_fixed.cuh"

using sphgb::Fixed128;
using sphgb::fixed_of;

static long g_bad = 0, g_checked = 0;

static void check(float c, int S)
{
    Fixed128 a{0, 0}, b{0, 0};
    const bool ka = fixed_of(c, S, a);
    const bool kb = fixed_of((double)c, S, b);
    if (!ka) a = Fixed128{0, 0};
    if (!kb) b = Fixed128{0, 0};
    ++g_checked;
    if (a.lo != b.lo || a.hi != b.hi) {
        if (g_bad < 5) std::printf("mismatch c=%a S=%d\n", (double)c, S);
        ++g_bad;
    }
}

int main()
{
    std::mt19937_64 g(20260101);
    // random bit patterns and scales, within the grid's bound |c| 2^S < 2^124
    for (long t = 0; t < 4000000; ++t) {
        const uint32_t bits = (uint32_t)g();
        float c;
        std::memcpy(&c, &bits, sizeof c);
        const int S = (int)(g() % 300) - 100;
        if (std::isfinite(c) && c != 0.0f && std::ilogb(c) + S >= 123) continue;
        check(c, S);
    }
    // halfway and near-halfway cases of the rounding shift, both signs
    for (int S = -30; S < 30; S += 3)
        for (uint32_t M = 0x800000u; M < 0x800000u + 3000u; ++M)
            for (int e = -30; e < 5; ++e) {
                const float c = std::ldexp((float)M, e - 23);
                check(c, S);
                check(-c, S);
            }
    // subnormals
    for (uint32_t m = 1; m < 200000; m += 7)
        for (int S = 100; S < 160; S += 5) {
            float c;
            std::memcpy(&c, &m, sizeof c);
            check(c, S);
            check(-c, S);
        }
    std::printf("checked %ld, mismatches %ld\n", g_checked, g_bad);
    return g_bad ? 1 : 0;
}
