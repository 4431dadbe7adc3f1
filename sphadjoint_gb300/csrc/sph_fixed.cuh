// Fixed-point grid values of the dJ/dtheta contributions: round(c 2^S) as a
// 128-bit two's-complement integer (lo, hi). Integer addition of these is
// associative, so the per-node sums are exact and independent of the order
// in which contributions arrive. Pure functions, compiled for the device by
// the kernels and for the host by the conversion test.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SPH_FIXED_HD __host__ __device__ __forceinline__
#else
#define SPH_FIXED_HD inline
#endif

namespace sphgb {

struct Fixed128 {
    unsigned long long lo, hi;
};

SPH_FIXED_HD uint32_t fixed_float_bits(float c)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(c);
#else
    uint32_t b;
    std::memcpy(&b, &c, sizeof b);
    return b;
#endif
}

SPH_FIXED_HD Fixed128 fixed_negate(Fixed128 v)
{
    v.lo = ~v.lo + 1ull;
    v.hi = ~v.hi + (v.lo == 0ull ? 1ull : 0ull);
    return v;
}

// round(c 2^S) (half to even) for finite c with |c| 2^S < 2^127; false when
// it is 0 or c is not finite
SPH_FIXED_HD bool fixed_of(double c, int S, Fixed128 &out)
{
    if (c == 0.0 || !std::isfinite(c)) return false;
    const double a = std::rint(std::ldexp(std::fabs(c), S));
    if (a == 0.0) return false;
    const double hid = std::floor(std::ldexp(a, -64));
    const double lod = a - std::ldexp(hid, 64);
    out.hi = (unsigned long long)hid;
    out.lo = (unsigned long long)lod;
    if (c < 0.0) out = fixed_negate(out);
    return true;
}

// The same integer for an FP32 contribution, with integer instructions only:
// c is M 2^E with a 24-bit integer M, so round(|c| 2^S) is M shifted by E + S,
// rounded half to even when the shift drops bits. That is what the double
// form's rint(ldexp(|c|, S)) gives for a float c (the double product is
// exact), without the double-precision pipe, which runs at a small fraction of
// the FP32 rate on this GPU.
SPH_FIXED_HD bool fixed_of(float c, int S, Fixed128 &out)
{
    const uint32_t bits = fixed_float_bits(c);
    const uint32_t ex = (bits >> 23) & 0xffu;
    if ((bits & 0x7fffffffu) == 0u || ex == 0xffu) return false; // zero, inf, NaN
    const uint32_t M = ex ? ((bits & 0x7fffffu) | 0x800000u) : (bits & 0x7fffffu);
    const int k = (ex ? (int)ex - 150 : -149) + S;
    if (k >= 104) return fixed_of((double)c, S, out); // beyond the 128-bit grid
    unsigned __int128 v;
    if (k >= 0) {
        v = (unsigned __int128)M << k;
    } else if (k <= -25) {
        return false; // below half a unit of the grid: rounds to 0
    } else {
        const int sh = -k;
        const uint32_t q = M >> sh, r = M & ((1u << sh) - 1u), half = 1u << (sh - 1);
        const uint32_t up = (r > half || (r == half && (q & 1u))) ? 1u : 0u;
        v = (unsigned __int128)(q + up);
    }
    if (v == 0) return false;
    if (bits >> 31) v = ~v + 1;
    out.lo = (unsigned long long)v;
    out.hi = (unsigned long long)(v >> 64);
    return true;
}

} // namespace sphgb
